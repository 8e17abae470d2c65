// Diagnostics of synchrad_gb300 (no counterpart in the reference):
//  * CUDA-event timing of the dominant kernel of each sr_spectrum call, on the
//    stream it is launched on, for the roofline figures of the benchmark;
//  * an FP32 fused-multiply-add throughput probe (scalar FFMA and packed
//    FFMA2), the FP32 roofline denominator measured on the device at hand.
#include <mutex>
#include <vector>

#include "sr_common.cuh"
#include "sr_internal.h"

namespace sr {
namespace {
std::mutex g_mu;
bool g_timing = false;
std::vector<std::pair<cudaEvent_t, cudaEvent_t>> g_events;
}  // namespace

bool timing_enabled() {
  std::lock_guard<std::mutex> lk(g_mu);
  return g_timing;
}

void timing_record(cudaStream_t s, bool start, void **token) {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_timing) return;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone)
    return;  // kernels inside a captured graph are not timed one by one
  cudaEvent_t e;
  if (cudaEventCreate(&e) != cudaSuccess) return;
  cudaEventRecord(e, s);
  if (start) {
    g_events.push_back({e, nullptr});
    *token = (void *)(g_events.size());
  } else if (*token) {
    g_events[(size_t)(*token) - 1].second = e;
  } else {
    cudaEventDestroy(e);
  }
}

namespace {

__global__ void fp32_probe_scalar(float *out, int iters) {
  float a = 1.0f + threadIdx.x * 1e-7f, b = 1e-7f;
  float c0 = threadIdx.x, c1 = c0 + 1, c2 = c0 + 2, c3 = c0 + 3, c4 = c0 + 4, c5 = c0 + 5,
        c6 = c0 + 6, c7 = c0 + 7;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      c0 = __fmaf_rn(c0, a, b); c1 = __fmaf_rn(c1, a, b); c2 = __fmaf_rn(c2, a, b);
      c3 = __fmaf_rn(c3, a, b); c4 = __fmaf_rn(c4, a, b); c5 = __fmaf_rn(c5, a, b);
      c6 = __fmaf_rn(c6, a, b); c7 = __fmaf_rn(c7, a, b);
    }
  }
  if (c0 + c1 + c2 + c3 + c4 + c5 + c6 + c7 == 1234.5f) out[0] = c0;
}

__global__ void fp32_probe_packed(float *out, int iters) {
  const float2 a = make_float2(1.0f + threadIdx.x * 1e-7f, 1.0f - threadIdx.x * 1e-7f);
  const float2 b = make_float2(1e-7f, 2e-7f);
  float2 c[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) c[k] = make_float2(threadIdx.x + k, k);
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int r = 0; r < 2; ++r)
#pragma unroll
      for (int k = 0; k < 8; ++k) c[k] = __ffma2_rn(c[k], a, b);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += c[k].x + c[k].y;
  if (s == 1234.5f) out[0] = s;
}

}  // namespace
}  // namespace sr

using namespace sr;

extern "C" int sr_timing_enable(int enable) {
  std::lock_guard<std::mutex> lk(g_mu);
  g_timing = enable != 0;
  return SR_OK;
}

extern "C" int sr_timing_read(double *total_ms, int *n_launches) {
  clear_error();
  std::lock_guard<std::mutex> lk(g_mu);
  double tot = 0.0;
  int n = 0;
  int rc = SR_OK;
  for (auto &pr : g_events) {
    if (pr.second) {
      cudaError_t e = cudaEventSynchronize(pr.second);
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, pr.first, pr.second);
      if (e != cudaSuccess && rc == SR_OK) rc = cuda_fail(e, "timing event");
      tot += ms;
      ++n;
      cudaEventDestroy(pr.second);
    }
    cudaEventDestroy(pr.first);
  }
  g_events.clear();
  if (total_ms) *total_ms = tot;
  if (n_launches) *n_launches = n;
  return rc;
}

extern "C" int sr_probe_fp32_peak(double *tflops_scalar, double *tflops_packed, void *stream) {
  clear_error();
  cudaStream_t s = (cudaStream_t)stream;
  int dev = 0, n_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  float *dummy = nullptr;
  cudaError_t e = cudaMallocAsync((void **)&dummy, 16, s);
  if (e != cudaSuccess) return cuda_fail(e, "probe buffer");
  const int blocks = n_sm * 4, threads = 256, iters = 1 << 16;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  double res[2] = {0, 0};
  for (int packed = 0; packed < 2; ++packed) {
    for (int rep = 0; rep < 2; ++rep) {  // first repetition warms up the clocks
      cudaEventRecord(a, s);
      if (packed)
        fp32_probe_packed<<<blocks, threads, 0, s>>>(dummy, iters);
      else
        fp32_probe_scalar<<<blocks, threads, 0, s>>>(dummy, iters);
      cudaEventRecord(b, s);
      e = cudaEventSynchronize(b);
      if (e != cudaSuccess) break;
      float ms = 0.f;
      cudaEventElapsedTime(&ms, a, b);
      // lane-FMAs per launch: blocks*threads*iters*32; 2 flops each
      const double flops = 2.0 * blocks * threads * (double)iters * 32.0;
      res[packed] = flops / (ms * 1e-3) / 1e12;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFreeAsync(dummy, s);
  if (e != cudaSuccess) return cuda_fail(e, "fp32 probe");
  if (tflops_scalar) *tflops_scalar = res[0];
  if (tflops_packed) *tflops_packed = res[1];
  return SR_OK;
}

namespace sr {
namespace {

// A wait that nothing ends: an mbarrier expecting one arrival that never
// comes, waited on with the bounded wait every kernel of the library uses.
// The wait gives up after limit_ns and the kernel records the timeout in the
// status word exactly as the spectrum kernels do; no copy is ever issued.
__global__ void wait_timeout_selftest_kernel(int *status, uint64_t limit_ns) {
  __shared__ uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool ok = mbar_wait_bounded(&bar, 0u, limit_ns);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(status, STATUS_WAIT_TIMEOUT);
}

}  // namespace
}  // namespace sr

extern "C" int sr_selftest_wait_timeout(int64_t limit_ns, void *workspace, void *stream) {
  clear_error();
  if (limit_ns <= 0 || limit_ns > 1000000000ll)
    return fail(SR_ERR_INVALID, "limit %lld ns (1 .. 1e9)", (long long)limit_ns);
  if (!workspace) {  // the static scratch of sr_spectrum_noalloc
    int *word = nullptr;
    const int rc = noalloc_status_word(&word);
    if (rc) return rc;
    workspace = word;
  }
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(workspace, 0, sizeof(int), s);
  if (e != cudaSuccess) return cuda_fail(e, "status reset");
  wait_timeout_selftest_kernel<<<1, 32, 0, s>>>((int *)workspace, (uint64_t)limit_ns);
  return cuda_fail(cudaGetLastError(), "self-test launch");
}
