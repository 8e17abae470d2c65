// Allocation-free entry point of the mixed-precision far field.
//
// sr_spectrum needs a caller-provided device workspace.  Some callers cannot
// obtain one: code that runs inside a host application which owns every device
// allocation (a plugin handed only input and output buffers), or code running
// where allocation is not permitted at that moment.  For them,
// sr_spectrum_noalloc evaluates the same kernels with their scratch memory in a
// fixed array compiled into this library (kScratchBytes, 64 MiB), so it calls
// no cudaMalloc, cudaFree or allocating library routine.  Every GPU that loads
// the library keeps that array until the process exits.
//
// Host code cannot use the array's name as a device address: it names a
// host-side stand-in.  The device address is looked up once per device, on the
// first call made with that device current, by cudaGetSymbolAddress; that first
// call should therefore come before any stream capture.  The cached address
// belongs to the device's context at that time: it does not survive
// cudaDeviceReset (or a primary context released and created again), after
// which these entry points must not be called in the same process.  All calls
// share the one array: calls that overlap on the GPU (two streams, or two host
// threads) race, and each call clears what must start at zero.
//
// The first 256 bytes of the array hold the kernels' status word, as at the
// start of sr_spectrum's workspace.  sr_noalloc_status reads it back: a bounded
// wait that ran out of time in the last call is reported there, not by the
// call's return code (the call returns once its kernels are queued).
#include <mutex>

#include "sr_common.cuh"
#include "sr_internal.h"

namespace sr {
namespace {

constexpr size_t kScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 128;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_scratch_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of the array on the current device (looked up once per device).
int scratch_address(void **addr) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(SR_ERR_INVALID, "device ordinal %d", dev);
  std::lock_guard<std::mutex> lk(g_scratch_mu);
  if (g_scratch_addr[dev] == nullptr) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the static scratch");
    g_scratch_addr[dev] = p;
  }
  *addr = g_scratch_addr[dev];
  return SR_OK;
}

}  // namespace

// The status word at the start of the static array, on the current device
// (sr_selftest_wait_timeout's target when it is given no workspace).
int noalloc_status_word(int **word) {
  void *p = nullptr;
  const int rc = scratch_address(&p);
  if (rc) return rc;
  *word = (int *)p;
  return SR_OK;
}

}  // namespace sr

using namespace sr;

extern "C" int sr_noalloc_status(void *stream) {
  clear_error();
  int *word = nullptr;
  int rc = noalloc_status_word(&word);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
  int status = 0;
  e = cudaMemcpy(&status, word, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "status read");
  if (status == STATUS_WAIT_TIMEOUT)
    return fail(SR_ERR_TIMEOUT, "a kernel wait on a staged copy ran out of time in the last "
                                "sr_spectrum_noalloc call; its outputs are incomplete");
  return SR_OK;
}

extern "C" int sr_spectrum_noalloc(const sr_tracks *t, const sr_grid *g, int comp,
                                   void *const *out, void *stream) {
  clear_error();
  int rc = validate_spectrum_args(t, g, comp, SR_PREC_MIXED, out);
  if (rc) return rc;
  if (g->mode != SR_MODE_FAR)
    return fail(SR_ERR_UNSUPPORTED, "sr_spectrum_noalloc evaluates the far field only");
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  if (P == 0 || t->n_tracks == 0 || t->n_snaps == 0) return SR_OK;

  // The workspace layout of sr_spectrum with one track subset, and as many
  // persistent CTAs as the remaining room holds for their compensated sums.
  FarMixedConfig cfg =
      far_mixed_choose(g->n_omega, g->n_theta * g->n_phi, t->n_tracks, device_sm_count());
  cfg.n_sub = 1;
  const uint32_t n_wtiles = (g->n_omega + (uint32_t)(cfg.L * cfg.K) - 1) / (uint32_t)(cfg.L * cfg.K);
  const uint64_t dgroups = ((uint64_t)g->n_theta * g->n_phi + cfg.dpw - 1) / cfg.dpw;
  const uint64_t groups = (dgroups * n_wtiles + cfg.W - 1) / cfg.W;
  const int n_out = n_outputs(comp);
  FarMixedConfig one = cfg;
  one.grid = 0;
  const size_t fixed = far_mixed_workspace(t->total_steps, P, n_out, t->n_snaps, one);
  const size_t per_cta = (size_t)cfg.W * cfg.K * 8 * 32 * sizeof(float);
  if (fixed + per_cta > kScratchBytes)
    return fail(SR_ERR_INVALID,
                "sr_spectrum_noalloc: these sizes need %zu bytes of scratch, the static array "
                "holds %zu (80 B per track step plus 8 B per point, output and snapshot)",
                fixed + per_cta, kScratchBytes);
  uint64_t grid = (kScratchBytes - fixed) / per_cta;
  if (grid > (uint64_t)cfg.grid) grid = (uint64_t)cfg.grid;
  if (grid > groups) grid = groups;
  cfg.grid = (int)(grid > 0 ? grid : 1);

  void *scratch = nullptr;
  rc = scratch_address(&scratch);
  if (rc) return rc;
  return launch_far_mixed(make_far_mixed_params(t, g, comp, out), cfg, scratch, kScratchBytes,
                          (cudaStream_t)stream);
}
