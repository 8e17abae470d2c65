// Device helpers shared by the mixed-precision far- and near-field kernels.
#pragma once

#include "sr_common.cuh"
#include "sr_internal.h"

namespace sr {
namespace {

constexpr int kStage = 128;         // steps per TMA stage
constexpr size_t kMaxSmemPerCta = 232448;  // opt-in shared memory per CTA (227 KB)
constexpr int kFoldStages = 32;     // near field: FP32 sums fold into compensated pairs every 4096 steps
// float4 per step record: 64 bytes of data and 16 of padding, so that 32
// lanes reading one record each from shared memory hit every bank once per
// quarter warp (at a 64-byte stride four lanes in eight share the same banks)
constexpr int kRecF4 = 5;
constexpr uint32_t kRecBytes = kRecF4 * 16;
constexpr float kPiLo = 3.14159265358979f * (1.0f - 4e-6f);
constexpr float kPiHi = 3.14159265358979f * (1.0f + 4e-6f);

__device__ __forceinline__ uint32_t lower_bound_i64(const int64_t *a, uint32_t n,
                                                    int64_t v) {
  uint32_t lo = 0, hi = n;  // first index in [0, n) with a[i] >= v, or n
  while (lo < hi) {
    const uint32_t mid = (lo + hi) >> 1;
    if (a[mid] < v) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// Track range [t0, t1) of subset `sub`: tracks whose first step lies in
// [sub*total/n_sub, (sub+1)*total/n_sub), so subsets carry equal step counts.
__device__ __forceinline__ void subset_tracks(const FarMixedParams &p, uint32_t sub,
                                              uint32_t &t0, uint32_t &t1) {
  const int64_t tot = p.total_steps;
  t0 = (sub == 0) ? 0u
                  : lower_bound_i64(p.offsets, p.n_tracks, (tot * (int64_t)sub) / p.n_sub);
  t1 = (sub + 1 == p.n_sub)
           ? p.n_tracks
           : lower_bound_i64(p.offsets, p.n_tracks, (tot * (int64_t)(sub + 1)) / p.n_sub);
}

__device__ __forceinline__ uint32_t track_body(const FarMixedParams &p, uint32_t t) {
  const int64_t n = p.offsets[t + 1] - p.offsets[t];
  const uint32_t it_end = p.it_end[t];
  if (n < 1 || it_end < 1) return 0;
  return (uint32_t)min((int64_t)it_end - 1, n - 1);
}

// exp(i 2 pi w tau) for a double-float frequency in revolutions: the phase is
// formed in double-float, its whole revolutions are dropped (p - rint(p) is
// exact), and the fraction goes to the SFU sin/cos.
__device__ __forceinline__ void phasor_rev(float wh, float wl, float th, float tl, float &s,
                                           float &c) {
  const float p = wh * th;
  float e = __fmaf_rn(wh, th, -p);
  e = __fmaf_rn(wh, tl, e);
  e = __fmaf_rn(wl, th, e);
  const float n = rintf(p);
  const float f = (p - n) + e;
  __sincosf(f * 6.28318530717958648f, &s, &c);
}

// The reference's mask test evaluated exactly as the FP64 kernel does it
// (synchrad/kernel_farfield.cl:65-72), for one point and step.
__device__ __noinline__ bool exact_mask(const FarMixedParams &p, int64_t base, uint32_t s,
                                        uint32_t it_start, double omega, double n0,
                                        double n1, double n2) {
  auto ld = [&](const void *a, int64_t i) -> double {
    return p.track_f32 ? (double)((const float *)a)[i] : ((const double *)a)[i];
  };
  auto phase_at = [&](uint32_t it) -> double {
    const double time = __dmul_rn((double)(uint32_t)(it_start + it), p.dt);
    const int64_t g = base + it;
    const double d = __dadd_rn(__dadd_rn(__dmul_rn(ld(p.x, g), n0), __dmul_rn(ld(p.y, g), n1)),
                               __dmul_rn(ld(p.z, g), n2));
    return __dmul_rn(omega, __dsub_rn(time, d));
  };
  const double ph = phase_at(s);
  const double prev = (s == 0) ? 0.0 : phase_at(s - 1);
  return fabs(__dsub_rn(ph, prev)) < M_PI;
}

// The reference's mask test evaluated exactly as the FP64 kernel does it
// (synchrad/kernel_nearfield.cl:64-74), for one point and step.
__device__ __noinline__ bool exact_mask_near(const FarMixedParams &p, int64_t base, uint32_t s,
                                             uint32_t it_start, double omega, double P0,
                                             double P1) {
  auto ld = [&](const void *a, int64_t i) -> double {
    return p.track_f32 ? (double)((const float *)a)[i] : ((const double *)a)[i];
  };
  auto phase_at = [&](uint32_t it) -> double {
    const double time = __dmul_rn((double)(uint32_t)(it_start + it), p.dt);
    const int64_t g = base + it;
    const double d0 = __dsub_rn(P0, ld(p.x, g));
    const double d1 = __dsub_rn(P1, ld(p.y, g));
    const double d2 = __dsub_rn(p.L_screen, ld(p.z, g));
    const double rr = __dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2));
    return __dmul_rn(omega, __dadd_rn(time, __dsqrt_rn(rr)));
  };
  const double ph = phase_at(s);
  const double prev = (s == 0) ? 0.0 : phase_at(s - 1);
  return fabs(__dsub_rn(ph, prev)) < M_PI;
}

// Bits j in [0, nv) of a uniform omega chunk (omega_j = w0 + j dw) with
// |omega_j| < wb: an index interval, found from its two float bounds.  The
// caller passes 1/dw and forms wb from 1/adt: products instead of divisions
// move the bounds by a few ulp of (wb - w0)/dw, far inside the 4e-6 guard
// band between kPiLo and kPiHi.
__device__ __forceinline__ uint32_t omega_range_bits_r(float w0, float dw, float inv_dw, float wb,
                                                       int nv) {
  const uint32_t all = (nv >= 32) ? 0xffffffffu : ((1u << nv) - 1u);
  if (!(wb > 0.f)) return 0u;
  float lo, hi;
  if (dw > 0.f) {
    lo = (-wb - w0) * inv_dw;
    hi = (wb - w0) * inv_dw;
  } else if (dw < 0.f) {
    lo = (wb - w0) * inv_dw;
    hi = (-wb - w0) * inv_dw;
  } else {
    return fabsf(w0) < wb ? all : 0u;
  }
  lo = fminf(fmaxf(lo, -2.f), 40.f);
  hi = fminf(fmaxf(hi, -2.f), 40.f);
  const int jf = max(0, (int)floorf(lo) + 1);      // first j > lo
  const int jl = min(nv - 1, (int)ceilf(hi) - 1);  // last j < hi
  if (jf > jl) return 0u;
  const uint32_t upto = (jl >= 31) ? 0xffffffffu : ((2u << jl) - 1u);
  const uint32_t below = (1u << jf) - 1u;
  return upto & ~below & all;
}

// Indices j in [0, n) of a uniform omega axis (omega_j = w0 + j dw) with
// |omega_j| < wb: an interval [jf, jl] (empty when jf > jl), from its two float
// bounds.  Float rounding of w0, dw and the products moves the bounds by about
// 1e-7 of |omega| at the bound, inside the 4e-6 guard band between kPiLo and
// kPiHi whose points are tested exactly.
__device__ __forceinline__ void omega_interval(float w0, float dw, float inv_dw, float wb, int n,
                                               int &jf, int &jl) {
  jf = 1;
  jl = 0;
  if (!(wb > 0.f)) return;
  float lo, hi;
  if (dw > 0.f) {
    lo = (-wb - w0) * inv_dw;
    hi = (wb - w0) * inv_dw;
  } else if (dw < 0.f) {
    lo = (wb - w0) * inv_dw;
    hi = (-wb - w0) * inv_dw;
  } else {
    if (fabsf(w0) < wb) { jf = 0; jl = n - 1; }
    return;
  }
  const float top = (float)n + 1.f;
  lo = fminf(fmaxf(lo, -2.f), top);
  hi = fminf(fmaxf(hi, -2.f), top);
  jf = max(0, (int)floorf(lo) + 1);      // first j > lo
  jl = min(n - 1, (int)ceilf(hi) - 1);   // last j < hi
}

// Bits (j - j0) of the indices j in [a, b] clamped to [j0, j0 + nv), nv <= 32.
__device__ __forceinline__ uint32_t range_bits(int a, int b, int j0, int nv) {
  const int lo = max(a, j0) - j0, hi = min(b, j0 + nv - 1) - j0;
  if (lo > hi) return 0u;
  const uint32_t upto = (hi >= 31) ? 0xffffffffu : ((2u << hi) - 1u);
  return upto & ~((1u << lo) - 1u);
}

// (zr + i zi) * (rc + i rs) for two points at once, factors given as pairs.
__device__ __forceinline__ void rot2p(float2 zr, float2 zi, float2 rc, float2 rs, float2 nrs,
                                      float2 &or_, float2 &oi) {
  const float2 u = __fmul2_rn(zi, nrs);
  const float2 v = __fmul2_rn(zr, rs);
  or_ = __ffma2_rn(zr, rc, u);
  oi = __ffma2_rn(zi, rc, v);
}

__device__ __forceinline__ void cmul(float ar, float ai, float br, float bi, float &cr,
                                     float &ci) {
  cr = ar * br - ai * bi;
  ci = ar * bi + ai * br;
}

// out[c][k*P + g] += sum over subsets (fixed order) of partial[sub][c][k][g]
__global__ void mixed_reduce_kernel(FarMixedParams p) {
  const uint64_t P = (uint64_t)p.n_omega * p.n_theta * p.n_phi;
  const uint64_t per = (uint64_t)p.n_snaps * P;
  const uint64_t total = per * p.n_out;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t c = (uint32_t)(i / per);
    const uint64_t r = i - (uint64_t)c * per;
    double acc = 0.0;
    for (uint32_t s = 0; s < p.n_sub; ++s) acc += p.partial[((uint64_t)s * p.n_out + c) * per + r];
    p.out[c][r] += acc;
  }
}

}  // namespace
}  // namespace sr
