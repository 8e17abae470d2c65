// Shared device/host helpers of the synchrad_gb300 CUDA library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/synchrad_gb300.h"

namespace sr {

// ---------------------------------------------------------------------------
// Host-side error state (per calling thread), read by sr_last_error().
// ---------------------------------------------------------------------------
int fail(int code, const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);
void clear_error();

// Status word kept in the first bytes of every workspace.
enum : int { STATUS_OK = 0, STATUS_WAIT_TIMEOUT = 1 };

// Number of output arrays per comp (synchrad/calc.py:458-465).
inline int n_outputs(int comp) {
  switch (comp) {
    case SR_COMP_TOTAL: return 1;
    case SR_COMP_CARTESIAN: return 3;
    case SR_COMP_CARTESIAN_COMPLEX: return 6;
    case SR_COMP_SPHERIC: return 3;
    case SR_COMP_SPHERIC_COMPLEX: return 6;
    default: return 0;
  }
}

// Snapshot schedule of one track, restating the state machine of
// synchrad/kernel_farfield.cl:53-57 and :100-106: the index advances only when
// itStart + it + 2 equals the current snapshot iteration, so a snapshot that is
// missed (repeated or too early iteration) stops every later one.
struct SnapState {
  int64_t fire_it;  // local iteration of the next write, or NEVER
  uint32_t k;       // snapshot index it writes
  static constexpr int64_t NEVER = INT64_MAX;

  __host__ __device__ void init(uint32_t itStart, uint32_t itEnd,
                                const uint32_t *snaps, uint32_t n_snaps) {
    k = 0;
    while (k < n_snaps && !(itStart < snaps[k])) ++k;
    fire_it = NEVER;
    if (k < n_snaps) {
      const int64_t f = (int64_t)snaps[k] - 2 - (int64_t)itStart;
      if (f >= 0 && f <= (int64_t)itEnd - 2) fire_it = f;
    }
  }
  // Call after the write at fire_it.
  __host__ __device__ void advance(uint32_t itStart, uint32_t itEnd,
                                   const uint32_t *snaps, uint32_t n_snaps) {
    const int64_t prev = fire_it;
    ++k;
    fire_it = NEVER;
    if (k < n_snaps) {
      const int64_t f = (int64_t)snaps[k] - 2 - (int64_t)itStart;
      if (f > prev && f <= (int64_t)itEnd - 2) fire_it = f;
    }
  }
};

// ---------------------------------------------------------------------------
// Double-float ("df", value = hi + lo with |lo| <= ulp(hi)/2) helpers built on
// the error-free transformations of Knuth (TwoSum) and Dekker/Kahan
// (TwoProduct through FMA).
// ---------------------------------------------------------------------------
struct df {
  float hi, lo;
};

__device__ __forceinline__ df df_from_double(double v) {
  const float h = __double2float_rn(v);
  return df{h, __double2float_rn(v - (double)h)};
}
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = a + b;
  const float bb = s - a;
  const float e = (a - (s - bb)) + (b - bb);
  return df{s, e};
}
__device__ __forceinline__ df fast_two_sum(float a, float b) {  // |a| >= |b|
  const float s = a + b;
  return df{s, b - (s - a)};
}
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df df_mul(df a, df b) {
  const float p = a.hi * b.hi;
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p, e);
}
// Product without renormalisation (hi = rounded product, lo = the rest).
__device__ __forceinline__ df df_mul_raw(df a, df b) {
  const float p = a.hi * b.hi;
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return df{p, e};
}

__device__ __forceinline__ df df_neg(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df df_sub(df a, df b) { return df_add(a, df_neg(b)); }
// sqrt of a positive double-float: a float root from the hardware reciprocal
// square root, refined by one Newton step on the exact residual a - x^2
// (TwoProduct through FMA), which also absorbs the approximate root's error.
__device__ __forceinline__ df df_sqrt(df a) {
  if (!(a.hi > 0.f)) return df{0.f, 0.f};
  const float y = rsqrtf(a.hi);  // ~1/sqrt(a)
  const float x = a.hi * y;
  const float p = x * x;
  const float e = __fmaf_rn(x, x, -p);
  const float r = ((a.hi - p) - e) + a.lo;
  return fast_two_sum(x, r * (0.5f * y));
}
// a / b for double-floats: an approximate quotient, its exact remainder and
// one correction (the correction absorbs the first quotient's error).
__device__ __forceinline__ df df_div(df a, df b) {
  const float rb = __frcp_rn(b.hi);
  const float q1 = a.hi * rb;
  const df qb = df_mul(df{q1, 0.f}, b);
  const df r = df_sub(a, qb);
  const float q2 = (r.hi + r.lo) * rb;
  return fast_two_sum(q1, q2);
}

// 2*pi split for the Cody-Waite style reduction below.
#define SR_TWO_PI_HI 6.28318548202514648f
#define SR_TWO_PI_LO (-1.74845553146951720e-07f)
#define SR_INV_TWO_PI 0.159154943091895336f

// Reduce a double-float phase p = hi + lo to r in about [-pi, pi] with
// r = p - 2*pi*n.  n*TWO_PI_HI is split exactly by an FMA, and hi - fl(n*2pi_hi)
// is exact by Sterbenz's lemma since both lie within a factor of two once
// |hi| >= pi.  The result is accurate to a few ulp of pi for |p| < 2^22.
__device__ __forceinline__ float reduce_2pi(float hi, float lo) {
  const float n = rintf(hi * SR_INV_TWO_PI);
  const float h = n * SR_TWO_PI_HI;
  const float he = __fmaf_rn(n, SR_TWO_PI_HI, -h);
  float r = hi - h;
  r = r - he;
  r = r + lo;
  return __fmaf_rn(-n, SR_TWO_PI_LO, r);
}

// ---------------------------------------------------------------------------
// Inline-PTX wrappers: mbarrier, bulk async copy (TMA, non-tensor form),
// global timer for bounded waits.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar,
                                                      uint32_t bytes) {
  asm volatile(
      "mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
          smem_u32(bar)),
      "r"(bytes)
      : "memory");
}
// 1-D bulk copy global -> shared, completion signalled on `bar` (tx bytes).
// Both addresses 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src,
                                         uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes "
      "[%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait on an mbarrier phase: gives up after `limit_ns` nanoseconds and
// returns false (the caller records the timeout in the status word).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity,
                                                  uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  while (true) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s

}  // namespace sr
