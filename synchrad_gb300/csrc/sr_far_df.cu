// Double-float far-field radiation integral for GB300 (sm_103a): spectra of
// FP64 accuracy computed on the FP32 pipe (precision SR_PREC_DF).
//
// The sum is the reference's (synchrad/kernel_farfield.cl:59-107) in the form
// the mixed kernel uses (sr_far_mixed.cu): A carried on theta-hat and phi-hat,
// tau = (t - z) + (1 - cos theta) z - n_x x - n_y y, the |dphase| < pi mask
// decided from |omega| |dtau| with a guard band and the reference's own FP64
// test inside it.  What changes is the arithmetic of every per-point term,
// which here keeps about 48 significant bits (double-float: value = hi + lo):
//  * per (direction, step), in FP64: tau, |dtau|, the amplitude on theta-hat
//    and phi-hat, and the phase d_omega * tau in revolutions, whose whole turns
//    are dropped exactly; the rotations R = exp(i d_omega tau) and R^2 as
//    double-floats;
//  * per lane and step: the phase of its first point, omega_0 tau, from a
//    double-float frequency and tau, whole turns dropped, and exp(2 pi i f) of
//    the fraction f from a 1024-entry double-float table of exp(2 pi i k/1024)
//    times a Taylor step over the remaining |2 pi r| <= pi/1024;
//  * the lane's K points in pairs: rotation of a pair by R^2 and the four
//    accumulations A_theta, A_phi (re, im) as packed double-float arithmetic
//    (FFMA2 / FADD2 / FMUL2 error-free transformations);
//  * per-track |A|^2 (or the comp's components) in FP64 into per-subset
//    partial spectra, added in fixed order: deterministic results.
// The accumulators keep a hi sum with its TwoSum errors, product errors and
// cross terms gathered in a lo sum: after N steps the sum is accurate to about
// N 2^-48 of the terms' magnitudes.
//
// Decomposition: a warp owns 32/L directions and, for each, an omega tile of
// L*K points; a CTA of kDW warps owns kDW consecutive warp tasks and one track
// subset; one CTA per (task group, subset) item.  Every warp reads the FP64
// step records of its subset directly (one record per lane per 32-step chunk,
// coalesced) and broadcasts its per-(direction, step) setup through shared
// memory.  Nothing waits on another CTA or on an asynchronous copy.
#include <algorithm>
#include <cmath>

#include "sr_common.cuh"
#include "sr_internal.h"
#include "sr_mixed_common.cuh"

namespace sr {
namespace {

constexpr int kDW = 8;           // warps per CTA
constexpr int kTabBits = 10;
constexpr int kTab = 1 << kTabBits;  // exp(2 pi i k / kTab) table entries
constexpr int kDMaxDpw = 4;      // directions per warp
constexpr int kDSetupF4 = 4;     // float4 per (direction, step) in the setup

// Per-step record in FP64 (96 bytes): q = t - z, x, y, z, bbar (3),
// 1 - bbar_z, a (3) as in the mixed records (far_prepass_kernel), unrounded.
struct __align__(16) DfRecord {
  double q, x, y, z, bx, by, bz, omb, ax, ay, az, pad;
};

template <typename TT>
__global__ void df_prepass_kernel(FarMixedParams p, DfRecord *rec) {
  const TT *X = (const TT *)p.x, *Y = (const TT *)p.y, *Z = (const TT *)p.z;
  const TT *UX = (const TT *)p.ux, *UY = (const TT *)p.uy, *UZ = (const TT *)p.uz;
  const double dtInv = 1.0 / p.dt;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.total_steps;
       g += (int64_t)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = p.n_tracks;  // track of step g: last t with offsets[t] <= g
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (p.offsets[mid] <= g) lo = mid; else hi = mid;
    }
    const uint32_t t = lo;
    const int64_t base = p.offsets[t];
    const int64_t n = p.offsets[t + 1] - base;
    const int64_t s = g - base;
    DfRecord r;
    if (s + 1 >= n) {
      r.q = r.x = r.y = r.z = r.bx = r.by = r.bz = r.omb = r.ax = r.ay = r.az = r.pad = 0.0;
      rec[g] = r;
      continue;
    }
    const double time = (double)(uint32_t)(p.it_start[t] + (uint32_t)s) * p.dt;
    r.x = (double)X[g];
    r.y = (double)Y[g];
    r.z = (double)Z[g];
    r.q = time - r.z;
    double b0[3], b1[3], omb[2];
    for (int k = 0; k < 2; ++k) {
      const double ux = (double)UX[g + k], uy = (double)UY[g + k], uz = (double)UZ[g + k];
      const double tr = ux * ux + uy * uy;
      const double gam = sqrt(1.0 + (tr + uz * uz));
      const double gi = 1.0 / gam;
      double *b = k ? b1 : b0;
      b[0] = ux * gi; b[1] = uy * gi; b[2] = uz * gi;
      omb[k] = (uz > 0.0) ? (1.0 + tr) / (gam * (gam + uz)) : (gam - uz) * gi;
    }
    r.bx = 0.5 * (b1[0] + b0[0]);
    r.by = 0.5 * (b1[1] + b0[1]);
    r.bz = 0.5 * (b1[2] + b0[2]);
    r.omb = 0.5 * (omb[0] + omb[1]);
    r.ax = (b1[0] - b0[0]) * dtInv;
    r.ay = (b1[1] - b0[1]) * dtInv;
    r.az = (b1[2] - b0[2]) * dtInv;
    r.pad = 0.0;
    rec[g] = r;
  }
}

// exp(2 pi i k / kTab) = (cos hi, cos lo, sin hi, sin lo), from FP64 sincospi.
__global__ void df_table_kernel(float4 *tab) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < kTab) {
    double s, c;
    sincospi(2.0 * (double)k / (double)kTab, &s, &c);
    const df ch = df_from_double(c), sh = df_from_double(s);
    tab[k] = make_float4(ch.hi, ch.lo, sh.hi, sh.lo);
  }
}

// exp(2 pi i f) for a double-float fraction |f| <= 1/2 (+ a few ulp):
// table entry k = rint(f kTab) times exp(i theta), theta = 2 pi (f - k/kTab),
// |theta| <= pi/kTab: sin = theta - theta^3/6, cos = 1 - theta^2/2 + theta^4/24
// (the first dropped terms are below 3e-15).
__device__ __forceinline__ void df_cis(const float4 *tab, df f, df &c, df &s) {
  const float kf = rintf(f.hi * (float)kTab);
  const float4 T = tab[((int)kf) & (kTab - 1)];
  const df r = two_sum(f.hi - kf * (1.0f / (float)kTab), f.lo);  // the difference is exact
  const df th = df_mul(df{SR_TWO_PI_HI, SR_TWO_PI_LO}, r);
  const float t2 = th.hi * th.hi;
  float e2 = __fmaf_rn(th.hi, th.hi, -t2);
  e2 = __fmaf_rn(2.0f * th.hi, th.lo, e2);  // theta^2 = t2 + e2
  const df sn = fast_two_sum(th.hi, th.lo - th.hi * t2 * (1.0f / 6.0f));
  df cs = two_sum(1.0f, -0.5f * t2);
  cs.lo += t2 * t2 * (1.0f / 24.0f) - 0.5f * e2;
  cs = fast_two_sum(cs.hi, cs.lo);
  const df Tc{T.x, T.y}, Ts{T.z, T.w};
  c = df_sub(df_mul(Tc, cs), df_mul(Ts, sn));
  s = df_add(df_mul(Tc, sn), df_mul(Ts, cs));
}

// Whole revolutions of a double-float phase dropped: the fraction in about
// [-1/2, 1/2] (hi - rint(hi) is exact).
__device__ __forceinline__ df df_frac(df r) {
  const float n = rintf(r.hi);
  return two_sum(r.hi - n, r.lo);
}

// ---- packed double-float pairs (two points per register pair) ----
struct df2 {
  float2 hi, lo;
};
__device__ __forceinline__ float2 f2(float a) { return make_float2(a, a); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {  // a - b, one rounding
  return __ffma2_rn(b, f2(-1.0f), a);
}
__device__ __forceinline__ void two_sum2(float2 a, float2 b, float2 &s, float2 &e) {
  s = __fadd2_rn(a, b);
  const float2 bb = sub2(s, a);
  e = __fadd2_rn(sub2(a, sub2(s, bb)), sub2(b, bb));
}
// acc += a z for a double-float scalar a = (ah, al) broadcast (nah = -ah).
__device__ __forceinline__ void df2_acc(df2 &acc, float2 ah, float2 al, float2 nah,
                                        const df2 &z) {
  const float2 p = __fmul2_rn(ah, z.hi);
  const float2 ne = __ffma2_rn(nah, z.hi, p);  // p - ah z.hi: the product's error, negated
  const float2 cr = __ffma2_rn(ah, z.lo, __fmul2_rn(al, z.hi));
  float2 s, e;
  two_sum2(acc.hi, p, s, e);
  acc.hi = s;
  acc.lo = __fadd2_rn(acc.lo, __fadd2_rn(e, sub2(cr, ne)));
}
// a x + b y for pairs a, b and per-slot double-floats x, y (nxh = -x.hi,
// nyh = -y.hi), renormalised.
__device__ __forceinline__ df2 df2_dot(const df2 &a, float2 xh, float2 xl, float2 nxh,
                                       const df2 &b, float2 yh, float2 yl, float2 nyh) {
  const float2 p1 = __fmul2_rn(a.hi, xh);
  const float2 ne1 = __ffma2_rn(a.hi, nxh, p1);
  const float2 p2 = __fmul2_rn(b.hi, yh);
  const float2 ne2 = __ffma2_rn(b.hi, nyh, p2);
  float2 s, e;
  two_sum2(p1, p2, s, e);
  float2 cr = __ffma2_rn(a.hi, xl, __fmul2_rn(a.lo, xh));
  cr = __ffma2_rn(b.hi, yl, __ffma2_rn(b.lo, yh, cr));
  const float2 lo = __fadd2_rn(e, sub2(cr, __fadd2_rn(ne1, ne2)));
  df2 r;
  r.hi = __fadd2_rn(s, lo);
  r.lo = sub2(lo, sub2(r.hi, s));
  return r;
}

// Per-direction constants of a work item.
struct DirConstDf {
  double sT, cT, sPh, cPh, n0, n1, omc;  // omc = 1 - cos(theta)
  double tprev;                          // tau of the step before the current chunk
};

template <int K>
struct DfAcc {  // pairs of points, 4 sums each: A_theta re/im, A_phi re/im
  df2 tr[K / 2], ti[K / 2], pr[K / 2], pi[K / 2];
};

template <int K>
__global__ void __launch_bounds__(kDW * 32, 1)
    far_df_kernel(FarMixedParams p, const DfRecord *__restrict__ rec,
                  const float4 *__restrict__ gtab) {
  static_assert(K == 8, "K (more points per lane spill at 255 registers)");
  constexpr int KP = K / 2;
  __shared__ float4 tab[kTab];
  __shared__ DirConstDf dcs[kDW][kDMaxDpw];
  extern __shared__ float4 setup_all[];  // [kDW][dpw][kDSetupF4][32]
  for (int i = threadIdx.x; i < kTab; i += blockDim.x) tab[i] = gtab[i];

  const int dpw = (int)p.dpw, L = 32 / dpw;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int dsub = lane / L, ll = lane % L;
  float4 *setup = setup_all + (size_t)warp * 32 * dpw * kDSetupF4;

  const uint32_t nO = p.n_omega, nT = p.n_theta;
  const uint32_t n_dirs = nT * p.n_phi;
  const uint64_t P = (uint64_t)nO * n_dirs;
  const uint32_t n_groups_dir = (n_dirs + dpw - 1) / dpw;
  const uint32_t n_wt = n_groups_dir * p.n_wtiles;
  const double inv2pi = 0.15915494309189533577;
  const double dw_glob = (nO > 1) ? (p.omega[nO - 1] - p.omega[0]) / (double)(nO - 1) : 0.0;
  const double dw_rev = dw_glob * inv2pi;

  const uint32_t item = blockIdx.x;
  const uint32_t sub = item / p.n_groups, grp = item % p.n_groups;
  const uint32_t wt = grp * kDW + warp;
  const bool active_w = wt < n_wt;
  const uint32_t dgrp = active_w ? wt / p.n_wtiles : 0u;
  const uint32_t tile = active_w ? wt % p.n_wtiles : 0u;
  const uint32_t dir_raw = dgrp * dpw + dsub;
  const bool active = active_w && dir_raw < n_dirs;
  const uint32_t dir = active ? dir_raw : 0u;
  const int j0 = (int)(tile * (uint32_t)(L * K)) + ll * K;
  const int nv = active ? max(0, min(K, (int)nO - j0)) : 0;

  if (ll == 0) {
    const uint32_t iT = dir % nT, iP = dir / nT;
    DirConstDf &d = dcs[warp][dsub];
    d.sT = p.sin_theta[iT];
    d.cT = p.cos_theta[iT];
    d.sPh = p.sin_phi[iP];
    d.cPh = p.cos_phi[iP];
    d.n0 = d.sT * d.cPh;
    d.n1 = d.sT * d.sPh;
    d.omc = 1.0 - d.cT;
    d.tprev = 0.0;
  }
  // lane constants: first frequency in revolutions, uniformity, |omega| range
  const double w0d = nv > 0 ? p.omega[j0] : 0.0;
  const df w0_rev = df_from_double(w0d * inv2pi);
  const float w0f = (float)w0d, dwf = (float)dw_glob;
  const float inv_dwf = (dwf != 0.f) ? 1.0f / dwf : 0.f;
  bool uniform = true;
  float wabs_min = 3.0e38f, wabs_max = 0.f;
  for (int m = 0; m < nv; ++m) {
    const double wm = p.omega[j0 + m];
    if (fabs(wm - (w0d + (double)m * dw_glob)) > 1e-12 * fabs(wm) + 1e-300) uniform = false;
    wabs_min = fminf(wabs_min, (float)fabs(wm));
    wabs_max = fmaxf(wabs_max, (float)fabs(wm));
  }
  if (nv == 0) { wabs_min = 0.f; wabs_max = 0.f; }
  __syncthreads();  // table and direction constants

  uint32_t t0, t1;
  subset_tracks(p, sub, t0, t1);
  for (uint32_t t = t0; t < t1; ++t) {
    const int64_t base = p.offsets[t];
    const uint32_t n_body = track_body(p, t);
    const uint32_t it_start = p.it_start[t], it_end = p.it_end[t];
    const double wp = p.weight[t];
    const uint32_t *snaps = p.snap_its + (size_t)t * p.snap_stride;
    SnapState snap;
    snap.init(it_start, it_end, snaps, p.n_snaps);
    DfAcc<K> acc;
#pragma unroll
    for (int q = 0; q < KP; ++q) {
      acc.tr[q].hi = acc.tr[q].lo = acc.ti[q].hi = acc.ti[q].lo = f2(0.f);
      acc.pr[q].hi = acc.pr[q].lo = acc.pi[q].hi = acc.pi[q].lo = f2(0.f);
    }

    // Snapshot write: A from the double-float sums, per comp, in FP64.
    auto flush = [&](uint32_t ksnap) {
      if (!active) return;
      const DirConstDf &d = dcs[warp][dsub];
      const double wpdt2 = wp * p.dt * p.dt;
      const double wpdt = sqrt(wp) * p.dt;
      const double thxd = d.cT * d.cPh, thyd = d.cT * d.sPh, thzd = -d.sT;
      const double phxd = -d.sPh, phyd = d.cPh;
      double *part = p.partial + ((uint64_t)sub * p.n_out * p.n_snaps) * P;
#pragma unroll
      for (int q = 0; q < KP; ++q) {
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int m = 2 * q + e;
          if (m >= nv) continue;
          auto val = [&](const df2 &v) {
            return e ? (double)v.hi.y + (double)v.lo.y : (double)v.hi.x + (double)v.lo.x;
          };
          const double Ar = val(acc.tr[q]), Ai = val(acc.ti[q]);
          const double Br = val(acc.pr[q]), Bi = val(acc.pi[q]);
          const uint64_t gti = (uint64_t)(j0 + m) + (uint64_t)nO * dir;
          if (p.save_A != nullptr) {  // the adjoint's forward record, per snapshot
            float4 *sa = reinterpret_cast<float4 *>(p.save_A) +
                         ((uint64_t)t * p.n_snaps + ksnap) * P + gti;
            *sa = make_float4((float)Ar, (float)Ai, (float)Br, (float)Bi);
          }
          auto add = [&](int c, double v) {
            part[((uint64_t)c * p.n_snaps + ksnap) * P + gti] += v;
          };
          switch (p.comp) {
            case SR_COMP_TOTAL:
              add(0, wpdt2 * (Ar * Ar + Ai * Ai + Br * Br + Bi * Bi));
              break;
            case SR_COMP_CARTESIAN: {
              const double xr = thxd * Ar + phxd * Br, xi = thxd * Ai + phxd * Bi;
              const double yr = thyd * Ar + phyd * Br, yi = thyd * Ai + phyd * Bi;
              const double zr = thzd * Ar, zi = thzd * Ai;
              add(0, wpdt2 * (xr * xr + xi * xi));
              add(1, wpdt2 * (yr * yr + yi * yi));
              add(2, wpdt2 * (zr * zr + zi * zi));
              break;
            }
            case SR_COMP_CARTESIAN_COMPLEX: {
              const double f = wpdt * p.form_factor[j0 + m];
              add(0, f * (thxd * Ar + phxd * Br));
              add(1, f * (thxd * Ai + phxd * Bi));
              add(2, f * (thyd * Ar + phyd * Br));
              add(3, f * (thyd * Ai + phyd * Bi));
              add(4, f * (thzd * Ar));
              add(5, f * (thzd * Ai));
              break;
            }
            case SR_COMP_SPHERIC:
              add(1, wpdt2 * (Ar * Ar + Ai * Ai));
              add(2, wpdt2 * (Br * Br + Bi * Bi));
              break;
            default:  // SR_COMP_SPHERIC_COMPLEX (FormFactor not applied)
              add(2, wpdt * Ar);
              add(3, wpdt * Ai);
              add(4, wpdt * Br);
              add(5, wpdt * Bi);
              break;
          }
        }
      }
    };

    for (uint32_t s0 = 0; s0 < n_body; s0 += 32) {
      const uint32_t mcnt = min(32u, n_body - s0);
      if (active_w) {
        // ---- per-(direction, step) setup: lane l -> step s0 + l ----
        {
          const uint32_t l = (uint32_t)lane < mcnt ? (uint32_t)lane : mcnt - 1;
          const DfRecord r = rec[base + s0 + l];
          const bool first = (s0 + l) == 0;
          for (int dd = 0; dd < dpw; ++dd) {
            DirConstDf &d = dcs[warp][dd];
            const double tau = r.q + d.omc * r.z - d.n0 * r.x - d.n1 * r.y;
            double prev = __shfl_up_sync(0xffffffffu, tau, 1);
            if (lane == 0) prev = d.tprev;
            // the track's first step compares the phase with zero
            // (synchrad/kernel_farfield.cl:49, 65-72)
            const double dtau = first ? tau : tau - prev;
            const double D = r.omb + d.omc * r.bz - d.n0 * r.bx - d.n1 * r.by;
            const double c2 = 1.0 / D;
            const double an = d.n0 * r.ax + d.n1 * r.ay + d.cT * r.az;
            const double c1 = an * c2 * c2;
            const double thx = d.cT * d.cPh, thy = d.cT * d.sPh, thz = -d.sT;
            const double tb = thx * r.bx + thy * r.by + thz * r.bz;
            const double ta = thx * r.ax + thy * r.ay + thz * r.az;
            const double pb = -d.sPh * r.bx + d.cPh * r.by;
            const double pa = -d.sPh * r.ax + d.cPh * r.ay;
            const df at = df_from_double(-(c1 * tb + c2 * ta));
            const df ap = df_from_double(-(c1 * pb + c2 * pa));
            // R = exp(2 pi i dw_rev tau), whole turns dropped in FP64 (exact)
            const double rr = dw_rev * tau;
            df Rc, Rs;
            df_cis(tab, df_from_double(rr - rint(rr)), Rc, Rs);
            const df R2c = df_sub(df_mul(Rc, Rc), df_mul(Rs, Rs));
            const df R2s = df_mul(df{2.f * Rs.hi, 2.f * Rs.lo}, Rc);
            const df tdf = df_from_double(tau);
            float4 *st = setup + (size_t)dd * kDSetupF4 * 32 + lane;
            st[0 * 32] = make_float4(tdf.hi, tdf.lo, (float)fabs(dtau), 0.f);
            st[1 * 32] = make_float4(at.hi, at.lo, ap.hi, ap.lo);
            st[2 * 32] = make_float4(Rc.hi, Rc.lo, Rs.hi, Rs.lo);
            st[3 * 32] = make_float4(R2c.hi, R2c.lo, R2s.hi, R2s.lo);
            const double last = __shfl_sync(0xffffffffu, tau, mcnt - 1);
            __syncwarp();
            if (lane == 0) d.tprev = last;
          }
        }
        __syncwarp();
        // ---- the points: K per lane, in pairs ----
#pragma unroll 1
        for (uint32_t i = 0; i < mcnt; ++i) {
          const uint32_t s = s0 + i;
          const float4 *st = setup + (size_t)dsub * kDSetupF4 * 32 + i;
          const float4 S0 = st[0], S1 = st[32], S2 = st[64], S3 = st[96];
          const float adt = S0.z;
          const bool all_in = wabs_max * adt < kPiLo;
          const bool all_out = wabs_min * adt > kPiHi;
          uint32_t mask = (nv == 0 || all_out) ? 0u : (nv >= 32 ? 0xffffffffu : ((1u << nv) - 1u));
          if (nv > 0 && !all_in && !all_out) {
            const DirConstDf &d = dcs[warp][dsub];
            if (uniform) {
              const float inv_adt = __frcp_rn(adt);  // adt > 0 here
              mask = omega_range_bits_r(w0f, dwf, inv_dwf, kPiLo * inv_adt, nv);
              uint32_t unc = omega_range_bits_r(w0f, dwf, inv_dwf, kPiHi * inv_adt, nv) & ~mask;
              while (unc) {
                const int m = __ffs(unc) - 1;
                unc &= unc - 1u;
                if (exact_mask(p, base, s, it_start, p.omega[j0 + m], d.n0, d.n1, d.cT))
                  mask |= 1u << m;
              }
            } else {
              mask = 0;
#pragma unroll 1
              for (int m = 0; m < nv; ++m) {
                const double wm = p.omega[j0 + m];
                const float ph = (float)fabs(wm) * adt;
                bool inc;
                if (ph < kPiLo) inc = true;
                else if (ph > kPiHi) inc = false;
                else inc = exact_mask(p, base, s, it_start, wm, d.n0, d.n1, d.cT);
                mask |= (uint32_t)inc << m;
              }
            }
          }
          if (mask != 0u) {
            const df tau{S0.x, S0.y};
            const float2 ath = f2(S1.x), atl = f2(S1.y), natb = f2(-S1.x);
            const float2 aph = f2(S1.z), apl = f2(S1.w), napb = f2(-S1.z);
            // first pair: (z0, z0 R), z0 = exp(2 pi i omega_0 tau)
            df2 zr, zi;
            {
              df c0, s0v;
              df_cis(tab, df_frac(df_mul_raw(w0_rev, tau)), c0, s0v);
              df2 a, b;
              a.hi = f2(c0.hi); a.lo = f2(c0.lo);
              b.hi = f2(s0v.hi); b.lo = f2(s0v.lo);
              // slot 0: (1, 0); slot 1: R
              const float2 xh = make_float2(1.f, S2.x), xl = make_float2(0.f, S2.y);
              const float2 yh = make_float2(0.f, S2.z), yl = make_float2(0.f, S2.w);
              zr = df2_dot(a, xh, xl, make_float2(-1.f, -S2.x), b, make_float2(0.f, -S2.z),
                           make_float2(0.f, -S2.w), make_float2(0.f, S2.z));
              zi = df2_dot(a, yh, yl, make_float2(0.f, -S2.z), b, xh, xl,
                           make_float2(-1.f, -S2.x));
            }
            const float2 r2ch = f2(S3.x), r2cl = f2(S3.y), nr2ch = f2(-S3.x);
            const float2 r2sh = f2(S3.z), r2sl = f2(S3.w), nr2sh = f2(-S3.z);
#pragma unroll
            for (int q = 0; q < KP; ++q) {
              if (!uniform) {  // non-uniform axis: each point's own phase
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                  const int m = min(2 * q + e, max(nv - 1, 0));
                  df c0, s0v;
                  df_cis(tab, df_frac(df_mul_raw(df_from_double(p.omega[j0 + m] * inv2pi), tau)),
                         c0, s0v);
                  if (e == 0) {
                    zr.hi.x = c0.hi; zr.lo.x = c0.lo; zi.hi.x = s0v.hi; zi.lo.x = s0v.lo;
                  } else {
                    zr.hi.y = c0.hi; zr.lo.y = c0.lo; zi.hi.y = s0v.hi; zi.lo.y = s0v.lo;
                  }
                }
              }
              const float g0 = ((mask >> (2 * q)) & 1u) ? 1.f : 0.f;
              const float g1 = ((mask >> (2 * q + 1)) & 1u) ? 1.f : 0.f;
              const float2 g = make_float2(g0, g1);
              const float2 at_h = __fmul2_rn(ath, g), at_l = __fmul2_rn(atl, g),
                           nat_h = __fmul2_rn(natb, g);
              const float2 ap_h = __fmul2_rn(aph, g), ap_l = __fmul2_rn(apl, g),
                           nap_h = __fmul2_rn(napb, g);
              df2_acc(acc.tr[q], at_h, at_l, nat_h, zr);
              df2_acc(acc.ti[q], at_h, at_l, nat_h, zi);
              df2_acc(acc.pr[q], ap_h, ap_l, nap_h, zr);
              df2_acc(acc.pi[q], ap_h, ap_l, nap_h, zi);
              if (q + 1 < KP && uniform) {
                const df2 nr = df2_dot(zr, r2ch, r2cl, nr2ch, zi, f2(-S3.z), f2(-S3.w), r2sh);
                const df2 ni = df2_dot(zr, r2sh, r2sl, nr2sh, zi, r2ch, r2cl, nr2ch);
                zr = nr;
                zi = ni;
              }
            }
          }
          if ((int64_t)s == snap.fire_it) {  // uniform over the CTA
            flush(snap.k);
            snap.advance(it_start, it_end, snaps, p.n_snaps);
          }
        }
        __syncwarp();
      } else {
        for (uint32_t i = 0; i < mcnt; ++i)
          if ((int64_t)(s0 + i) == snap.fire_it) snap.advance(it_start, it_end, snaps, p.n_snaps);
      }
    }
    while (snap.fire_it != SnapState::NEVER) {  // writes due after the last body step
      flush(snap.k);
      snap.advance(it_start, it_end, snaps, p.n_snaps);
    }
    if (ll == 0) dcs[warp][dsub].tprev = 0.0;  // the next track starts afresh
    __syncwarp();
  }
}

struct DfLayout {
  size_t records, partial, table, total;
};

DfLayout df_layout(int64_t total_steps, uint64_t P, int n_out, uint32_t n_snaps, int n_sub) {
  DfLayout l;
  size_t off = 256;  // status word
  l.records = off;
  off += ((size_t)total_steps * sizeof(DfRecord) + 255) / 256 * 256;
  l.partial = off;
  off += ((size_t)n_sub * n_out * n_snaps * P * 8 + 255) / 256 * 256;
  l.table = off;
  off += (size_t)kTab * sizeof(float4);
  l.total = off;
  return l;
}

template <int K>
int launch_df_main(const FarMixedParams &p, const DfRecord *rec, const float4 *tab,
                   cudaStream_t s) {
  const size_t smem = (size_t)kDW * 32 * p.dpw * kDSetupF4 * sizeof(float4);
  cudaError_t e = cudaFuncSetAttribute(far_df_kernel<K>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "far_df smem attribute");
  far_df_kernel<K><<<p.n_items, kDW * 32, smem, s>>>(p, rec, tab);
  return cuda_fail(cudaGetLastError(), "far_df kernel launch");
}

}  // namespace

// Work shape of the double-float far field: K = 8 points per lane (the 64
// double-float accumulator pairs of 16 points spill at 255 registers), L lanes
// per direction, and track subsets for about four CTAs per SM.
FarMixedConfig far_df_choose(uint32_t n_omega, uint32_t n_dirs, uint32_t n_tracks, int n_sm) {
  FarMixedConfig c;
  c.W = kDW;
  c.ctas_per_sm = 1;
  c.stage = 32;
  c.K = 8;
  int L = 32;
  while (L > 32 / kDMaxDpw && (uint32_t)(L / 2) * c.K >= n_omega) L /= 2;
  c.L = L;
  c.dpw = 32 / L;
  const uint64_t n_wtiles = (n_omega + (uint64_t)L * c.K - 1) / ((uint64_t)L * c.K);
  const uint64_t dgroups = (n_dirs + c.dpw - 1) / c.dpw;
  const uint64_t groups = (dgroups * n_wtiles + c.W - 1) / c.W;
  uint64_t nsub = (4 * (uint64_t)n_sm + groups - 1) / (groups ? groups : 1);
  if (nsub > n_tracks) nsub = n_tracks;
  if (nsub < 1) nsub = 1;
  if (nsub > 64) nsub = 64;
  c.n_sub = (int)nsub;
  c.grid = (int)(groups * nsub);
  return c;
}

size_t far_df_workspace(int64_t total_steps, uint64_t n_points, int n_out, uint32_t n_snaps,
                        const FarMixedConfig &cfg) {
  return df_layout(total_steps, n_points, n_out, n_snaps, cfg.n_sub).total;
}

int launch_far_df(FarMixedParams p, const FarMixedConfig &cfg, void *ws, size_t ws_bytes,
                  cudaStream_t stream) {
  const uint64_t P = (uint64_t)p.n_omega * p.n_theta * p.n_phi;
  if (P == 0 || p.n_tracks == 0 || p.n_snaps == 0) return SR_OK;
  const DfLayout lay = df_layout(p.total_steps, P, p.n_out, p.n_snaps, cfg.n_sub);
  if (ws == nullptr || ws_bytes < lay.total)
    return fail(SR_ERR_WORKSPACE, "workspace of %zu bytes needed, %zu given", lay.total, ws_bytes);
  if (((uintptr_t)ws & 255u) != 0) return fail(SR_ERR_WORKSPACE, "workspace not 256-byte aligned");
  if (cfg.K != 8) return fail(SR_ERR_INVALID, "points per lane %d (8)", cfg.K);
  unsigned char *w = (unsigned char *)ws;
  p.status = (int *)w;
  p.partial = (double *)(w + lay.partial);
  DfRecord *rec = (DfRecord *)(w + lay.records);
  float4 *tab = (float4 *)(w + lay.table);
  p.dpw = (uint32_t)cfg.dpw;
  p.n_wtiles = (p.n_omega + (uint32_t)(cfg.L * cfg.K) - 1) / (uint32_t)(cfg.L * cfg.K);
  const uint32_t n_dirs = p.n_theta * p.n_phi;
  const uint32_t dgroups = (n_dirs + cfg.dpw - 1) / cfg.dpw;
  p.n_groups = (uint32_t)(((uint64_t)dgroups * p.n_wtiles + cfg.W - 1) / cfg.W);
  p.n_sub = (uint32_t)cfg.n_sub;
  p.n_items = p.n_groups * p.n_sub;

  cudaError_t e = cudaMemsetAsync(w, 0, 256, stream);
  if (e != cudaSuccess) return cuda_fail(e, "status reset");
  e = cudaMemsetAsync(p.partial, 0, (size_t)p.n_sub * p.n_out * p.n_snaps * P * 8, stream);
  if (e != cudaSuccess) return cuda_fail(e, "partial reset");
  const int n_sm = device_sm_count();
  df_table_kernel<<<(kTab + 255) / 256, 256, 0, stream>>>(tab);
  if (p.total_steps > 0) {
    int64_t nb = (p.total_steps + 255) / 256;
    if (nb > 8 * (int64_t)n_sm * 16) nb = 8 * (int64_t)n_sm * 16;
    if (p.track_f32)
      df_prepass_kernel<float><<<(int)nb, 256, 0, stream>>>(p, rec);
    else
      df_prepass_kernel<double><<<(int)nb, 256, 0, stream>>>(p, rec);
  }
  int rc = cuda_fail(cudaGetLastError(), "far_df prepass launch");
  if (rc) return rc;
  void *tok = nullptr;
  timing_record(stream, true, &tok);
  rc = launch_df_main<8>(p, rec, tab, stream);
  timing_record(stream, false, &tok);
  if (rc) return rc;
  const uint64_t total = (uint64_t)p.n_out * p.n_snaps * P;
  uint64_t nb = (total + 255) / 256;
  if (nb > (uint64_t)n_sm * 64) nb = (uint64_t)n_sm * 64;
  mixed_reduce_kernel<<<(unsigned)nb, 256, 0, stream>>>(p);
  return cuda_fail(cudaGetLastError(), "far_df reduce launch");
}

}  // namespace sr
