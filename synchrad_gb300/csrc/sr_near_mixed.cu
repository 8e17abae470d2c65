// Mixed-precision near-field radiation integral for GB300 (sm_103a).
//
// Computes, per screen point P = (R cos phi, R sin phi, L), frequency omega
// and track, the reference's sum (synchrad/kernel_nearfield.cl:58-102)
//     A = sum_s (n/r^2 + i omega (beta - n)/r) exp(i omega (t_s + r)),
//     r = |P - x_s|, n = (P - x_s)/r, beta at step s,
// over the steps whose phase advance passes |dphase| < pi, and accumulates
// w dt^2 |A|^2 (or the comp's components) over tracks.
//
// Arithmetic (the "mixed" precision):
//  * the omega factor leaves the sum: A = S2 + i omega S1 with
//    S1 = sum (beta - n)/r e^{i phi} and S2 = sum n/r^2 e^{i phi}; a point
//    carries six complex sums and A is formed once per snapshot;
//  * the retarded time tau = t + r is formed in double-float, free of the
//    cancellation of t + |P - x|:  tau = (t - z) + L + rho^2 / (r + (L - z)),
//    rho^2 = (X - x)^2 + (Y - y)^2, with (t - z), x, y, z prepared in FP64;
//    beta_z - n_z = (1 - n_z) - (1 - beta_z), 1 - n_z = rho^2/((r + L - z) r);
//  * phasors, mask, compensated sums and FP64 results as in the far field
//    (sr_far_mixed.cu), with K = 8 or 16 points per lane (six complex sums per
//    point: 48 or 96 packed accumulator registers per lane).
#include <algorithm>
#include <cmath>

#include "sr_common.cuh"
#include "sr_internal.h"
#include "sr_mixed_common.cuh"

namespace sr {
namespace {

constexpr int kNKDefault = 16;  // points per lane (8 or 16)
constexpr int kNW = 8;          // warps per CTA
constexpr int kNMaxDpw = 4;     // screen points per warp
constexpr int kNOuter = 24;     // compensated values per point: 12 sums x (sum, comp)
constexpr int kNSetupF4 = 8;    // float4 per (screen point, step) in the setup

// Pre-pass: per-step records.
//   r0 = (q.hi, q.lo, x.hi, x.lo)   q = t - z, t = (itStart + s) dt
//   r1 = (y.hi, y.lo, z.hi, z.lo)
//   r2 = (beta_x, beta_y, beta_z, 1 - beta_z) at step s
//        (synchrad/kernel_nearfield.cl:79-82), 1 - beta_z = (1+ux^2+uy^2)/(gamma(gamma+uz))
//   r3 = r4 = 0 (padding: an 80-byte record stride spreads per-lane reads over the banks)
template <typename TT>
__global__ void near_prepass_kernel(FarMixedParams p) {
  const TT *X = (const TT *)p.x, *Y = (const TT *)p.y, *Z = (const TT *)p.z;
  const TT *UX = (const TT *)p.ux, *UY = (const TT *)p.uy, *UZ = (const TT *)p.uz;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.total_steps;
       g += (int64_t)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = p.n_tracks;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (p.offsets[mid] <= g) lo = mid; else hi = mid;
    }
    const uint32_t t = lo;
    const int64_t base = p.offsets[t];
    const int64_t n = p.offsets[t + 1] - base;
    const int64_t s = g - base;
    float4 *rec = p.records + g * kRecF4;
    if (s + 1 >= n) {
      const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
      rec[0] = zero; rec[1] = zero; rec[2] = zero; rec[3] = zero; rec[4] = zero;
      continue;
    }
    const double time = (double)(uint32_t)(p.it_start[t] + (uint32_t)s) * p.dt;
    const double x = (double)X[g], y = (double)Y[g], z = (double)Z[g];
    const double ux = (double)UX[g], uy = (double)UY[g], uz = (double)UZ[g];
    const double tr = ux * ux + uy * uy;
    const double gam = sqrt(1.0 + (tr + uz * uz));
    const double gi = 1.0 / gam;
    const double omb = (uz > 0.0) ? (1.0 + tr) / (gam * (gam + uz)) : (gam - uz) * gi;
    const df dq = df_from_double(time - z), dx = df_from_double(x), dy = df_from_double(y),
             dz = df_from_double(z);
    rec[0] = make_float4(dq.hi, dq.lo, dx.hi, dx.lo);
    rec[1] = make_float4(dy.hi, dy.lo, dz.hi, dz.lo);
    rec[2] = make_float4((float)(ux * gi), (float)(uy * gi), (float)(uz * gi), (float)omb);
    rec[3] = make_float4(0.f, 0.f, 0.f, 0.f);
    rec[4] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// Per screen point constants, written once per work item.
struct ScreenConst {
  double P0, P1;                 // R cos(phi), R sin(phi) rounded as the reference does
  float X_h, X_l, Y_h, Y_l;      // the same as double-floats
  float tprev_h, tprev_l;        // tau of the step before the current chunk
  float adt_max;                 // largest |dtau| of the current chunk
  float pad_;
};

template <int W>
struct NearSmemFixed {
  float4 stage[2][kStage * kRecF4];
  uint64_t bar[2];
  uint32_t next_item;   // broadcast of the work item taken from the queue
  uint32_t pad32_;
  uint64_t pad_[1];
  ScreenConst sc[W][kNMaxDpw];
  // followed by float4 setup[W][dpw][kNSetupF4][32]
};

// Packed accumulators of one lane: six complex sums for K points.
template <int K>
struct NearAcc {
  float2 s1r[3][K / 2], s1i[3][K / 2];  // sum (beta - n)/r e^{i phi}, x y z
  float2 s2r[3][K / 2], s2i[3][K / 2];  // sum n/r^2 e^{i phi}
};

// acc += amplitude (pairs) * Z for pair q.
template <int K>
__device__ __forceinline__ void near_accumulate(NearAcc<K> &a, int q, float2 zr, float2 zi,
                                                const float2 (&bb)[3], const float2 (&aa)[3]) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    a.s1r[c][q] = __ffma2_rn(zr, bb[c], a.s1r[c][q]);
    a.s1i[c][q] = __ffma2_rn(zi, bb[c], a.s1i[c][q]);
    a.s2r[c][q] = __ffma2_rn(zr, aa[c], a.s2r[c][q]);
    a.s2i[c][q] = __ffma2_rn(zi, aa[c], a.s2i[c][q]);
  }
}

template <int K, int W>
__global__ void __launch_bounds__(W * 32, 1) near_mixed_kernel(FarMixedParams p) {
  static_assert(K == 8 || K == 16, "K");
  constexpr int KP = K / 2, HP = KP / 2;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  NearSmemFixed<W> &sm = *reinterpret_cast<NearSmemFixed<W> *>(smem_raw);
  const int dpw = (int)p.dpw, L = 32 / dpw;
  float4 *setup_all = reinterpret_cast<float4 *>(smem_raw + sizeof(NearSmemFixed<W>));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int dsub = lane / L, ll = lane % L;
  float4 *setup = setup_all + (size_t)warp * 32 * dpw * kNSetupF4;

  if (threadIdx.x == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  const uint32_t nO = p.n_omega, nR = p.n_theta;
  const uint32_t n_dirs = nR * p.n_phi;
  const uint64_t P = (uint64_t)nO * n_dirs;
  const uint32_t n_groups_dir = (n_dirs + dpw - 1) / dpw;
  const uint32_t n_wt = n_groups_dir * p.n_wtiles;
  const double dw_glob = (nO > 1) ? (p.omega[nO - 1] - p.omega[0]) / (double)(nO - 1) : 0.0;
  const df d_dw = df_from_double(dw_glob);
  const df dL = df_from_double(p.L_screen);
  const double inv2pi = 0.15915494309189533577;
  float *outer = p.outer + ((size_t)blockIdx.x * W + warp) * K * kNOuter * 32;
  uint32_t stage_no = 0;

  // Work items: each CTA starts on its own, then takes the next one from a
  // counter in the workspace (zeroed at launch), so that items of unequal cost
  // (subsets of ragged tracks) keep every SM busy to the end.
  auto next_item = [&]() -> uint32_t {
    __syncthreads();  // every thread has read the previous item number
    if (threadIdx.x == 0) sm.next_item = gridDim.x + atomicAdd(p.queue, 1u);
    __syncthreads();
    return sm.next_item;
  };
  for (uint32_t item = blockIdx.x; item < p.n_items; item = next_item()) {
    const uint32_t sub = item / p.n_groups, grp = item % p.n_groups;
    const uint32_t wt = grp * W + warp;
    const bool active_w = wt < n_wt;
    const uint32_t dgrp = active_w ? wt / p.n_wtiles : 0u;
    const uint32_t tile = active_w ? wt % p.n_wtiles : 0u;
    const uint32_t dir_raw = dgrp * dpw + dsub;
    const bool active = active_w && dir_raw < n_dirs;
    const uint32_t dir = active ? dir_raw : 0u;
    const int j0 = (int)(tile * (uint32_t)(L * K)) + ll * K;
    const int nv = active ? max(0, min(K, (int)nO - j0)) : 0;

    if (ll == 0) {
      const uint32_t iR = dir % nR, iP = dir / nR;
      ScreenConst &c = sm.sc[warp][dsub];
      c.P0 = p.sin_theta[iR] * p.cos_phi[iP];  // radius * cos(phi)
      c.P1 = p.sin_theta[iR] * p.sin_phi[iP];  // radius * sin(phi)
      const df x0 = df_from_double(c.P0), y0 = df_from_double(c.P1);
      c.X_h = x0.hi; c.X_l = x0.lo; c.Y_h = y0.hi; c.Y_l = y0.lo;
      c.tprev_h = 0.f; c.tprev_l = 0.f;
    }
    const double w0d = nv > 0 ? p.omega[j0] : 0.0;
    const df d_w0 = df_from_double(w0d * inv2pi);
    const float w0f = (float)w0d, dwf = (float)dw_glob;
    bool uniform = true;
    float wabs_min = 3.0e38f, wabs_max = 0.f;
    for (int m = 0; m < nv; ++m) {
      const double wm = p.omega[j0 + m];
      if (fabs(wm - (w0d + (double)m * dw_glob)) > 1e-12 * fabs(wm) + 1e-300) uniform = false;
      wabs_min = fminf(wabs_min, (float)fabs(wm));
      wabs_max = fmaxf(wabs_max, (float)fabs(wm));
    }
    if (nv == 0) { wabs_min = 0.f; wabs_max = 0.f; }
    __syncwarp();

    uint32_t t0, t1;
    subset_tracks(p, sub, t0, t1);
    uint32_t cur_t = t0;
    while (cur_t < t1 && track_body(p, cur_t) == 0) ++cur_t;
    if (threadIdx.x == 0 && cur_t < t1) {
      const uint32_t cnt = min((uint32_t)kStage, track_body(p, cur_t));
      const int b = stage_no & 1;
      fence_proxy_async();
      mbar_arrive_expect_tx(&sm.bar[b], cnt * kRecBytes);
      bulk_g2s(sm.stage[b], p.records + (p.offsets[cur_t]) * kRecF4, cnt * kRecBytes,
               &sm.bar[b]);
    }

    for (uint32_t t = t0; t < t1; ++t) {
      const int64_t base = p.offsets[t];
      const uint32_t n_body = track_body(p, t);
      const uint32_t it_start = p.it_start[t], it_end = p.it_end[t];
      const double wp = p.weight[t];
      const uint32_t *snaps = p.snap_its + (size_t)t * p.snap_stride;
      SnapState snap;
      snap.init(it_start, it_end, snaps, p.n_snaps);

      NearAcc<K> acc;
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int q = 0; q < KP; ++q)
          acc.s1r[c][q] = acc.s1i[c][q] = acc.s2r[c][q] = acc.s2i[c][q] = make_float2(0.f, 0.f);
      bool outer_live = false;

      // Folds the FP32 sums into the compensated pairs in the workspace.
      // Value index v: 0-2 S1 re (x,y,z), 3-5 S1 im, 6-8 S2 re, 9-11 S2 im.
      auto fold = [&]() {
        if (!active) return;
#pragma unroll
        for (int m = 0; m < K; ++m) {
          const int q = m >> 1;
#pragma unroll
          for (int v = 0; v < 12; ++v) {
            const int c = v % 3;
            const float2 &pr = (v < 3) ? acc.s1r[c][q] : (v < 6) ? acc.s1i[c][q]
                             : (v < 9) ? acc.s2r[c][q] : acc.s2i[c][q];
            const float val = (m & 1) ? pr.y : pr.x;
            float *o = outer + ((size_t)m * kNOuter + v) * 32 + lane;
            if (outer_live) {
              const df e = two_sum(o[0], val);
              o[0] = e.hi;
              o[12 * 32] += e.lo;
            } else {
              o[0] = val;
              o[12 * 32] = 0.f;
            }
          }
        }
        outer_live = true;
#pragma unroll
        for (int c = 0; c < 3; ++c)
#pragma unroll
          for (int q = 0; q < KP; ++q)
            acc.s1r[c][q] = acc.s1i[c][q] = acc.s2r[c][q] = acc.s2i[c][q] = make_float2(0.f, 0.f);
      };

      // Snapshot write: A_c = S2_c + i omega S1_c (times exp(i omega L), the
      // phase of the screen distance left out of the sums), per comp, FP64.
      auto flush = [&](uint32_t ksnap) {
        fold();
        if (!active) return;
        const double wpdt2 = wp * p.dt * p.dt;
        const double wpdt = sqrt(wp) * p.dt;
        double *part = p.partial + ((uint64_t)sub * p.n_out * p.n_snaps) * P;
#pragma unroll 1
        for (int m = 0; m < nv; ++m) {
          const float *o = outer + (size_t)m * kNOuter * 32 + lane;
          auto val = [&](int v) { return (double)o[v * 32] + (double)o[(v + 12) * 32]; };
          const double w = p.omega[j0 + m];
          double Ar[3], Ai[3];
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            Ar[c] = val(6 + c) - w * val(3 + c);
            Ai[c] = val(9 + c) + w * val(c);
          }
          const uint64_t gti = (uint64_t)(j0 + m) + (uint64_t)nO * dir;
          if (p.save_A != nullptr) {  // the adjoint's forward record, per snapshot
            float4 *sa = reinterpret_cast<float4 *>(p.save_A) +
                         2 * (((uint64_t)t * p.n_snaps + ksnap) * P + gti);
            sa[0] = make_float4((float)Ar[0], (float)Ai[0], (float)Ar[1], (float)Ai[1]);
            sa[1] = make_float4((float)Ar[2], (float)Ai[2], 0.f, 0.f);
          }
          auto add = [&](int c, double v) {
            part[((uint64_t)c * p.n_snaps + ksnap) * P + gti] += v;
          };
          if (p.comp == SR_COMP_TOTAL) {
            add(0, wpdt2 * (Ar[0] * Ar[0] + Ar[1] * Ar[1] + Ar[2] * Ar[2] + Ai[0] * Ai[0] +
                            Ai[1] * Ai[1] + Ai[2] * Ai[2]));
          } else if (p.comp == SR_COMP_CARTESIAN) {
#pragma unroll
            for (int c = 0; c < 3; ++c) add(c, wpdt2 * (Ar[c] * Ar[c] + Ai[c] * Ai[c]));
          } else {  // cartesian_complex (FormFactor not applied)
            double sL, cL;
            sincos(w * p.L_screen, &sL, &cL);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
              add(2 * c, wpdt * (Ar[c] * cL - Ai[c] * sL));
              add(2 * c + 1, wpdt * (Ar[c] * sL + Ai[c] * cL));
            }
          }
        }
      };

      // The first pair's phasors of one step: the reseed e^{i omega_0 tau}
      // (the lane's own sin/cos, interleaved with the other steps' sums) and
      // its product with R = e^{i d_omega tau}.
      auto step_seed = [&](const float4 *st, uint32_t, float2 &ZrA, float2 &ZiA) {
        const float4 A = st[0];
        float zs, zc;
        phasor_rev(d_w0.hi, d_w0.lo, A.x, A.y, zs, zc);
        ZrA = make_float2(zc, zc * A.z - zs * A.w);
        ZiA = make_float2(zs, zc * A.w + zs * A.z);
      };
      // One fully included step on a uniform axis: two packed chains of pairs.
      auto step_fast = [&](const float4 *st, float2 ZrA, float2 ZiA) {
        const float4 F1 = st[1 * 32], F2 = st[2 * 32], F3 = st[3 * 32], R2 = st[4 * 32],
                     X = st[5 * 32], Y = st[6 * 32];
        const float2 aa[3] = {make_float2(F1.x, F1.y), make_float2(F1.z, F1.w),
                              make_float2(F2.x, F2.y)};
        const float2 bb[3] = {make_float2(F2.z, F2.w), make_float2(F3.x, F3.y),
                              make_float2(F3.z, F3.w)};
        const float2 r2c = make_float2(R2.x, R2.y), r2s = make_float2(R2.z, R2.w);
        const float2 nr2s = make_float2(X.x, X.y), hc = make_float2(X.z, X.w);
        const float2 hs = make_float2(Y.x, Y.y), nhs = make_float2(Y.z, Y.w);
        float2 ZrB, ZiB;
        rot2p(ZrA, ZiA, hc, hs, nhs, ZrB, ZiB);
#pragma unroll
        for (int q = 0; q < HP; ++q) {
          near_accumulate(acc, q, ZrA, ZiA, bb, aa);
          near_accumulate(acc, HP + q, ZrB, ZiB, bb, aa);
          if (q + 1 < HP) {
            rot2p(ZrA, ZiA, r2c, r2s, nr2s, ZrA, ZiA);
            rot2p(ZrB, ZiB, r2c, r2s, nr2s, ZrB, ZiB);
          }
        }
      };

      uint32_t stage_in_track = 0;
      for (uint32_t s0 = 0; s0 < n_body; s0 += kStage, ++stage_in_track) {
        const uint32_t cnt = min((uint32_t)kStage, n_body - s0);
        const int b = stage_no & 1;
        if (threadIdx.x == 0) {
          uint32_t nt = t, ns0 = s0 + kStage;
          if (ns0 >= n_body) {
            nt = t + 1;
            ns0 = 0;
            while (nt < t1 && track_body(p, nt) == 0) ++nt;
          }
          if (nt < t1) {
            const uint32_t ncnt = min((uint32_t)kStage, track_body(p, nt) - ns0);
            const int nbuf = (stage_no + 1) & 1;
            fence_proxy_async();
            mbar_arrive_expect_tx(&sm.bar[nbuf], ncnt * kRecBytes);
            bulk_g2s(sm.stage[nbuf], p.records + (p.offsets[nt] + ns0) * kRecF4, ncnt * kRecBytes,
                     &sm.bar[nbuf]);
          }
        }
        const bool ok = mbar_wait_bounded(&sm.bar[b], (stage_no >> 1) & 1, kWaitLimitNs);
        if (__syncthreads_or(!ok)) {
          if (threadIdx.x == 0) {
            atomicExch(p.status, STATUS_WAIT_TIMEOUT);
            mbar_wait_bounded(&sm.bar[(stage_no + 1) & 1], ((stage_no + 1) >> 1) & 1,
                              kWaitLimitNs);
          }
          __syncthreads();
          return;
        }
        const float4 *stg = sm.stage[b];

        if (active_w) {
          for (uint32_t c0 = 0; c0 < cnt; c0 += 32) {
            const uint32_t mcnt = min(32u, cnt - c0);
            // ---- per-step setup: lane l -> step s0 + c0 + l, every screen point ----
            {
              const uint32_t l = (uint32_t)lane < mcnt ? (uint32_t)lane : mcnt - 1;
              const float4 r0 = stg[(c0 + l) * kRecF4 + 0];
              const float4 r1 = stg[(c0 + l) * kRecF4 + 1];
              const float4 r2 = stg[(c0 + l) * kRecF4 + 2];
              const bool first = (s0 + c0 + l) == 0;
              for (int dd = 0; dd < dpw; ++dd) {
                ScreenConst &c = sm.sc[warp][dd];
                // tau' = t + r - L = (t - z) + rho^2/(r + L - z)   (double-float)
                const df ddx = df_sub(df{c.X_h, c.X_l}, df{r0.z, r0.w});
                const df ddy = df_sub(df{c.Y_h, c.Y_l}, df{r1.x, r1.y});
                const df D = df_sub(dL, df{r1.z, r1.w});
                const df rho2 = df_add(df_mul(ddx, ddx), df_mul(ddy, ddy));
                const df r = df_sqrt(df_add(rho2, df_mul(D, D)));
                const df F = (D.hi > 0.f) ? df_div(rho2, df_add(r, D)) : df_sub(r, D);
                const df tau = df_add(df{r0.x, r0.y}, F);
                float ph = __shfl_up_sync(0xffffffffu, tau.hi, 1);
                float pl = __shfl_up_sync(0xffffffffu, tau.lo, 1);
                if (lane == 0) { ph = c.tprev_h; pl = c.tprev_l; }
                // the track's first step compares the whole phase with zero
                // (synchrad/kernel_nearfield.cl:48, 70-72)
                const float dtau = first ? ((tau.hi + tau.lo) + (dL.hi + dL.lo))
                                         : ((tau.hi - ph) + (tau.lo - pl));
                const float rf = r.hi + r.lo;
                const float rinv = __frcp_rn(rf);
                const float nx = (ddx.hi + ddx.lo) * rinv, ny = (ddy.hi + ddy.lo) * rinv;
                const float nz = (D.hi + D.lo) * rinv;
                const float omn = (F.hi + F.lo) * rinv;  // 1 - n_z
                const float bx = (r2.x - nx) * rinv, by = (r2.y - ny) * rinv;
                const float bz = (omn - r2.w) * rinv;
                const float rr = rinv * rinv;
                const float ax = nx * rr, ay = ny * rr, az = nz * rr;
                const df rp = df_mul_raw(d_dw, tau);
                float Rs, Rc;
                sincosf(reduce_2pi(rp.hi, rp.lo), &Rs, &Rc);
                float R2c, R2s;
                cmul(Rc, Rs, Rc, Rs, R2c, R2s);
                float Hc = R2c, Hs = R2s;  // R^(K/2) by squaring R^2
#pragma unroll
                for (int e = K / 4; e > 1; e >>= 1) cmul(Hc, Hs, Hc, Hs, Hc, Hs);
                // setup[dd][k][step]: consecutive lanes store consecutive float4
                float4 *st = setup + (size_t)dd * kNSetupF4 * 32 + lane;
                st[0 * 32] = make_float4(tau.hi, tau.lo, Rc, Rs);
                st[1 * 32] = make_float4(ax, ax, ay, ay);
                st[2 * 32] = make_float4(az, az, bx, bx);
                st[3 * 32] = make_float4(by, by, bz, bz);
                st[4 * 32] = make_float4(R2c, R2c, R2s, R2s);
                st[5 * 32] = make_float4(-R2s, -R2s, Hc, Hc);
                st[6 * 32] = make_float4(Hs, Hs, -Hs, -Hs);
                st[7 * 32] = make_float4(fabsf(dtau), 0.f, 0.f, 0.f);
                const float am = (uint32_t)lane < mcnt ? fabsf(dtau) : 0.f;
                const float amax =
                    __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(am)));
                const float th_last = __shfl_sync(0xffffffffu, tau.hi, mcnt - 1);
                const float tl_last = __shfl_sync(0xffffffffu, tau.lo, mcnt - 1);
                __syncwarp();
                if (lane == 0) { c.tprev_h = th_last; c.tprev_l = tl_last; c.adt_max = amax; }
              }
            }
            __syncwarp();
            const bool fire_here = snap.fire_it >= (int64_t)(s0 + c0) &&
                                   snap.fire_it < (int64_t)(s0 + c0 + mcnt);
            // warp-uniform choice: the whole warp runs the tight loop or the
            // general one (lanes of a warp never diverge between the two)
            if (__all_sync(0xffffffffu, uniform && !fire_here &&
                           wabs_max * sm.sc[warp][dsub].adt_max < kPiLo)) {
              const float4 *st = setup + (size_t)dsub * kNSetupF4 * 32;
              for (uint32_t i = 0; i < mcnt; ++i) {
                float2 zr, zi;
                step_seed(st + i, i, zr, zi);
                step_fast(st + i, zr, zi);
              }
            } else {
#pragma unroll 1
              for (uint32_t i = 0; i < mcnt; ++i) {
                const float4 *st = setup + (size_t)dsub * kNSetupF4 * 32 + i;
                const float adt = st[7 * 32].x;
                const uint32_t s = s0 + c0 + i;
                const bool all_in = wabs_max * adt < kPiLo;
                const bool all_out = wabs_min * adt > kPiHi;
                if (__all_sync(0xffffffffu, uniform && (all_in || nv == 0))) {
                  // every point of the warp included: the straight-line step
                  // (the same products as the masked path with a full mask)
                  float2 zr, zi;
                  step_seed(st, i, zr, zi);
                  step_fast(st, zr, zi);
                } else if (!__all_sync(0xffffffffu, all_out || nv == 0)) {
                  // one masked path for every lane of the warp (excluded lanes
                  // carry a zero mask); skipped only when the whole warp is out
                  const float4 A = st[0], F1 = st[1 * 32], F2 = st[2 * 32], F3 = st[3 * 32],
                               R2 = st[4 * 32], X = st[5 * 32], Y = st[6 * 32];
                  uint32_t mask = (all_out || nv == 0) ? 0u : 0xffffffffu;
                  if (!all_in && !all_out && nv > 0) {
                    const ScreenConst &c = sm.sc[warp][dsub];
                    if (uniform) {
                      // included points form an index interval; only points
                      // inside the guard band need the exact FP64 test
                      const float inv_adt = __frcp_rn(adt);  // adt > 0 here
                      const float inv_dwf = (dwf != 0.f) ? __frcp_rn(dwf) : 0.f;
                      mask = omega_range_bits_r(w0f, dwf, inv_dwf, kPiLo * inv_adt, nv);
                      uint32_t unc =
                          omega_range_bits_r(w0f, dwf, inv_dwf, kPiHi * inv_adt, nv) & ~mask;
                      while (unc) {
                        const int m = __ffs(unc) - 1;
                        unc &= unc - 1u;
                        if (exact_mask_near(p, base, s, it_start, p.omega[j0 + m], c.P0, c.P1))
                          mask |= 1u << m;
                      }
                    } else {
                      mask = 0;
#pragma unroll 1
                      for (int m = 0; m < nv; ++m) {
                        const double wm = p.omega[j0 + m];
                        const float phd = (float)fabs(wm) * adt;
                        bool inc;
                        if (phd < kPiLo) inc = true;
                        else if (phd > kPiHi) inc = false;
                        else inc = exact_mask_near(p, base, s, it_start, wm, c.P0, c.P1);
                        mask |= (uint32_t)inc << m;
                      }
                    }
                  }
                  // phasors as two packed chains (uniform axis) or one reseed per
                  // point (non-uniform axis); amplitudes zeroed where masked out
                  float2 ZrA, ZiA;
                  step_seed(st, i, ZrA, ZiA);
                  float2 ZrB, ZiB;
                  rot2p(ZrA, ZiA, make_float2(X.z, X.w), make_float2(Y.x, Y.y),
                        make_float2(Y.z, Y.w), ZrB, ZiB);
#pragma unroll
                  for (int q = 0; q < HP; ++q) {
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                      float2 &zr = h ? ZrB : ZrA;
                      float2 &zi = h ? ZiB : ZiA;
                      const int m0 = h * (K / 2) + 2 * q;
                      if (!uniform) {
#pragma unroll
                        for (int e = 0; e < 2; ++e) {
                          const df wr =
                              df_from_double(p.omega[j0 + min(m0 + e, max(nv - 1, 0))] * inv2pi);
                          float ss, cc;
                          phasor_rev(wr.hi, wr.lo, A.x, A.y, ss, cc);
                          if (e == 0) { zr.x = cc; zi.x = ss; } else { zr.y = cc; zi.y = ss; }
                        }
                      }
                      // masked points: their phasors (not the six amplitudes)
                      // are zeroed, one packed product per component
                      const float2 g = make_float2(((mask >> m0) & 1u) ? 1.f : 0.f,
                                                   ((mask >> (m0 + 1)) & 1u) ? 1.f : 0.f);
                      const float2 aa[3] = {make_float2(F1.x, F1.y), make_float2(F1.z, F1.w),
                                            make_float2(F2.x, F2.y)};
                      const float2 bb[3] = {make_float2(F2.z, F2.w), make_float2(F3.x, F3.y),
                                            make_float2(F3.z, F3.w)};
                      near_accumulate(acc, h * HP + q, __fmul2_rn(zr, g), __fmul2_rn(zi, g), bb,
                                      aa);
                    }
                    if (q + 1 < HP && uniform) {
                      rot2p(ZrA, ZiA, make_float2(R2.x, R2.y), make_float2(R2.z, R2.w),
                            make_float2(X.x, X.y), ZrA, ZiA);
                      rot2p(ZrB, ZiB, make_float2(R2.x, R2.y), make_float2(R2.z, R2.w),
                            make_float2(X.x, X.y), ZrB, ZiB);
                    }
                  }
                }
                if ((int64_t)s == snap.fire_it) {
                  flush(snap.k);
                  snap.advance(it_start, it_end, snaps, p.n_snaps);
                }
              }
            }
            __syncwarp();
          }
          if ((stage_in_track + 1) % kFoldStages == 0) fold();
        } else {
          for (uint32_t i = 0; i < cnt; ++i) {
            if ((int64_t)(s0 + i) == snap.fire_it)
              snap.advance(it_start, it_end, snaps, p.n_snaps);
          }
        }
        ++stage_no;
        __syncthreads();
      }
      while (snap.fire_it != SnapState::NEVER) {
        flush(snap.k);
        snap.advance(it_start, it_end, snaps, p.n_snaps);
      }
      if (ll == 0) { sm.sc[warp][dsub].tprev_h = 0.f; sm.sc[warp][dsub].tprev_l = 0.f; }
      __syncwarp();
    }
    __syncwarp();
  }
}

size_t near_smem_bytes(int dpw) {
  return sizeof(NearSmemFixed<kNW>) + (size_t)kNW * 32 * dpw * kNSetupF4 * sizeof(float4);
}

template <int K>
int launch_near_main(const FarMixedParams &p, int grid, cudaStream_t s) {
  const size_t smem = near_smem_bytes((int)p.dpw);
  if (smem > kMaxSmemPerCta)
    return fail(SR_ERR_INVALID, "work shape needs %zu bytes of shared memory per CTA (at most %zu)",
                smem, kMaxSmemPerCta);
  cudaError_t e = cudaFuncSetAttribute(near_mixed_kernel<K, kNW>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "near_mixed smem attribute");
  near_mixed_kernel<K, kNW><<<grid, kNW * 32, smem, s>>>(p);
  return cuda_fail(cudaGetLastError(), "near_mixed kernel launch");
}

}  // namespace

// A complete configuration from K points per lane (8 or 16), L lanes per
// direction and the track subsets (0: enough subsets for about 16 work items
// per SM).
FarMixedConfig near_mixed_make(uint32_t n_omega, uint32_t n_screen, uint32_t n_tracks, int n_sm,
                               int K, int L, int n_sub) {
  FarMixedConfig c;
  c.W = kNW;
  c.ctas_per_sm = 1;
  c.K = K;
  c.stage = kStage;
  c.L = L;
  c.dpw = 32 / L;
  const uint64_t n_wtiles = (n_omega + (uint64_t)L * c.K - 1) / ((uint64_t)L * c.K);
  const uint64_t dgroups = (n_screen + c.dpw - 1) / c.dpw;
  const uint64_t groups = (dgroups * n_wtiles + c.W - 1) / c.W;
  const uint64_t capacity = (uint64_t)n_sm * c.ctas_per_sm;
  uint64_t nsub = n_sub > 0 ? (uint64_t)n_sub
                            : (16 * capacity + groups - 1) / (groups ? groups : 1);
  if (nsub > n_tracks) nsub = n_tracks;
  if (nsub < 1) nsub = 1;
  if (nsub > 64) nsub = 64;
  c.n_sub = (int)nsub;
  c.grid = (int)std::min<uint64_t>(groups * nsub, capacity);
  if (c.grid < 1) c.grid = 1;
  return c;
}

// Default work shape: 16 points per lane (the per-step reseed and setup loads
// amortised over twice the points of K = 8) wherever the omega axis fills
// most of the lanes; short axes fall back to 8.
FarMixedConfig near_mixed_choose(uint32_t n_omega, uint32_t n_screen, uint32_t n_tracks,
                                 int n_sm) {
  int K = kNKDefault;
  if ((uint32_t)(K * (32 / kNMaxDpw)) > n_omega + n_omega / 3) K = 8;
  int L = 32;
  while (L > 32 / kNMaxDpw && (uint32_t)(L / 2) * K >= n_omega) L /= 2;
  return near_mixed_make(n_omega, n_screen, n_tracks, n_sm, K, L, 0);
}

// The near-field step records for another kernel of the library (the adjoint).
void launch_near_prepass(const FarMixedParams &p, int blocks, cudaStream_t stream) {
  if (p.track_f32)
    near_prepass_kernel<float><<<blocks, 256, 0, stream>>>(p);
  else
    near_prepass_kernel<double><<<blocks, 256, 0, stream>>>(p);
}

size_t near_mixed_workspace(int64_t total_steps, uint64_t n_points, int n_out, uint32_t n_snaps,
                            const FarMixedConfig &cfg) {
  size_t b = 256;
  b += ((size_t)total_steps * kRecBytes + 255) / 256 * 256;
  b += ((size_t)cfg.n_sub * n_out * n_snaps * n_points * 8 + 255) / 256 * 256;
  b += (size_t)cfg.grid * cfg.W * cfg.K * kNOuter * 32 * sizeof(float);
  return b;
}

int launch_near_mixed(FarMixedParams p, const FarMixedConfig &cfg, void *ws, size_t ws_bytes,
                      cudaStream_t stream) {
  const uint64_t P = (uint64_t)p.n_omega * p.n_theta * p.n_phi;
  if (P == 0 || p.n_tracks == 0 || p.n_snaps == 0) return SR_OK;
  const size_t need = near_mixed_workspace(p.total_steps, P, p.n_out, p.n_snaps, cfg);
  if (ws == nullptr || ws_bytes < need)
    return fail(SR_ERR_WORKSPACE, "workspace of %zu bytes needed, %zu given", need, ws_bytes);
  if (((uintptr_t)ws & 255u) != 0) return fail(SR_ERR_WORKSPACE, "workspace not 256-byte aligned");
  unsigned char *w = (unsigned char *)ws;
  size_t off = 256;
  p.status = (int *)w;
  p.queue = (unsigned int *)(w + 128);  // in the zeroed 256-byte status block
  p.records = (float4 *)(w + off);
  off += ((size_t)p.total_steps * kRecBytes + 255) / 256 * 256;
  p.partial = (double *)(w + off);
  off += ((size_t)cfg.n_sub * p.n_out * p.n_snaps * P * 8 + 255) / 256 * 256;
  p.outer = (float *)(w + off);
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
  int dev = 0, n_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  if (p.total_steps > 0) {
    const int blk = 256;
    int64_t nb = (p.total_steps + blk - 1) / blk;
    if (nb > 8 * n_sm * 16) nb = 8 * n_sm * 16;
    if (p.track_f32)
      near_prepass_kernel<float><<<(int)nb, blk, 0, stream>>>(p);
    else
      near_prepass_kernel<double><<<(int)nb, blk, 0, stream>>>(p);
    int rc = cuda_fail(cudaGetLastError(), "near prepass launch");
    if (rc) return rc;
  }
  if (cfg.K != 8 && cfg.K != 16)
    return fail(SR_ERR_INVALID, "near field: points per lane %d (8 or 16)", cfg.K);
  void *tok = nullptr;
  timing_record(stream, true, &tok);
  int rc = (cfg.K == 16) ? launch_near_main<16>(p, cfg.grid, stream)
                         : launch_near_main<8>(p, cfg.grid, stream);
  timing_record(stream, false, &tok);
  if (rc) return rc;
  const uint64_t total = (uint64_t)p.n_out * p.n_snaps * P;
  uint64_t nb = (total + 255) / 256;
  if (nb > (uint64_t)n_sm * 64) nb = (uint64_t)n_sm * 64;
  mixed_reduce_kernel<<<(unsigned)nb, 256, 0, stream>>>(p);
  return cuda_fail(cudaGetLastError(), "near reduce launch");
}

}  // namespace sr
