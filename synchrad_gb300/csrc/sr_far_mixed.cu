// Mixed-precision far-field radiation integral for GB300 (sm_103a).
//
// Computes, per spectral point (omega, n) and track, the reference's sum
// (synchrad/kernel_farfield.cl:59-107)
//     A = sum_s amp_s exp(i omega tau_s),   tau_s = t_s - n.x_s,
//     amp = c1 (n - bbar) - c2 a,  c2 = 1/(1 - n.bbar),  c1 = (a.n) c2^2,
// over the steps whose phase advance passes |dphase| < pi, and accumulates
// w dt^2 |A|^2 (or the comp's components) over tracks.
//
// Arithmetic (the "mixed" precision):
//  * amp is transverse (n.amp = 0 exactly), so A is carried as its two
//    components on theta-hat and phi-hat; every comp is a projection of those
//    two complex sums (the radial part the FP64 reference accumulates is
//    rounding noise).
//  * tau is formed in double-float from per-step records prepared in FP64
//    (q = t - z, x, y, z) and per-direction constants (1 - cos(theta),
//    n_x, n_y): tau = q + (1 - cos theta) z - n_x x - n_y y, free of the
//    cancellation of t - n.x.
//  * exp(i omega_j tau) along a lane's K consecutive omega points is a
//    rotation recurrence z_{j+1} = z_j R, R = exp(i domega tau), run as two
//    packed chains (FFMA2/FMUL2 on point pairs) from an exact double-float
//    reseed of the lane's first point at every step;
//  * the |dphase| < pi mask is decided per step from |omega| |dtau| with a
//    guard band; inside the band the reference's FP64 expression is evaluated
//    bit for bit from the original track data.
//  * sums are FP32 for 2048 steps at a time and then folded into compensated
//    (Knuth TwoSum) FP32 pairs kept in an L2-resident workspace; per-track
//    results are formed and accumulated in FP64.
//
// Work decomposition: a warp owns 32/L directions and, for each, an omega
// tile of L*K points (lane: K consecutive points); a CTA of W warps owns W
// consecutive warp tasks and loops over a contiguous subset of the tracks.
// Track records are streamed through shared memory by 1-D bulk TMA copies
// (cp.async.bulk + mbarrier, double buffered) and reused by every warp; the
// per-(direction, step) setup is computed once per warp and broadcast through
// shared memory.  Each (task group, track subset) item writes its own partial
// spectrum; a final kernel adds the subsets in fixed order, so results are
// deterministic.
#include <algorithm>
#include <cmath>

#include "sr_common.cuh"
#include "sr_internal.h"
#include "sr_mixed_common.cuh"

namespace sr {
namespace {

// ------------------------------------------------------------------------
// Pre-pass: per-step records in FP64, stored as floats / double-floats.
//   r0 = (q.hi, q.lo, x.hi, x.lo)   q = t - z, t = (itStart + s) dt
//   r1 = (y.hi, y.lo, z.hi, z.lo)
//   r2 = (bbar_x, bbar_y, bbar_z, 1 - bbar_z)
//   r3 = (a_x, a_y, a_z, 0)
//   r4 = 0 (padding: an 80-byte record stride spreads per-lane reads over the banks)
// with beta = u / sqrt(1 + u.u) at s and s+1, a = (beta_{s+1} - beta_s)/dt,
// bbar their mean (synchrad/kernel_farfield.cl:74-83), and 1 - beta_z formed
// as (1 + ux^2 + uy^2) / (gamma (gamma + uz)) to avoid cancellation.
// ------------------------------------------------------------------------
template <typename TT>
__global__ void far_prepass_kernel(FarMixedParams p) {
  const TT *X = (const TT *)p.x, *Y = (const TT *)p.y, *Z = (const TT *)p.z;
  const TT *UX = (const TT *)p.ux, *UY = (const TT *)p.uy, *UZ = (const TT *)p.uz;
  const double dtInv = 1.0 / p.dt;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.total_steps;
       g += (int64_t)gridDim.x * blockDim.x) {
    // track of step g: last t with offsets[t] <= g
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
    const double q = time - z;
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
    const df dq = df_from_double(q), dx = df_from_double(x), dy = df_from_double(y),
             dz = df_from_double(z);
    rec[0] = make_float4(dq.hi, dq.lo, dx.hi, dx.lo);
    rec[1] = make_float4(dy.hi, dy.lo, dz.hi, dz.lo);
    rec[2] = make_float4((float)(0.5 * (b1[0] + b0[0])), (float)(0.5 * (b1[1] + b0[1])),
                         (float)(0.5 * (b1[2] + b0[2])), (float)(0.5 * (omb[0] + omb[1])));
    rec[3] = make_float4((float)((b1[0] - b0[0]) * dtInv), (float)((b1[1] - b0[1]) * dtInv),
                         (float)((b1[2] - b0[2]) * dtInv), 0.f);
    rec[4] = make_float4(0.f, 0.f, 0.f, 0.f);  // padding
  }
}


// Per-direction constants, written once per work item.
struct DirConst {
  double sT, cT, sPh, cPh, n0, n1;  // n = (n0, n1, cT) rounded as the reference does
  float dc_h, dc_l, dsx_h, dsx_l, dsy_h, dsy_l;  // 1 - cos(theta), n0, n1 as double-floats
  float f_c, f_sx, f_sy, f_cz;                   // the same in FP32
  float thx, thy, thz, phx, phy;                 // theta-hat, phi-hat
  float tprev_h, tprev_l;                        // tau of the step before the current chunk
  float adt_max;                                 // largest |dtau| of the current chunk
};

constexpr int kMaxDpw = 4;  // directions per warp (omega tiles narrower than 32 lanes)
// float4 per direction in a warp's setup block: 6 values x 32 steps, plus one
// so that the blocks of two directions read by the same 16-lane half-warp
// (4 directions per warp) start in different 16-byte bank groups
constexpr int kSetupStride = 6 * 32 + 1;

// Direction of the warp slot v = (direction group) * dpw + (direction in the
// warp).  A group holds dpw neighbouring theta at one phi (their masks agree
// on most steps, so the warp takes the masked path on fewer of them), and
// the groups run phi first: the W groups of a CTA share their theta range,
// on which the share of masked steps mostly depends, and wait less for each
// other at the stage barriers.  Directions are numbered theta first
// (theta + n_theta * phi); when dpw does not divide n_theta the slots keep
// that order.
__device__ __forceinline__ uint32_t dir_of_slot(uint32_t v, uint32_t dpw, uint32_t nT,
                                                uint32_t nP) {
  if (nT % dpw != 0u) return v;
  const uint32_t g = v / dpw;
  if (g >= (nT / dpw) * nP) return v;
  return (g / nP) * dpw + v % dpw + nT * (g % nP);
}

template <int W>
struct SmemFixed {
  uint64_t bar[2];
  uint32_t next_item;   // broadcast of the work item taken from the queue
  uint32_t pad32_;
  uint64_t pad_[1];
  float2 gate[4];       // gate[b] = (b & 1, b >> 1): a point pair's mask bits as factors
  DirConst dc[W][kMaxDpw];
  // followed by float4 setup[W][dpw][kSetupStride] ([6][32] used), then the two stage buffers of
  // p.stage_steps step records each
};

// Kernel of the mixed-precision far field.  K points per lane (two packed
// rotation chains of K/2), L lanes per direction, 32/L directions per warp.
template <int K, int W>
__global__ void __launch_bounds__(W * 32, 1) far_mixed_kernel(FarMixedParams p) {
  static_assert(K % 4 == 0 && K >= 4 && K <= 32, "K");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  SmemFixed<W> &sm = *reinterpret_cast<SmemFixed<W> *>(smem_raw);
  const int dpw = (int)p.dpw, L = 32 / dpw;
  float4 *setup_all = reinterpret_cast<float4 *>(smem_raw + sizeof(SmemFixed<W>));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int dsub = lane / L, ll = lane % L;
  float4 *setup = setup_all + (size_t)warp * dpw * kSetupStride;
  const uint32_t S = p.stage_steps;  // steps per TMA stage
  float4 *stage_buf[2];
  stage_buf[0] = setup_all + (size_t)W * dpw * kSetupStride;
  stage_buf[1] = stage_buf[0] + (size_t)S * kRecF4;
  constexpr int KP = K / 2, HP = KP / 2;

  if (threadIdx.x == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    fence_mbar_init();
  }
  if (threadIdx.x < 4)
    sm.gate[threadIdx.x] = make_float2((float)(threadIdx.x & 1u), (float)(threadIdx.x >> 1));
  __syncthreads();

  const uint32_t nO = p.n_omega, nT = p.n_theta;
  const uint32_t n_dirs = nT * p.n_phi;
  const uint64_t P = (uint64_t)nO * n_dirs;
  const uint32_t n_groups_dir = (n_dirs + dpw - 1) / dpw;  // direction groups
  const uint32_t n_wt = n_groups_dir * p.n_wtiles;         // warp tasks
  const double dw_glob = (nO > 1) ? (p.omega[nO - 1] - p.omega[0]) / (double)(nO - 1) : 0.0;
  const df d_dw = df_from_double(dw_glob);
  const double inv2pi = 0.15915494309189533577;
  float *outer = p.outer + ((size_t)blockIdx.x * W + warp) * K * 8 * 32;
  uint32_t stage_no = 0;  // running stage counter (mbarrier phase bookkeeping)
  // A uniform omega axis (omega_j = omega_0 + j d_omega to 1e-12): the points of
  // a (direction, step) that pass the mask form one index interval, found once
  // per (direction, step) in the setup and shared by the lanes.
  bool axis_ok = nO < 65535u;
  for (uint32_t j = threadIdx.x; j < nO && axis_ok; j += blockDim.x) {
    const double wj = p.omega[j];
    if (fabs(wj - (p.omega[0] + (double)j * dw_glob)) > 1e-12 * fabs(wj) + 1e-300) axis_ok = false;
  }
  const bool iv = __syncthreads_and(axis_ok) != 0;
  const float w0g = nO > 0 ? (float)p.omega[0] : 0.f;
  const float dwg = (float)dw_glob, inv_dwg = (dwg != 0.f) ? 1.0f / dwg : 0.f;

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
    const uint32_t dir_raw = dir_of_slot(dgrp * dpw + dsub, dpw, nT, p.n_phi);
    const bool active = active_w && dir_raw < n_dirs;
    const uint32_t dir = active ? dir_raw : 0u;
    const int j0 = (int)(tile * (uint32_t)(L * K)) + ll * K;
    const int nv = active ? max(0, min(K, (int)nO - j0)) : 0;

    if (ll == 0) {
      const uint32_t iT = dir % nT, iP = dir / nT;
      DirConst &d = sm.dc[warp][dsub];
      d.sT = p.sin_theta[iT];
      d.cT = p.cos_theta[iT];
      d.sPh = p.sin_phi[iP];
      d.cPh = p.cos_phi[iP];
      d.n0 = d.sT * d.cPh;
      d.n1 = d.sT * d.sPh;
      const df c = df_from_double(1.0 - d.cT), sx = df_from_double(d.n0),
               sy = df_from_double(d.n1);
      d.dc_h = c.hi; d.dc_l = c.lo; d.dsx_h = sx.hi; d.dsx_l = sx.lo;
      d.dsy_h = sy.hi; d.dsy_l = sy.lo;
      d.f_c = (float)(1.0 - d.cT); d.f_sx = (float)d.n0; d.f_sy = (float)d.n1;
      d.f_cz = (float)d.cT;
      d.thx = (float)(d.cT * d.cPh); d.thy = (float)(d.cT * d.sPh); d.thz = (float)(-d.sT);
      d.phx = (float)(-d.sPh); d.phy = (float)d.cPh;
    }

    // Lane omega constants (revolutions) and uniformity of its chunk.
    const double w0d = nv > 0 ? p.omega[j0] : 0.0;
    const df d_w0 = df_from_double(w0d * inv2pi);
    const float w0f = (float)w0d, dwf = (float)dw_glob;
    const float inv_dwf = (dwf != 0.f) ? 1.0f / dwf : 0.f;
    bool uniform = true;
    float wabs_min = 3.0e38f, wabs_max = 0.f;
    for (int m = 0; m < nv; ++m) {
      const double wm = p.omega[j0 + m];
      const double pred = w0d + (double)m * dw_glob;
      if (fabs(wm - pred) > 1e-12 * fabs(wm) + 1e-300) uniform = false;
      const float a = (float)fabs(wm);
      wabs_min = fminf(wabs_min, a);
      wabs_max = fmaxf(wabs_max, a);
    }
    if (nv == 0) { wabs_min = 0.f; wabs_max = 0.f; }
    __syncwarp();

    uint32_t t0, t1;
    subset_tracks(p, sub, t0, t1);

    // First stage of this item.
    uint32_t cur_t = t0;
    while (cur_t < t1 && track_body(p, cur_t) == 0) ++cur_t;
    if (threadIdx.x == 0 && cur_t < t1) {
      const uint32_t cnt = min(S, track_body(p, cur_t));
      const int b = stage_no & 1;
      fence_proxy_async();
      mbar_arrive_expect_tx(&sm.bar[b], cnt * kRecBytes);
      bulk_g2s(stage_buf[b], p.records + (p.offsets[cur_t]) * kRecF4, cnt * kRecBytes,
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

      float2 aTr[KP], aTi[KP], aPr[KP], aPi[KP];
#pragma unroll
      for (int q = 0; q < KP; ++q) aTr[q] = aTi[q] = aPr[q] = aPi[q] = make_float2(0.f, 0.f);
      bool outer_live = false;  // outer compensated sums hold this track's data

      // Folds the FP32 sums into the compensated pairs in the workspace.
      auto fold = [&]() {
        if (!active) return;
#pragma unroll
        for (int m = 0; m < K; ++m) {
          const int q = m >> 1;
          const float v[4] = {(m & 1) ? aTr[q].y : aTr[q].x, (m & 1) ? aTi[q].y : aTi[q].x,
                              (m & 1) ? aPr[q].y : aPr[q].x, (m & 1) ? aPi[q].y : aPi[q].x};
          float *o = outer + (size_t)m * 8 * 32 + lane;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            if (outer_live) {
              const df e = two_sum(o[c * 32], v[c]);
              o[c * 32] = e.hi;
              o[(c + 4) * 32] += e.lo;
            } else {
              o[c * 32] = v[c];
              o[(c + 4) * 32] = 0.f;
            }
          }
        }
        outer_live = true;
#pragma unroll
        for (int q = 0; q < KP; ++q) aTr[q] = aTi[q] = aPr[q] = aPi[q] = make_float2(0.f, 0.f);
      };

      // Snapshot write: A = the compensated sums, per comp, in FP64.
      auto flush = [&](uint32_t ksnap) {
        fold();
        if (!active) return;
        const DirConst &d = sm.dc[warp][dsub];
        const double wpdt2 = wp * p.dt * p.dt;
        const double wpdt = sqrt(wp) * p.dt;
        const double thxd = d.cT * d.cPh, thyd = d.cT * d.sPh, thzd = -d.sT;
        const double phxd = -d.sPh, phyd = d.cPh;
        double *part = p.partial + ((uint64_t)sub * p.n_out * p.n_snaps) * P;
#pragma unroll 1
        for (int m = 0; m < nv; ++m) {
          const float *o = outer + (size_t)m * 8 * 32 + lane;
          const double Ar = (double)o[0 * 32] + (double)o[4 * 32];
          const double Ai = (double)o[1 * 32] + (double)o[5 * 32];
          const double Br = (double)o[2 * 32] + (double)o[6 * 32];
          const double Bi = (double)o[3 * 32] + (double)o[7 * 32];
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
      };

      uint32_t stage_in_track = 0;
      for (uint32_t s0 = 0; s0 < n_body; s0 += S, ++stage_in_track) {
        const uint32_t cnt = min(S, n_body - s0);
        const int b = stage_no & 1;
        // Issue the next stage (this track or the next non-empty one of the item).
        if (threadIdx.x == 0) {
          uint32_t nt = t, ns0 = s0 + S;
          if (ns0 >= n_body) {
            nt = t + 1;
            ns0 = 0;
            while (nt < t1 && track_body(p, nt) == 0) ++nt;
          }
          if (nt < t1) {
            const uint32_t ncnt = min(S, track_body(p, nt) - ns0);
            const int nbuf = (stage_no + 1) & 1;
            fence_proxy_async();
            mbar_arrive_expect_tx(&sm.bar[nbuf], ncnt * kRecBytes);
            bulk_g2s(stage_buf[nbuf], p.records + (p.offsets[nt] + ns0) * kRecF4, ncnt * kRecBytes,
                     &sm.bar[nbuf]);
          }
        }
        const bool ok = mbar_wait_bounded(&sm.bar[b], (stage_no >> 1) & 1, kWaitLimitNs);
        if (__syncthreads_or(!ok)) {
          if (threadIdx.x == 0) {
            atomicExch(p.status, STATUS_WAIT_TIMEOUT);
            // the copy issued above for the next stage may still be in flight
            mbar_wait_bounded(&sm.bar[(stage_no + 1) & 1], ((stage_no + 1) >> 1) & 1,
                              kWaitLimitNs);
          }
          __syncthreads();
          return;
        }
        const float4 *stg = stage_buf[b];

        if (active_w) {
          for (uint32_t c0 = 0; c0 < cnt; c0 += 32) {
            const uint32_t mcnt = min(32u, cnt - c0);
            // Classes of the chunk's steps on a uniform axis, one bit per step:
            // every point of the warp's omega tile included (for all of its
            // directions), or none possibly included.
            uint32_t fast_bits = 0u, out_bits = 0u;
            // ---- per-step setup: lane l -> step s0 + c0 + l, every direction ----
            {
              const uint32_t l = (uint32_t)lane < mcnt ? (uint32_t)lane : mcnt - 1;
              const int tlo = (int)(tile * (uint32_t)(L * K));
              const int thi = min(tlo + L * K, (int)nO) - 1;
              bool in_all = true, out_all = true;
              const float4 r0 = stg[(c0 + l) * kRecF4 + 0];
              const float4 r1 = stg[(c0 + l) * kRecF4 + 1];
              const float4 r2 = stg[(c0 + l) * kRecF4 + 2];
              const float4 r3 = stg[(c0 + l) * kRecF4 + 3];
              const bool first = (s0 + c0 + l) == 0;
              for (int dd = 0; dd < dpw; ++dd) {
                DirConst &d = sm.dc[warp][dd];
                // tau = q + (1 - cos th) z - n_x x - n_y y   (double-float)
                df tau = df{r0.x, r0.y};
                tau = df_add(tau, df_mul(df{d.dc_h, d.dc_l}, df{r1.z, r1.w}));
                const df nx = df_mul(df{d.dsx_h, d.dsx_l}, df{r0.z, r0.w});
                const df ny = df_mul(df{d.dsy_h, d.dsy_l}, df{r1.x, r1.y});
                tau = df_add(tau, df{-nx.hi, -nx.lo});
                tau = df_add(tau, df{-ny.hi, -ny.lo});
                // previous step's tau (lane 0: carried; the track's first step
                // compares with a zero phase, synchrad/kernel_farfield.cl:49)
                float ph = __shfl_up_sync(0xffffffffu, tau.hi, 1);
                float pl = __shfl_up_sync(0xffffffffu, tau.lo, 1);
                if (lane == 0) { ph = d.tprev_h; pl = d.tprev_l; }
                const float dtau = first ? (tau.hi + tau.lo) : ((tau.hi - ph) + (tau.lo - pl));
                // amplitude on theta-hat / phi-hat
                const float D = r2.w + d.f_c * r2.z - d.f_sx * r2.x - d.f_sy * r2.y;
                const float c2 = __frcp_rn(D);
                const float an = d.f_sx * r3.x + d.f_sy * r3.y + d.f_cz * r3.z;
                const float c1 = an * c2 * c2;
                const float tb = d.thx * r2.x + d.thy * r2.y + d.thz * r2.z;
                const float ta = d.thx * r3.x + d.thy * r3.y + d.thz * r3.z;
                const float pb = d.phx * r2.x + d.phy * r2.y;
                const float pa = d.phx * r3.x + d.phy * r3.y;
                const float amp_t = -(c1 * tb + c2 * ta);
                const float amp_p = -(c1 * pb + c2 * pa);
                // rotation between neighbouring omega points, its square, and
                // its power K/2 (start of the second chain)
                const df rp = df_mul_raw(d_dw, tau);
                const float rr = reduce_2pi(rp.hi, rp.lo);
                float Rs, Rc;
                sincosf(rr, &Rs, &Rc);
                float R2c, R2s;
                cmul(Rc, Rs, Rc, Rs, R2c, R2s);
                // H = R^(K/2) = (R^2)^(K/4) by binary powering from R^2 (the
                // exponent is a compile-time constant: K = 32 takes three
                // squarings, K = 24 two squarings and one product)
                float Hc = R2c, Hs = R2s, Pc = R2c, Ps = R2s;
                bool h_set = false;
#pragma unroll
                for (int e = K / 4; e > 0; e >>= 1) {
                  if (e & 1) {
                    if (h_set) cmul(Hc, Hs, Pc, Ps, Hc, Hs);
                    else { Hc = Pc; Hs = Ps; h_set = true; }
                  }
                  if (e > 1) cmul(Pc, Ps, Pc, Ps, Pc, Ps);
                }
                // setup[dd][k][step]: consecutive lanes store consecutive float4
                float4 *st = setup + (size_t)dd * kSetupStride + lane;
                st[0 * 32] = make_float4(tau.hi, tau.lo, Rc, Rs);
                st[1 * 32] = make_float4(amp_t, amp_t, amp_p, amp_p);
                st[2 * 32] = make_float4(R2c, R2c, R2s, R2s);
                st[3 * 32] = make_float4(-R2s, -R2s, Hc, Hc);
                st[4 * 32] = make_float4(Hs, Hs, -Hs, -Hs);
                // the mask's index intervals over the whole omega axis: points
                // certainly included (below kPiLo) and possibly included (kPiHi)
                int jfc = 1, jlc = 0, jfu = 1, jlu = 0;
                if (iv) {
                  const float inv_adt = __frcp_rn(fabsf(dtau));
                  omega_interval(w0g, dwg, inv_dwg, kPiLo * inv_adt, (int)nO, jfc, jlc);
                  omega_interval(w0g, dwg, inv_dwg, kPiHi * inv_adt, (int)nO, jfu, jlu);
                  if (dgrp * dpw + dd < n_dirs) {  // slots map onto [0, n_dirs) one to one
                    in_all = in_all && jfc <= tlo && jlc >= thi;
                    out_all = out_all && (jlu < tlo || jfu > thi);
                  }
                }
                st[5 * 32] = make_float4(fabsf(dtau), __int_as_float(jfc), __int_as_float(jlc),
                                         __uint_as_float((uint32_t)jfu | ((uint32_t)(jlu + 1) << 16)));
                // largest |dtau| of the chunk: decides the chunk's fast loop
                const float am = (uint32_t)lane < mcnt ? fabsf(dtau) : 0.f;
                const float amax = __uint_as_float(__reduce_max_sync(0xffffffffu, __float_as_uint(am)));
                const float th_last = __shfl_sync(0xffffffffu, tau.hi, mcnt - 1);
                const float tl_last = __shfl_sync(0xffffffffu, tau.lo, mcnt - 1);
                __syncwarp();
                if (lane == 0) { d.tprev_h = th_last; d.tprev_l = tl_last; d.adt_max = amax; }
              }
              fast_bits = __ballot_sync(0xffffffffu, iv && (uint32_t)lane < mcnt && in_all);
              out_bits = __ballot_sync(0xffffffffu, iv && (uint32_t)lane < mcnt && out_all && !in_all);
            }
            __syncwarp();
            // ---- the points: K per lane as two packed rotation chains ----
            // A chunk whose steps are all included for this lane's omega range,
            // with a uniform axis and no snapshot write, runs the tight loop.
            const bool fire_here = snap.fire_it >= (int64_t)(s0 + c0) &&
                                   snap.fire_it < (int64_t)(s0 + c0 + mcnt);
            // The first pair's phasors of one step: the reseed e^{i omega_0 tau}
            // (the lane's own sin/cos, interleaved with the other steps' sums)
            // and its product with R = e^{i d_omega tau}.
            auto step_seed = [&](const float4 *st, uint32_t, float2 &ZrA, float2 &ZiA) {
              const float4 A = st[0];
              float zs, zc;
              phasor_rev(d_w0.hi, d_w0.lo, A.x, A.y, zs, zc);
              ZrA = make_float2(zc, zc * A.z - zs * A.w);
              ZiA = make_float2(zs, zc * A.w + zs * A.z);
            };
            // One fully included step on a uniform axis: two packed chains.
            auto step_fast = [&](const float4 *st, float2 ZrA, float2 ZiA) {
              const float4 AT = st[1 * 32], R2 = st[2 * 32], X = st[3 * 32], Y = st[4 * 32];
              const float2 at = make_float2(AT.x, AT.y), ap = make_float2(AT.z, AT.w);
              const float2 r2c = make_float2(R2.x, R2.y), r2s = make_float2(R2.z, R2.w);
              const float2 nr2s = make_float2(X.x, X.y), hc = make_float2(X.z, X.w);
              const float2 hs = make_float2(Y.x, Y.y), nhs = make_float2(Y.z, Y.w);
              float2 ZrB, ZiB;
              rot2p(ZrA, ZiA, hc, hs, nhs, ZrB, ZiB);
#pragma unroll
              for (int q = 0; q < HP; ++q) {
                aTr[q] = __ffma2_rn(ZrA, at, aTr[q]);
                aTi[q] = __ffma2_rn(ZiA, at, aTi[q]);
                aPr[q] = __ffma2_rn(ZrA, ap, aPr[q]);
                aPi[q] = __ffma2_rn(ZiA, ap, aPi[q]);
                aTr[HP + q] = __ffma2_rn(ZrB, at, aTr[HP + q]);
                aTi[HP + q] = __ffma2_rn(ZiB, at, aTi[HP + q]);
                aPr[HP + q] = __ffma2_rn(ZrB, ap, aPr[HP + q]);
                aPi[HP + q] = __ffma2_rn(ZiB, ap, aPi[HP + q]);
                if (q + 1 < HP) {
                  rot2p(ZrA, ZiA, r2c, r2s, nr2s, ZrA, ZiA);
                  rot2p(ZrB, ZiB, r2c, r2s, nr2s, ZrB, ZiB);
                }
              }
            };
            // warp-uniform choices (lanes of a warp never diverge between paths)
            if (__all_sync(0xffffffffu, uniform && !fire_here &&
                           wabs_max * sm.dc[warp][dsub].adt_max < kPiLo)) {
              // every step of the chunk included for every point: the tight loop
              const float4 *st = setup + (size_t)dsub * kSetupStride;
              for (uint32_t i = 0; i < mcnt; ++i) {
                float2 zr, zi;
                step_seed(st + i, i, zr, zi);
                step_fast(st + i, zr, zi);
              }
            } else if (iv && __all_sync(0xffffffffu, uniform)) {
              // Uniform axis: each step's class comes from the setup's ballots
              // (no per-step vote). Runs of included steps go through the
              // straight-line loop; a step that is neither fully included nor
              // fully excluded for the warp takes the masked step (its points'
              // phasors times 0/1 factors: the included points form the index
              // interval of the setup, widened by the exact FP64 test of the
              // points inside the guard band). In a chunk with a snapshot write
              // every step takes the per-step path, which checks for the write
              // after each step (an included step there is a masked step with a
              // full mask).
              const float4 *stb = setup + (size_t)dsub * kSetupStride;
              const uint32_t fb = fire_here ? 0u : fast_bits;
              uint32_t i = 0;
#pragma unroll 1
              while (i < mcnt) {
                const uint32_t run = min((uint32_t)__ffs(~(fb >> i)) - 1u, mcnt - i);
                for (const uint32_t e = i + run; i < e; ++i) {
                  float2 zr, zi;
                  step_seed(stb + i, i, zr, zi);
                  step_fast(stb + i, zr, zi);
                }
                if (i >= mcnt) break;
                const float4 *st = stb + i;
                const uint32_t s = s0 + c0 + i;
                if (!((out_bits >> i) & 1u)) {
                  const float4 M = st[5 * 32];
                  const int jfc = __float_as_int(M.y), jlc = __float_as_int(M.z);
                  const uint32_t pu = __float_as_uint(M.w);
                  const int jfu = (int)(pu & 0xffffu), jlu = (int)(pu >> 16) - 1;
                  uint32_t mask = range_bits(jfc, jlc, j0, nv);
                  uint32_t unc = range_bits(jfu, jlu, j0, nv) & ~mask;
                  if (unc) {
                    const DirConst &d = sm.dc[warp][dsub];
                    do {
                      const int m = __ffs(unc) - 1;
                      unc &= unc - 1u;
                      if (exact_mask(p, base, s, it_start, p.omega[j0 + m], d.n0, d.n1, d.cT))
                        mask |= 1u << m;
                    } while (unc);
                  }
                  float2 ZrA, ZiA;
                  step_seed(st, i, ZrA, ZiA);
                  const float4 AT = st[1 * 32], R2 = st[2 * 32], X = st[3 * 32], Y = st[4 * 32];
                  const float2 at = make_float2(AT.x, AT.y), ap = make_float2(AT.z, AT.w);
                  const float2 r2c = make_float2(R2.x, R2.y), r2s = make_float2(R2.z, R2.w);
                  const float2 nr2s = make_float2(X.x, X.y);
                  float2 ZrB, ZiB;
                  rot2p(ZrA, ZiA, make_float2(X.z, X.w), make_float2(Y.x, Y.y),
                        make_float2(Y.z, Y.w), ZrB, ZiB);
#pragma unroll
                  for (int q = 0; q < HP; ++q) {
                    // the pair's two mask bits pick its 0/1 factors from a
                    // 4-entry table (one shared load, no per-point selects)
                    const float2 gA = sm.gate[(mask >> (2 * q)) & 3u];
                    const float2 gB = sm.gate[(mask >> (K / 2 + 2 * q)) & 3u];
                    const float2 mrA = __fmul2_rn(ZrA, gA), miA = __fmul2_rn(ZiA, gA);
                    const float2 mrB = __fmul2_rn(ZrB, gB), miB = __fmul2_rn(ZiB, gB);
                    aTr[q] = __ffma2_rn(mrA, at, aTr[q]);
                    aTi[q] = __ffma2_rn(miA, at, aTi[q]);
                    aPr[q] = __ffma2_rn(mrA, ap, aPr[q]);
                    aPi[q] = __ffma2_rn(miA, ap, aPi[q]);
                    aTr[HP + q] = __ffma2_rn(mrB, at, aTr[HP + q]);
                    aTi[HP + q] = __ffma2_rn(miB, at, aTi[HP + q]);
                    aPr[HP + q] = __ffma2_rn(mrB, ap, aPr[HP + q]);
                    aPi[HP + q] = __ffma2_rn(miB, ap, aPi[HP + q]);
                    if (q + 1 < HP) {
                      rot2p(ZrA, ZiA, r2c, r2s, nr2s, ZrA, ZiA);
                      rot2p(ZrB, ZiB, r2c, r2s, nr2s, ZrB, ZiB);
                    }
                  }
                }
                if ((int64_t)s == snap.fire_it) {  // uniform over the CTA
                  flush(snap.k);
                  snap.advance(it_start, it_end, snaps, p.n_snaps);
                }
                ++i;
              }
            } else {
              // General loop (an omega axis that is not uniform as a whole):
              // per-step vote, per-lane index interval on uniform lanes and a
              // per-point test with one reseed per point on the others.
#pragma unroll 1
              for (uint32_t i = 0; i < mcnt; ++i) {
                const float4 *st = setup + (size_t)dsub * kSetupStride + i;
                const float adt = st[5 * 32].x;
                const uint32_t s = s0 + c0 + i;
                // a lane is all in (out) when its largest (smallest) |omega|
                // passes (fails) the rule with the guard band
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
                  const float4 A = st[0], AT = st[1 * 32], R2 = st[2 * 32], X = st[3 * 32],
                               Y = st[4 * 32];
                  uint32_t mask = (all_out || nv == 0) ? 0u : 0xffffffffu;
                  if (!all_in && !all_out && nv > 0) {
                    const DirConst &d = sm.dc[warp][dsub];
                    if (uniform) {
                      // included points form an index interval; only points
                      // inside the guard band need the exact FP64 test
                      const float inv_adt = __frcp_rn(adt);  // adt > 0 here
                      mask = omega_range_bits_r(w0f, dwf, inv_dwf, kPiLo * inv_adt, nv);
                      uint32_t unc =
                          omega_range_bits_r(w0f, dwf, inv_dwf, kPiHi * inv_adt, nv) & ~mask;
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
                  // phasors as two packed chains from the reseeded first point
                  // (uniform axis) or one reseed per point (non-uniform axis);
                  // amplitudes zeroed per point where the step is masked out
                  float2 ZrA, ZiA;
                  step_seed(st, i, ZrA, ZiA);
                  float2 ZrB, ZiB;
                  rot2p(ZrA, ZiA, make_float2(X.z, X.w), make_float2(Y.x, Y.y),
                        make_float2(Y.z, Y.w), ZrB, ZiB);
#pragma unroll
                  for (int q = 0; q < HP; ++q) {
                    if (!uniform) {
#pragma unroll
                      for (int h = 0; h < 2; ++h) {
#pragma unroll
                        for (int e = 0; e < 2; ++e) {
                          const int m = h * (K / 2) + 2 * q + e;
                          const df wr = df_from_double(p.omega[j0 + min(m, max(nv - 1, 0))] * inv2pi);
                          float ss, cc;
                          phasor_rev(wr.hi, wr.lo, A.x, A.y, ss, cc);
                          float2 &zr = h ? ZrB : ZrA;
                          float2 &zi = h ? ZiB : ZiA;
                          if (e == 0) { zr.x = cc; zi.x = ss; } else { zr.y = cc; zi.y = ss; }
                        }
                      }
                    }
                    // masked points: their phasors (not the amplitudes) are
                    // zeroed, one packed product per chain and component
                    const int mA = 2 * q, mB = K / 2 + 2 * q;
                    const float2 gA = make_float2(((mask >> mA) & 1u) ? 1.f : 0.f,
                                                  ((mask >> (mA + 1)) & 1u) ? 1.f : 0.f);
                    const float2 gB = make_float2(((mask >> mB) & 1u) ? 1.f : 0.f,
                                                  ((mask >> (mB + 1)) & 1u) ? 1.f : 0.f);
                    const float2 at = make_float2(AT.x, AT.y), ap = make_float2(AT.z, AT.w);
                    const float2 mrA = __fmul2_rn(ZrA, gA), miA = __fmul2_rn(ZiA, gA);
                    const float2 mrB = __fmul2_rn(ZrB, gB), miB = __fmul2_rn(ZiB, gB);
                    aTr[q] = __ffma2_rn(mrA, at, aTr[q]);
                    aTi[q] = __ffma2_rn(miA, at, aTi[q]);
                    aPr[q] = __ffma2_rn(mrA, ap, aPr[q]);
                    aPi[q] = __ffma2_rn(miA, ap, aPi[q]);
                    aTr[HP + q] = __ffma2_rn(mrB, at, aTr[HP + q]);
                    aTi[HP + q] = __ffma2_rn(miB, at, aTi[HP + q]);
                    aPr[HP + q] = __ffma2_rn(mrB, ap, aPr[HP + q]);
                    aPi[HP + q] = __ffma2_rn(miB, ap, aPi[HP + q]);
                    if (q + 1 < HP && uniform) {
                      rot2p(ZrA, ZiA, make_float2(R2.x, R2.y), make_float2(R2.z, R2.w),
                            make_float2(X.x, X.y), ZrA, ZiA);
                      rot2p(ZrB, ZiB, make_float2(R2.x, R2.y), make_float2(R2.z, R2.w),
                            make_float2(X.x, X.y), ZrB, ZiB);
                    }
                  }
                }
                if ((int64_t)s == snap.fire_it) {  // uniform over the CTA
                  flush(snap.k);
                  snap.advance(it_start, it_end, snaps, p.n_snaps);
                }
              }
            }
            __syncwarp();
          }
          // ---- fold the FP32 sums into the compensated pairs every few stages ----
          // (all warps at the same stage: a fold staggered by warp made the
          // other warps wait for it at every stage barrier)
          if ((stage_in_track + 1) % p.fold_stages == 0) fold();
        } else {
          // inactive warp: keep the snapshot state in step with the others
          for (uint32_t i = 0; i < cnt; ++i) {
            if ((int64_t)(s0 + i) == snap.fire_it)
              snap.advance(it_start, it_end, snaps, p.n_snaps);
          }
        }
        ++stage_no;
        __syncthreads();  // every warp is done with buffer b before it is refilled
      }
      // Snapshot writes due after the last body step (A no longer changes).
      while (snap.fire_it != SnapState::NEVER) {
        flush(snap.k);
        snap.advance(it_start, it_end, snaps, p.n_snaps);
      }
      // the next track starts with empty carried tau
      if (ll == 0) { sm.dc[warp][dsub].tprev_h = 0.f; sm.dc[warp][dsub].tprev_l = 0.f; }
      __syncwarp();
    }
    __syncwarp();
  }
}

constexpr int kW = 8;  // warps per CTA

size_t smem_bytes(int dpw, int stage) {
  return sizeof(SmemFixed<kW>) + (size_t)kW * dpw * kSetupStride * sizeof(float4) +
         (size_t)2 * stage * kRecF4 * sizeof(float4);
}

template <int K>
int launch_main(const FarMixedParams &p, int grid, cudaStream_t s) {
  const size_t smem = smem_bytes((int)p.dpw, (int)p.stage_steps);
  if (smem > kMaxSmemPerCta)
    return fail(SR_ERR_INVALID,
                "work shape needs %zu bytes of shared memory per CTA (at most %zu): fewer "
                "steps per stage or more lanes per direction",
                smem, kMaxSmemPerCta);
  cudaError_t e = cudaFuncSetAttribute(far_mixed_kernel<K, kW>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "far_mixed smem attribute");
  far_mixed_kernel<K, kW><<<grid, kW * 32, smem, s>>>(p);
  return cuda_fail(cudaGetLastError(), "far_mixed kernel launch");
}

int dispatch_k(int K, const FarMixedParams &p, int grid, cudaStream_t s) {
  switch (K) {
    case 8: return launch_main<8>(p, grid, s);
    case 16: return launch_main<16>(p, grid, s);
    case 24: return launch_main<24>(p, grid, s);
    case 32: return launch_main<32>(p, grid, s);
    default: return fail(SR_ERR_INVALID, "unsupported points per lane %d", K);
  }
}

}  // namespace

// Shared memory per CTA of a far-field work shape (dpw directions per warp,
// steps per stage), for the checks of sr_config_set.
size_t far_mixed_smem_bytes(int dpw, int stage) { return smem_bytes(dpw, stage); }

// The far-field step records for another kernel of the library (the adjoint).
void launch_far_prepass(const FarMixedParams &p, int blocks, cudaStream_t stream) {
  if (p.track_f32)
    far_prepass_kernel<float><<<blocks, 256, 0, stream>>>(p);
  else
    far_prepass_kernel<double><<<blocks, 256, 0, stream>>>(p);
}

// A complete configuration from its free parameters: K points per lane, L
// lanes per direction (32/L directions per warp), steps per stage and track
// subsets (0: enough subsets for about 16 work items per SM).
FarMixedConfig far_mixed_make(uint32_t n_omega, uint32_t n_dirs, uint32_t n_tracks, int n_sm,
                              int K, int L, int stage, int n_sub) {
  FarMixedConfig c;
  c.W = kW;
  c.ctas_per_sm = 1;
  c.K = K;
  c.L = L;
  c.dpw = 32 / L;
  c.stage = stage;
  const uint64_t n_wtiles = (n_omega + (uint64_t)L * K - 1) / ((uint64_t)L * K);
  const uint64_t dgroups = (n_dirs + c.dpw - 1) / c.dpw;
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

// Default work shape: the widest lane chunk (K = 32) amortises the per-step
// reseed best; narrower omega axes put several directions in one warp and
// shrink K while the lanes of a direction would idle.
FarMixedConfig far_mixed_choose(uint32_t n_omega, uint32_t n_dirs, uint32_t n_tracks,
                                int n_sm) {
  int K = 32, L = 32;
  while (L > 32 / kMaxDpw && (uint32_t)(L / 2) * 32u >= n_omega) L /= 2;
  while (K > 8 && (uint32_t)(L * (K - 8)) >= n_omega) K -= 8;
  return far_mixed_make(n_omega, n_dirs, n_tracks, n_sm, K, L, kStage, 0);
}

size_t far_mixed_workspace(int64_t total_steps, uint64_t n_points, int n_out, uint32_t n_snaps,
                           const FarMixedConfig &cfg) {
  size_t b = 256;                                                    // status word
  b += ((size_t)total_steps * kRecBytes + 255) / 256 * 256;          // step records
  b += ((size_t)cfg.n_sub * n_out * n_snaps * n_points * 8 + 255) / 256 * 256;  // partials
  b += (size_t)cfg.grid * cfg.W * cfg.K * 8 * 32 * sizeof(float);   // compensated sums
  return b;
}

int launch_far_mixed(FarMixedParams p, const FarMixedConfig &cfg, void *ws, size_t ws_bytes,
                     cudaStream_t stream) {
  const uint64_t P = (uint64_t)p.n_omega * p.n_theta * p.n_phi;
  if (P == 0 || p.n_tracks == 0 || p.n_snaps == 0) return SR_OK;
  const size_t need = far_mixed_workspace(p.total_steps, P, p.n_out, p.n_snaps, cfg);
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
  if (cfg.stage < 32 || cfg.stage > 512 || (cfg.stage & 31) != 0)
    return fail(SR_ERR_INVALID, "steps per stage %d (multiples of 32 in [32, 512])", cfg.stage);
  p.stage_steps = (uint32_t)cfg.stage;
  p.fold_stages = (uint32_t)std::max(1, 2048 / cfg.stage);  // fold about every 2048 steps

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
      far_prepass_kernel<float><<<(int)nb, blk, 0, stream>>>(p);
    else
      far_prepass_kernel<double><<<(int)nb, blk, 0, stream>>>(p);
    int rc = cuda_fail(cudaGetLastError(), "far prepass launch");
    if (rc) return rc;
  }
  void *tok = nullptr;
  timing_record(stream, true, &tok);
  int rc = dispatch_k(cfg.K, p, cfg.grid, stream);
  timing_record(stream, false, &tok);
  if (rc) return rc;
  const uint64_t total = (uint64_t)p.n_out * p.n_snaps * P;
  uint64_t nb = (total + 255) / 256;
  if (nb > (uint64_t)n_sm * 64) nb = (uint64_t)n_sm * 64;
  mixed_reduce_kernel<<<(unsigned)nb, 256, 0, stream>>>(p);
  return cuda_fail(cudaGetLastError(), "far reduce launch");
}

}  // namespace sr
