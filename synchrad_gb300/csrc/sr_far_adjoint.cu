// Adjoint of the mixed-precision far field (comp 'total', one snapshot).
//
// Forward (sr_far_mixed.cu):  S(p) = sum_t w_t dt^2 |A_t(p)|^2,
//   A_t(p) = sum_s m_s(p) amp_s(p) exp(i omega tau_s(p)),  carried on
//   theta-hat and phi-hat, amp = -(c1 (e.bbar) + c2 (e.a)) for e in {th, ph},
//   c2 = 1/(1 - n.bbar), c1 = (a.n) c2^2, tau_s = t_s - n.x_s.
// Given g(p) = dL/dS(p), with U_c = 2 g w dt^2 conj(A_c) and W_c = omega U_c:
//   dL/dw_t       = sum_p g dt^2 |A_t|^2
//   dL/damp_c,s   = E_c(d,s) = sum_omega Re(U_c z_s)
//   dL/dx_s       = sum_d n (amp_th F_th + amp_ph F_ph),  F_c = sum_omega Im(W_c z_s)
//   dL/dbbar_s, dL/da_s from amp(bbar, a), then bbar_s = (beta_s + beta_{s+1})/2,
//   a_s = (beta_{s+1} - beta_s)/dt, beta = u/gamma.
// The |dphase| < pi mask is held fixed (its decisions are the forward's).
// Phases are recomputed, not stored: the kernel streams the same step records
// as the forward and rebuilds exp(i omega tau) with the same packed rotation
// chains; E and F are reduced over the omega points of a direction with warp
// shuffles, the chain rule runs once per (direction, step), and per-CTA sums
// over directions go to per-group partials that a final kernel adds in fixed
// order.
#include <algorithm>
#include <cmath>

#include "sr_common.cuh"
#include "sr_internal.h"
#include "sr_mixed_common.cuh"

namespace sr {
namespace {

constexpr int kAK = 8;       // omega points per lane
constexpr int kAW = 8;       // warps per CTA
constexpr int kAMaxDpw = 4;  // directions per warp
constexpr int kAG = 9;       // per-step gradient components: x (3), bbar (3), a (3)

struct AdjParams {
  FarMixedParams f;            // tracks, grid, records, status, decomposition
  const double *grad_spec;     // [P] dL/dS in the device layout
  const float4 *save_A;        // [n_tracks][P] (A_th re, im, A_ph re, im)
  float4 *consts;              // [n_tracks][P][2] U/W constants
  float *gpart;                // [n_groups][total_steps][kAG]
  double *grad[6];             // x, y, z, ux, uy, uz  [total_steps]
  double *grad_w;              // [n_tracks]
};

// U/W constants per (track, point):
//   c0 = (Re U_th, -Im U_th, Re U_ph, -Im U_ph),  c1 = (Re W_th, Im W_th, Re W_ph, Im W_ph)
__global__ void adj_prep_kernel(AdjParams a) {
  const FarMixedParams &p = a.f;
  const uint64_t P = (uint64_t)p.n_omega * p.n_theta * p.n_phi;
  const uint64_t total = P * p.n_tracks;
  const double dt2 = p.dt * p.dt;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
       i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t t = i / P, g = i - t * P;
    const float4 A = a.save_A[i];
    const double G = 2.0 * a.grad_spec[g] * p.weight[t] * dt2;
    const double w = p.omega[g % p.n_omega];
    const double ur = G * A.x, ui = -G * A.y, vr = G * A.z, vi = -G * A.w;
    a.consts[2 * i] = make_float4((float)ur, (float)(-ui), (float)vr, (float)(-vi));
    a.consts[2 * i + 1] = make_float4((float)(w * ur), (float)(w * ui), (float)(w * vr),
                                      (float)(w * vi));
  }
}

// dL/dw_t = sum_p g(p) dt^2 |A_t(p)|^2, one block per track (fixed order).
__global__ void adj_weight_kernel(AdjParams a) {
  const FarMixedParams &p = a.f;
  const uint64_t P = (uint64_t)p.n_omega * p.n_theta * p.n_phi;
  const uint32_t t = blockIdx.x;
  double acc = 0.0;
  for (uint64_t g = threadIdx.x; g < P; g += blockDim.x) {
    const float4 A = a.save_A[(uint64_t)t * P + g];
    const double a2 = (double)A.x * A.x + (double)A.y * A.y + (double)A.z * A.z +
                      (double)A.w * A.w;
    acc += a.grad_spec[g] * a2;
  }
  __shared__ double red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) a.grad_w[t] = red[0] * p.dt * p.dt;
}

// Per-step gradients: sum the groups' partials (fixed order), then map
// dL/dbbar and dL/da of steps s-1 and s to dL/dbeta_s and dL/du_s.
template <typename TT>
__global__ void adj_final_kernel(AdjParams a) {
  const FarMixedParams &p = a.f;
  const TT *UX = (const TT *)p.ux, *UY = (const TT *)p.uy, *UZ = (const TT *)p.uz;
  const double dtInv = 1.0 / p.dt;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.total_steps;
       g += (int64_t)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = p.n_tracks;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (p.offsets[mid] <= g) lo = mid; else hi = mid;
    }
    const uint32_t t = lo;
    const int64_t base = p.offsets[t];
    const int64_t s = g - base;
    const int64_t n = p.offsets[t + 1] - base;
    const uint32_t it_end = p.it_end[t];
    const int64_t n_body = (n < 1 || it_end < 1) ? 0 : min((int64_t)it_end - 1, n - 1);
    double cur[kAG] = {0}, prev[kAG] = {0};
    if (s < n_body)
      for (uint32_t q = 0; q < p.n_groups; ++q)
        for (int c = 0; c < kAG; ++c)
          cur[c] += (double)a.gpart[((uint64_t)q * p.total_steps + g) * kAG + c];
    if (s >= 1 && s - 1 < n_body)
      for (uint32_t q = 0; q < p.n_groups; ++q)
        for (int c = 3; c < kAG; ++c)
          prev[c] += (double)a.gpart[((uint64_t)q * p.total_steps + g - 1) * kAG + c];
    a.grad[0][g] = cur[0];
    a.grad[1][g] = cur[1];
    a.grad[2][g] = cur[2];
    // dL/dbeta_s = (gb_s + gb_{s-1})/2 + (ga_{s-1} - ga_s)/dt
    double gb[3];
    for (int c = 0; c < 3; ++c)
      gb[c] = 0.5 * (cur[3 + c] + prev[3 + c]) + (prev[6 + c] - cur[6 + c]) * dtInv;
    const double ux = (double)UX[g], uy = (double)UY[g], uz = (double)UZ[g];
    const double gam = sqrt(1.0 + (ux * ux + uy * uy + uz * uz));
    const double ug = (ux * gb[0] + uy * gb[1] + uz * gb[2]) / (gam * gam * gam);
    a.grad[3][g] = gb[0] / gam - ux * ug;
    a.grad[4][g] = gb[1] / gam - uy * ug;
    a.grad[5][g] = gb[2] / gam - uz * ug;
  }
}

struct AdjDir {
  double n0, n1, cT;
  float dc_h, dc_l, dsx_h, dsx_l, dsy_h, dsy_l;
  float f_c, f_sx, f_sy, f_cz;
  float thx, thy, thz, phx, phy;
  float tprev_h, tprev_l, adt_max;
  float pad_[3];
};

template <int W>
struct AdjSmemFixed {
  float4 stage[2][kStage * kRecF4];
  uint64_t bar[2];
  uint64_t pad_[2];
  AdjDir dc[W][kAMaxDpw];
  float4 red[W][32][kAMaxDpw];      // per (step, direction): E_th, E_ph, F_th, F_ph
  float cta[W][kStage][kAG];        // per (warp, step) gradient contributions
  // followed by float4 setup[W][32][dpw][6]
};

template <int W>
__global__ void __launch_bounds__(W * 32, 1) adj_far_kernel(AdjParams a) {
  constexpr int K = kAK, KP = K / 2, HP = KP / 2;
  const FarMixedParams &p = a.f;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  AdjSmemFixed<W> &sm = *reinterpret_cast<AdjSmemFixed<W> *>(smem_raw);
  const int dpw = (int)p.dpw, L = 32 / dpw;
  float4 *setup_all = reinterpret_cast<float4 *>(smem_raw + sizeof(AdjSmemFixed<W>));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int dsub = lane / L, ll = lane % L;
  float4 *setup = setup_all + (size_t)warp * 32 * dpw * 6;

  if (threadIdx.x == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  const uint32_t nO = p.n_omega, nT = p.n_theta;
  const uint32_t n_dirs = nT * p.n_phi;
  const uint64_t P = (uint64_t)nO * n_dirs;
  const uint32_t n_wt = ((n_dirs + dpw - 1) / dpw) * p.n_wtiles;
  const double dw_glob = (nO > 1) ? (p.omega[nO - 1] - p.omega[0]) / (double)(nO - 1) : 0.0;
  const df d_dw = df_from_double(dw_glob);
  const double inv2pi = 0.15915494309189533577;
  uint32_t stage_no = 0;

  for (uint32_t item = blockIdx.x; item < p.n_items; item += gridDim.x) {
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
      const uint32_t iT = dir % nT, iP = dir / nT;
      AdjDir &d = sm.dc[warp][dsub];
      const double sT = p.sin_theta[iT], cT = p.cos_theta[iT];
      const double sPh = p.sin_phi[iP], cPh = p.cos_phi[iP];
      d.n0 = sT * cPh;
      d.n1 = sT * sPh;
      d.cT = cT;
      const df c = df_from_double(1.0 - cT), sx = df_from_double(d.n0), sy = df_from_double(d.n1);
      d.dc_h = c.hi; d.dc_l = c.lo; d.dsx_h = sx.hi; d.dsx_l = sx.lo;
      d.dsy_h = sy.hi; d.dsy_l = sy.lo;
      d.f_c = (float)(1.0 - cT); d.f_sx = (float)d.n0; d.f_sy = (float)d.n1; d.f_cz = (float)cT;
      d.thx = (float)(cT * cPh); d.thy = (float)(cT * sPh); d.thz = (float)(-sT);
      d.phx = (float)(-sPh); d.phy = (float)cPh;
      d.tprev_h = 0.f; d.tprev_l = 0.f;
    }
    const double w0d = nv > 0 ? p.omega[j0] : 0.0;
    const df d_w0 = df_from_double(w0d * inv2pi);
    const float w0f = (float)w0d, dwf = (float)dw_glob;
    bool uniform = true;
    float wabs_min = 3.0e38f, wabs_max = 0.f;
    for (int m = 0; m < nv; ++m) {
      const double wm = p.omega[j0 + m];
      if (fabs(wm - (w0d + (double)m * dw_glob)) > 1e-12 * fabs(wm) + 1e-300) uniform = false;
      const float aw = (float)fabs(wm);
      wabs_min = fminf(wabs_min, aw);
      wabs_max = fmaxf(wabs_max, aw);
    }
    if (nv == 0) { wabs_min = 0.f; wabs_max = 0.f; }
    const uint32_t valid = (nv >= 32) ? 0xffffffffu : ((1u << nv) - 1u);
    __syncwarp();

    uint32_t t0, t1;
    subset_tracks(p, sub, t0, t1);
    uint32_t cur_t = t0;
    while (cur_t < t1 && track_body(p, cur_t) == 0) ++cur_t;
    if (threadIdx.x == 0 && cur_t < t1) {
      const uint32_t cnt = min((uint32_t)kStage, track_body(p, cur_t));
      const int b = stage_no & 1;
      fence_proxy_async();
      mbar_arrive_expect_tx(&sm.bar[b], cnt * 64u);
      bulk_g2s(sm.stage[b], p.records + (p.offsets[cur_t]) * kRecF4, cnt * 64u, &sm.bar[b]);
    }

    for (uint32_t t = t0; t < t1; ++t) {
      const int64_t base = p.offsets[t];
      const uint32_t n_body = track_body(p, t);
      const uint32_t it_start = p.it_start[t];
      // this lane's U/W constants as point pairs (zero for points it does not own)
      float2 uT[KP], nuT[KP], uP[KP], nuP[KP], wTr[KP], wTi[KP], wPr[KP], wPi[KP];
#pragma unroll
      for (int q = 0; q < KP; ++q) {
        float4 c0[2], c1[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int m = 2 * q + e;
          if (m < nv) {
            const uint64_t i = (uint64_t)t * P + (uint64_t)(j0 + m) + (uint64_t)nO * dir;
            c0[e] = a.consts[2 * i];
            c1[e] = a.consts[2 * i + 1];
          } else {
            c0[e] = c1[e] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
        uT[q] = make_float2(c0[0].x, c0[1].x); nuT[q] = make_float2(c0[0].y, c0[1].y);
        uP[q] = make_float2(c0[0].z, c0[1].z); nuP[q] = make_float2(c0[0].w, c0[1].w);
        wTr[q] = make_float2(c1[0].x, c1[1].x); wTi[q] = make_float2(c1[0].y, c1[1].y);
        wPr[q] = make_float2(c1[0].z, c1[1].z); wPi[q] = make_float2(c1[0].w, c1[1].w);
      }

      for (uint32_t s0 = 0; s0 < n_body; s0 += kStage) {
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
            mbar_arrive_expect_tx(&sm.bar[nbuf], ncnt * 64u);
            bulk_g2s(sm.stage[nbuf], p.records + (p.offsets[nt] + ns0) * kRecF4, ncnt * 64u,
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

        for (uint32_t c0 = 0; c0 < cnt; c0 += 32) {
          const uint32_t mcnt = min(32u, cnt - c0);
          if (active_w) {
            // ---- per-step setup (as in the forward) ----
            const uint32_t l = (uint32_t)lane < mcnt ? (uint32_t)lane : mcnt - 1;
            const float4 r0 = stg[(c0 + l) * kRecF4 + 0];
            const float4 r1 = stg[(c0 + l) * kRecF4 + 1];
            const float4 r2 = stg[(c0 + l) * kRecF4 + 2];
            const float4 r3 = stg[(c0 + l) * kRecF4 + 3];
            const bool first = (s0 + c0 + l) == 0;
            for (int dd = 0; dd < dpw; ++dd) {
              AdjDir &d = sm.dc[warp][dd];
              df tau = df{r0.x, r0.y};
              tau = df_add(tau, df_mul(df{d.dc_h, d.dc_l}, df{r1.z, r1.w}));
              const df nx = df_mul(df{d.dsx_h, d.dsx_l}, df{r0.z, r0.w});
              const df ny = df_mul(df{d.dsy_h, d.dsy_l}, df{r1.x, r1.y});
              tau = df_add(tau, df{-nx.hi, -nx.lo});
              tau = df_add(tau, df{-ny.hi, -ny.lo});
              float ph = __shfl_up_sync(0xffffffffu, tau.hi, 1);
              float pl = __shfl_up_sync(0xffffffffu, tau.lo, 1);
              if (lane == 0) { ph = d.tprev_h; pl = d.tprev_l; }
              const float dtau = first ? (tau.hi + tau.lo) : ((tau.hi - ph) + (tau.lo - pl));
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
              const df rp = df_mul_raw(d_dw, tau);
              float Rs, Rc;
              sincosf(reduce_2pi(rp.hi, rp.lo), &Rs, &Rc);
              float R2c, R2s, Hc, Hs;
              cmul(Rc, Rs, Rc, Rs, R2c, R2s);
              cmul(R2c, R2s, R2c, R2s, Hc, Hs);  // R^(K/2)
              float4 *st = setup + ((size_t)lane * dpw + dd) * 6;
              st[0] = make_float4(tau.hi, tau.lo, Rc, Rs);
              st[1] = make_float4(amp_t, amp_t, amp_p, amp_p);
              st[2] = make_float4(R2c, R2c, R2s, R2s);
              st[3] = make_float4(-R2s, -R2s, Hc, Hc);
              st[4] = make_float4(Hs, Hs, -Hs, -Hs);
              st[5] = make_float4(fabsf(dtau), 0.f, 0.f, 0.f);
              const float th_last = __shfl_sync(0xffffffffu, tau.hi, mcnt - 1);
              const float tl_last = __shfl_sync(0xffffffffu, tau.lo, mcnt - 1);
              __syncwarp();
              if (lane == 0) { d.tprev_h = th_last; d.tprev_l = tl_last; }
            }
            __syncwarp();
            // ---- per step: E and F over this lane's points, reduced over the
            // direction's lanes ----
#pragma unroll 1
            for (uint32_t i = 0; i < mcnt; ++i) {
              const float4 *st = setup + ((size_t)i * dpw + dsub) * 6;
              const float4 A = st[0], R2 = st[2], X = st[3], Y = st[4];
              const float adt = st[5].x;
              const uint32_t s = s0 + c0 + i;
              const bool all_in = wabs_max * adt < kPiLo;
              const bool all_out = wabs_min * adt > kPiHi;
              uint32_t mask = (all_out || nv == 0) ? 0u : valid;
              if (!all_in && !all_out && nv > 0) {
                const AdjDir &d = sm.dc[warp][dsub];
                if (uniform) {
                  mask = omega_range_bits(w0f, dwf, kPiLo / adt, nv);
                  uint32_t unc = omega_range_bits(w0f, dwf, kPiHi / adt, nv) & ~mask;
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
              mask &= valid;
              float2 eT = make_float2(0.f, 0.f), eP = eT, fT = eT, fP = eT;
              if (__any_sync(0xffffffffu, mask != 0u)) {
                float zs, zc;
                phasor_rev(d_w0.hi, d_w0.lo, A.x, A.y, zs, zc);
                float2 ZrA = make_float2(zc, zc * A.z - zs * A.w);
                float2 ZiA = make_float2(zs, zc * A.w + zs * A.z);
                float2 ZrB, ZiB;
                rot2p(ZrA, ZiA, make_float2(X.z, X.w), make_float2(Y.x, Y.y),
                      make_float2(Y.z, Y.w), ZrB, ZiB);
#pragma unroll
                for (int q = 0; q < HP; ++q) {
                  if (!uniform) {  // one reseed per point on a non-uniform axis
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
#pragma unroll
                      for (int e = 0; e < 2; ++e) {
                        const int m = h * (K / 2) + 2 * q + e;
                        const df wr =
                            df_from_double(p.omega[j0 + min(m, max(nv - 1, 0))] * inv2pi);
                        float ss, cc;
                        phasor_rev(wr.hi, wr.lo, A.x, A.y, ss, cc);
                        float2 &zr = h ? ZrB : ZrA;
                        float2 &zi = h ? ZiB : ZiA;
                        if (e == 0) { zr.x = cc; zi.x = ss; } else { zr.y = cc; zi.y = ss; }
                      }
                    }
                  }
#pragma unroll
                  for (int h = 0; h < 2; ++h) {
                    const int m0 = h * (K / 2) + 2 * q, qq = h * HP + q;
                    const float g0 = ((mask >> m0) & 1u) ? 1.f : 0.f;
                    const float g1 = ((mask >> (m0 + 1)) & 1u) ? 1.f : 0.f;
                    const float2 zr = h ? ZrB : ZrA, zi = h ? ZiB : ZiA;
                    const float2 mr = make_float2(zr.x * g0, zr.y * g1);
                    const float2 mi = make_float2(zi.x * g0, zi.y * g1);
                    eT = __ffma2_rn(uT[qq], mr, eT);
                    eT = __ffma2_rn(nuT[qq], mi, eT);
                    eP = __ffma2_rn(uP[qq], mr, eP);
                    eP = __ffma2_rn(nuP[qq], mi, eP);
                    fT = __ffma2_rn(wTr[qq], mi, fT);
                    fT = __ffma2_rn(wTi[qq], mr, fT);
                    fP = __ffma2_rn(wPr[qq], mi, fP);
                    fP = __ffma2_rn(wPi[qq], mr, fP);
                  }
                  if (q + 1 < HP && uniform) {
                    rot2p(ZrA, ZiA, make_float2(R2.x, R2.y), make_float2(R2.z, R2.w),
                          make_float2(X.x, X.y), ZrA, ZiA);
                    rot2p(ZrB, ZiB, make_float2(R2.x, R2.y), make_float2(R2.z, R2.w),
                          make_float2(X.x, X.y), ZrB, ZiB);
                  }
                }
              }
              float4 v = make_float4(eT.x + eT.y, eP.x + eP.y, fT.x + fT.y, fP.x + fP.y);
              for (int o = L / 2; o > 0; o >>= 1) {
                v.x += __shfl_xor_sync(0xffffffffu, v.x, o);
                v.y += __shfl_xor_sync(0xffffffffu, v.y, o);
                v.z += __shfl_xor_sync(0xffffffffu, v.z, o);
                v.w += __shfl_xor_sync(0xffffffffu, v.w, o);
              }
              if (ll == 0) sm.red[warp][i][dsub] = v;
            }
            __syncwarp();
            // ---- chain rule per (direction, step): lane l handles step c0 + l ----
            if ((uint32_t)lane < mcnt) {
              const float4 q2 = stg[(c0 + lane) * kRecF4 + 2];
              const float4 q3 = stg[(c0 + lane) * kRecF4 + 3];
              float g[kAG] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
              for (int dd = 0; dd < dpw; ++dd) {
                if (dgrp * dpw + dd >= n_dirs) continue;
                const AdjDir &d = sm.dc[warp][dd];
                const float4 v = sm.red[warp][lane][dd];
                const float D = q2.w + d.f_c * q2.z - d.f_sx * q2.x - d.f_sy * q2.y;
                const float c2 = 1.f / D;
                const float an = d.f_sx * q3.x + d.f_sy * q3.y + d.f_cz * q3.z;
                const float c1 = an * c2 * c2;
                const float tb = d.thx * q2.x + d.thy * q2.y + d.thz * q2.z;
                const float ta = d.thx * q3.x + d.thy * q3.y + d.thz * q3.z;
                const float pb = d.phx * q2.x + d.phy * q2.y;
                const float pa = d.phx * q3.x + d.phy * q3.y;
                const float amp_t = -(c1 * tb + c2 * ta);
                const float amp_p = -(c1 * pb + c2 * pa);
                const float nv3[3] = {d.f_sx, d.f_sy, d.f_cz};
                const float th3[3] = {d.thx, d.thy, d.thz};
                const float ph3[3] = {d.phx, d.phy, 0.f};
                // x: n (amp_t F_t + amp_p F_p)
                const float fx = amp_t * v.z + amp_p * v.w;
                // bbar: -(2 an c2^3 e.b + c2^2 e.a) n E - c1 e E, a: -(c2^2 e.b) n E - c2 e E
                const float c22 = c2 * c2;
                const float kb = -(v.x * (2.f * an * c22 * c2 * tb + c22 * ta) +
                                   v.y * (2.f * an * c22 * c2 * pb + c22 * pa));
                const float ka = -(v.x * c22 * tb + v.y * c22 * pb);
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                  g[c] += nv3[c] * fx;
                  g[3 + c] += kb * nv3[c] - c1 * (v.x * th3[c] + v.y * ph3[c]);
                  g[6 + c] += ka * nv3[c] - c2 * (v.x * th3[c] + v.y * ph3[c]);
                }
              }
#pragma unroll
              for (int c = 0; c < kAG; ++c) sm.cta[warp][c0 + lane][c] = g[c];
            }
            __syncwarp();
          } else if ((uint32_t)lane < mcnt) {
#pragma unroll
            for (int c = 0; c < kAG; ++c) sm.cta[warp][c0 + lane][c] = 0.f;
          }
        }
        __syncthreads();
        // ---- sum over the CTA's warps; one partial per (group, step) ----
        for (uint32_t e = threadIdx.x; e < cnt * kAG; e += blockDim.x) {
          const uint32_t st = e / kAG, c = e - st * kAG;
          float acc = 0.f;
#pragma unroll
          for (int w = 0; w < W; ++w) acc += sm.cta[w][st][c];
          a.gpart[((uint64_t)grp * p.total_steps + (uint64_t)base + s0 + st) * kAG + c] = acc;
        }
        ++stage_no;
        __syncthreads();
      }
      if (ll == 0) { sm.dc[warp][dsub].tprev_h = 0.f; sm.dc[warp][dsub].tprev_l = 0.f; }
      __syncwarp();
    }
    __syncwarp();
  }
}

size_t adj_smem_bytes(int dpw) {
  return sizeof(AdjSmemFixed<kAW>) + (size_t)kAW * 32 * dpw * 6 * sizeof(float4);
}

struct AdjLayout {
  size_t records, consts, gpart, total;
};

AdjLayout adj_layout(int64_t total_steps, uint64_t P, uint32_t n_tracks, uint32_t n_groups) {
  AdjLayout l;
  l.records = 256;
  l.consts = l.records + ((size_t)total_steps * 64 + 255) / 256 * 256;
  l.gpart = l.consts + ((size_t)n_tracks * P * 32 + 255) / 256 * 256;
  l.total = l.gpart + ((size_t)n_groups * total_steps * kAG * 4 + 255) / 256 * 256;
  return l;
}

// Decomposition of the adjoint: K = 8 points per lane (the near-field shape).
FarMixedConfig adj_config(const sr_grid *g, uint32_t n_tracks, uint32_t &n_groups,
                          uint32_t &n_wtiles) {
  FarMixedConfig cfg = near_mixed_choose(g->n_omega, g->n_theta * g->n_phi, n_tracks,
                                         device_sm_count());
  n_wtiles = (g->n_omega + (uint32_t)(cfg.L * cfg.K) - 1) / (uint32_t)(cfg.L * cfg.K);
  const uint32_t dgroups = (g->n_theta * g->n_phi + cfg.dpw - 1) / cfg.dpw;
  n_groups = (uint32_t)(((uint64_t)dgroups * n_wtiles + cfg.W - 1) / cfg.W);
  return cfg;
}

int check_adjoint_args(const sr_tracks *t, const sr_grid *g, void *const *out) {
  int rc = validate_spectrum_args(t, g, SR_COMP_TOTAL, SR_PREC_MIXED, out);
  if (rc) return rc;
  if (g->mode != SR_MODE_FAR) return fail(SR_ERR_UNSUPPORTED, "the adjoint is far field only");
  if (t->n_snaps != 1)
    return fail(SR_ERR_UNSUPPORTED, "the adjoint differentiates a single snapshot (n_snaps = 1)");
  return SR_OK;
}

}  // namespace
}  // namespace sr

using namespace sr;

extern "C" int sr_far_total_forward_saved(const sr_tracks *t, const sr_grid *g, double *spectrum,
                                          float *saved_A, void *workspace,
                                          size_t workspace_bytes, void *stream) {
  clear_error();
  void *out[6] = {spectrum};
  int rc = check_adjoint_args(t, g, out);
  if (rc) return rc;
  if (!saved_A) return fail(SR_ERR_INVALID, "saved_A is NULL");
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  if (P == 0 || t->n_tracks == 0) return SR_OK;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(saved_A, 0, (size_t)t->n_tracks * P * 16, s);
  if (e != cudaSuccess) return cuda_fail(e, "saved_A reset");
  const FarMixedConfig cfg = far_mixed_choose(g->n_omega, g->n_theta * g->n_phi, t->n_tracks,
                                              device_sm_count());
  FarMixedParams p = make_far_mixed_params(t, g, SR_COMP_TOTAL, out);
  p.save_A = saved_A;
  return launch_far_mixed(p, cfg, workspace, workspace_bytes, s);
}

extern "C" int64_t sr_far_total_backward_workspace_bytes(const sr_tracks *t, const sr_grid *g) {
  if (!t || !g) return -1;
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  uint32_t n_groups = 0, n_wtiles = 0;
  adj_config(g, t->n_tracks, n_groups, n_wtiles);
  return (int64_t)adj_layout(t->total_steps, P, t->n_tracks, n_groups).total;
}

extern "C" int sr_far_total_backward(const sr_tracks *t, const sr_grid *g,
                                     const double *grad_spectrum, const float *saved_A,
                                     double *const *grad_track, double *grad_weight,
                                     void *workspace, size_t workspace_bytes, void *stream) {
  clear_error();
  void *dummy[6] = {(void *)grad_spectrum};
  int rc = check_adjoint_args(t, g, dummy);
  if (rc) return rc;
  if (!saved_A || !grad_track || !grad_weight)
    return fail(SR_ERR_INVALID, "saved_A, grad_track and grad_weight must not be NULL");
  for (int i = 0; i < 6; ++i)
    if (!grad_track[i]) return fail(SR_ERR_INVALID, "grad_track[%d] is NULL", i);
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  cudaStream_t s = (cudaStream_t)stream;
  if (t->n_tracks == 0) return SR_OK;
  uint32_t n_groups = 0, n_wtiles = 0;
  const FarMixedConfig cfg = adj_config(g, t->n_tracks, n_groups, n_wtiles);
  const AdjLayout lay = adj_layout(t->total_steps, P, t->n_tracks, n_groups);
  if (!workspace || workspace_bytes < lay.total)
    return fail(SR_ERR_WORKSPACE, "workspace of %zu bytes needed, %zu given", lay.total,
                workspace_bytes);
  if (((uintptr_t)workspace & 255u) != 0)
    return fail(SR_ERR_WORKSPACE, "workspace not 256-byte aligned");
  unsigned char *w = (unsigned char *)workspace;

  AdjParams a;
  memset(&a, 0, sizeof(a));
  a.f = make_far_mixed_params(t, g, SR_COMP_TOTAL, dummy);
  a.f.status = (int *)w;
  a.f.records = (float4 *)(w + lay.records);
  a.f.dpw = (uint32_t)cfg.dpw;
  a.f.n_wtiles = n_wtiles;
  a.f.n_groups = n_groups;
  a.f.n_sub = (uint32_t)cfg.n_sub;
  a.f.n_items = n_groups * a.f.n_sub;
  a.grad_spec = grad_spectrum;
  a.save_A = (const float4 *)saved_A;
  a.consts = (float4 *)(w + lay.consts);
  a.gpart = (float *)(w + lay.gpart);
  for (int i = 0; i < 6; ++i) a.grad[i] = grad_track[i];
  a.grad_w = grad_weight;

  cudaError_t e = cudaMemsetAsync(w, 0, 256, s);
  if (e != cudaSuccess) return cuda_fail(e, "status reset");
  int dev = 0, n_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev);
  if (t->total_steps > 0) {
    int64_t nb = (t->total_steps + 255) / 256;
    if (nb > 8 * n_sm * 16) nb = 8 * n_sm * 16;
    launch_far_prepass(a.f, (int)nb, s);
  }
  {
    uint64_t nb = ((uint64_t)t->n_tracks * P + 255) / 256;
    if (nb > (uint64_t)n_sm * 64) nb = (uint64_t)n_sm * 64;
    adj_prep_kernel<<<(unsigned)nb, 256, 0, s>>>(a);
    adj_weight_kernel<<<t->n_tracks, 256, 0, s>>>(a);
  }
  rc = cuda_fail(cudaGetLastError(), "adjoint prep launch");
  if (rc) return rc;
  const size_t smem = adj_smem_bytes(cfg.dpw);
  e = cudaFuncSetAttribute(adj_far_kernel<kAW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint smem attribute");
  const int grid = std::max(1, std::min<int>((int)a.f.n_items, n_sm));
  void *tok = nullptr;
  timing_record(s, true, &tok);
  adj_far_kernel<kAW><<<grid, kAW * 32, smem, s>>>(a);
  timing_record(s, false, &tok);
  rc = cuda_fail(cudaGetLastError(), "adjoint kernel launch");
  if (rc) return rc;
  if (t->total_steps > 0) {
    int64_t nb = (t->total_steps + 255) / 256;
    if (nb > 8 * n_sm * 16) nb = 8 * n_sm * 16;
    if (a.f.track_f32)
      adj_final_kernel<float><<<(int)nb, 256, 0, s>>>(a);
    else
      adj_final_kernel<double><<<(int)nb, 256, 0, s>>>(a);
  }
  return cuda_fail(cudaGetLastError(), "adjoint final launch");
}
