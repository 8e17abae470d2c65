// Adjoint of the mixed-precision far field (every comp, one snapshot).
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
// The comps differ only in how the loss sees A (point sensitivity, below):
//   quadratic comps (total, cartesian, spheric: outputs w dt^2 |b_k . A|^2
//   with b_k the output's unit vector on (theta-hat, phi-hat)):
//     U = w M A,  M = 2 dt^2 sum_k g_k b_k b_k^T (2 x 2, real);
//   linear comps (cartesian_complex, spheric_complex: outputs sqrt(w) dt
//   f(omega) Re/Im (b_k . A), f the FormFactor or 1):
//     U = sqrt(w) V,  V = dt f sum_k (g_k,re + i g_k,im) b_k;
// so that dL = Re(conj(U) . dA), and dL/dw_t = sum_p Re(conj(U) . A_t) / (2 w_t).
//
// Layout: E and F are sums over omega for each (direction, step), so a lane
// owns one step and walks the omega axis of a direction with the rotation
// recurrence z <- z exp(i domega tau) (reseeded from the double-float phase
// every 8 points); U and W of a block of (direction, omega) points are built
// in shared memory from the saved amplitudes and read by every lane
// (broadcast).  A CTA owns 256 consecutive steps of one track and loops over
// every direction, so each step's gradient is summed in registers and written
// once: no atomics, no cross-lane reductions, a deterministic result.
// Phases are recomputed, not stored.
#include <algorithm>
#include <cmath>

#include "sr_common.cuh"
#include "sr_internal.h"
#include "sr_mixed_common.cuh"
#include "sr_adjoint_common.cuh"

namespace sr {
namespace {

constexpr int kAW = 8;                // warps per CTA
constexpr int kASteps = kAW * 32;     // steps per work item (one per lane)
constexpr int kAStage = 1024;         // (direction, omega) points per constants stage
constexpr int kARS = 8;               // omega points per phasor reseed
constexpr int kAG = 9;                // per-step gradient components: x (3), bbar (3), a (3)

struct AdjParams {
  FarMixedParams f;            // tracks, grid, records, status
  const double *grad_out[6];   // [P] dL/dS_k per output of the comp, device layout
  int linear;                  // comp is linear in A (the *_complex comps)
  const float4 *save_A;        // [n_tracks][P] (A_th re, im, A_ph re, im)
  float4 *gcst;                // [P] point sensitivity in FP32: M (xx, xy, yy, 0) or V
  float4 *wtab;                // [nO] (omega/2pi hi, lo, omega, |omega|) in FP32
  float4 *dirtab;              // [n_dirs][4] direction constants
  AdjGlobals *glob;
  int64_t *item_off;           // [n_tracks + 1] first work item of each track
  double *gstep;               // [total_steps][kAG] per-step gradients (bbar, a form)
  double *grad[6];             // x, y, z, ux, uy, uz  [total_steps]
  double *grad_w;              // [n_tracks]
};

// Point sensitivity of the loss to (A_theta, A_phi) for output gradients g_k
// at point gi: M = (xx, xy, yy) of the quadratic comps (2 dt^2 included) or V
// = (th re, th im, ph re, ph im) of the linear ones (dt and FormFactor
// included), in FP64.
__device__ __forceinline__ void point_sens(const AdjParams &a, uint32_t ksnap, uint64_t gi,
                                           double out[4]) {
  const FarMixedParams &p = a.f;
  const uint32_t nO = p.n_omega, nT = p.n_theta;
  const uint64_t gk = (uint64_t)ksnap * nO * nT * p.n_phi + gi;  // snapshot ksnap's slot
  const uint64_t d = gi / nO;
  const uint32_t m = (uint32_t)(gi - d * nO);
  const uint32_t iT = (uint32_t)(d % nT), iP = (uint32_t)(d / nT);
  const double sT = p.sin_theta[iT], cT = p.cos_theta[iT];
  const double sP = p.sin_phi[iP], cP = p.cos_phi[iP];
  // output unit vectors x, y, z on (theta-hat, phi-hat)
  const double bt[3] = {cT * cP, cT * sP, -sT}, bp[3] = {-sP, cP, 0.0};
  const double s2 = 2.0 * p.dt * p.dt;
  auto g = [&](int k) { return a.grad_out[k][gk]; };
  out[0] = out[1] = out[2] = out[3] = 0.0;
  switch (p.comp) {
    case SR_COMP_TOTAL:
      out[0] = out[2] = s2 * g(0);
      break;
    case SR_COMP_CARTESIAN:
      for (int k = 0; k < 3; ++k) {
        const double gk = s2 * g(k);
        out[0] += gk * bt[k] * bt[k];
        out[1] += gk * bt[k] * bp[k];
        out[2] += gk * bp[k] * bp[k];
      }
      break;
    case SR_COMP_SPHERIC:  // outputs r (identically 0), theta, phi
      out[0] = s2 * g(1);
      out[2] = s2 * g(2);
      break;
    case SR_COMP_CARTESIAN_COMPLEX: {
      const double f = p.dt * p.form_factor[m];
      for (int k = 0; k < 3; ++k) {
        const double gr = f * g(2 * k), gim = f * g(2 * k + 1);
        out[0] += gr * bt[k];
        out[1] += gim * bt[k];
        out[2] += gr * bp[k];
        out[3] += gim * bp[k];
      }
      break;
    }
    default:  // SR_COMP_SPHERIC_COMPLEX: rre, rim (identically 0), theta, phi re/im
      out[0] = p.dt * g(2);
      out[1] = p.dt * g(3);
      out[2] = p.dt * g(4);
      out[3] = p.dt * g(5);
      break;
  }
}

// Point sensitivities in FP32, and the direction table:
//   [0] (1 - cos theta hi, lo, n_x hi, lo)   [1] (n_y hi, lo, 1 - cos theta, n_x)
//   [2] (n_y, n_z, theta-hat x, y)           [3] (theta-hat z, phi-hat x, y, 0)
__global__ void adj_prep_kernel(AdjParams a) {
  const FarMixedParams &p = a.f;
  const uint32_t nT = p.n_theta;
  const uint64_t n_dirs = (uint64_t)nT * p.n_phi;
  const uint64_t P = n_dirs * p.n_omega;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P * p.n_snaps;
       i += stride) {
    double v[4];
    point_sens(a, (uint32_t)(i / P), i % P, v);
    a.gcst[i] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
  }
  for (uint64_t d = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n_dirs; d += stride) {
    const uint32_t iT = (uint32_t)(d % nT), iP = (uint32_t)(d / nT);
    const double sT = p.sin_theta[iT], cT = p.cos_theta[iT];
    const double sPh = p.sin_phi[iP], cPh = p.cos_phi[iP];
    const double n0 = sT * cPh, n1 = sT * sPh;
    const df c = df_from_double(1.0 - cT), sx = df_from_double(n0), sy = df_from_double(n1);
    float4 *o = a.dirtab + 4 * d;
    o[0] = make_float4(c.hi, c.lo, sx.hi, sx.lo);
    o[1] = make_float4(sy.hi, sy.lo, (float)(1.0 - cT), (float)n0);
    o[2] = make_float4((float)n1, (float)cT, (float)(cT * cPh), (float)(cT * sPh));
    o[3] = make_float4((float)(-sT), (float)(-sPh), (float)cPh, 0.f);
  }
}


// dL/dw_t = sum_p Re(conj(U) . A_t) / (2 w_t) in two fixed-order stages:
// block (t, b) sums chunk b of track t's points into wpart[t][b] (FP64, from
// the FP64 point sensitivities), then one thread per track adds its chunks.
__global__ void adj_weight_partial_far_kernel(AdjParams a, uint64_t P, uint32_t n_chunks,
                                              double *wpart) {
  const uint32_t t = blockIdx.x / n_chunks, b = blockIdx.x % n_chunks;
  const uint64_t chunk = (P + n_chunks - 1) / n_chunks;
  const uint64_t g0 = (uint64_t)b * chunk, g1 = min(P, g0 + chunk);
  double acc = 0.0;
  for (uint64_t g = g0 + threadIdx.x; g < g1; g += blockDim.x) {
    for (uint32_t k = 0; k < a.f.n_snaps; ++k) {  // a snapshot that never fired has A = 0
      double v[4];
      point_sens(a, k, g, v);
      const float4 A = a.save_A[((uint64_t)t * a.f.n_snaps + k) * P + g];
      const double ar = A.x, ai = A.y, br = A.z, bi = A.w;
      if (a.linear)  // Re(conj(V) . A)
        acc += v[0] * ar + v[1] * ai + v[2] * br + v[3] * bi;
      else           // A^H M A
        acc += v[0] * (ar * ar + ai * ai) + 2.0 * v[1] * (ar * br + ai * bi) +
               v[2] * (br * br + bi * bi);
    }
  }
  __shared__ double red[kWeightThreads];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) wpart[blockIdx.x] = red[0];
}

// quadratic comps: dL/dw = (A^H M A) / 2 (M holds 2 dt^2); linear comps:
// dL/dw = Re(conj(V) . A) / (2 sqrt(w)).
__global__ void adj_weight_final_far_kernel(const double *wpart, uint32_t n_tracks,
                                            uint32_t n_chunks, int linear, const double *weight,
                                            double *grad_w) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tracks) return;
  double s = 0.0;
  for (uint32_t b = 0; b < n_chunks; ++b) s += wpart[(uint64_t)t * n_chunks + b];
  grad_w[t] = linear ? (weight[t] > 0.0 ? s / (2.0 * sqrt(weight[t])) : 0.0) : 0.5 * s;
}

// Per-step gradients: map dL/dbbar and dL/da of steps s-1 and s to dL/dbeta_s
// and dL/du_s.
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
    const int64_t s = g - p.offsets[t];
    const int64_t n_body = (int64_t)track_body(p, t);
    double cur[kAG] = {0}, prev[kAG] = {0};
    if (s < n_body)
      for (int c = 0; c < kAG; ++c) cur[c] = a.gstep[g * kAG + c];
    if (s >= 1 && s - 1 < n_body)
      for (int c = 3; c < kAG; ++c) prev[c] = a.gstep[(g - 1) * kAG + c];
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

// Shared memory of one CTA.  Constants are stored per pair of omega slots
// (m, m+1) of a direction whose omega axis is padded to a multiple of kARS
// slots (padding slots carry zero constants):
//   [0] (U_th re m, m+1, -Im U_th m, m+1)   [1] the same for U_ph
//   [2] (Re W_th m, m+1, Im W_th m, m+1)    [3] the same for W_ph
//   [4] (omega/2pi hi, lo of m, of m+1)     [5] (|omega| of m, m+1, 0, 0)
constexpr int kARecS = kRecF4;  // record stride in shared memory (80 bytes, as in HBM)

struct AdjSmem {
  float4 rec[kASteps + 1][kARecS];  // step records r0 - 1 .. r0 + 255
  float4 cst[kAStage / 2][6];
  uint64_t bar;
  uint64_t pad_;
};

__device__ __forceinline__ float2 lo2(const float4 &v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4 &v) { return make_float2(v.z, v.w); }

// E += Re(U z), F += Im(W z) on theta-hat and phi-hat for a pair of points.
struct EF2 {
  float2 et, ep, ft, fp;
  __device__ __forceinline__ void add(const float4 *c, float2 zr, float2 zi) {
    const float4 c0 = c[0], c1 = c[1], c2 = c[2], c3 = c[3];
    et = __ffma2_rn(lo2(c0), zr, et);
    et = __ffma2_rn(hi2(c0), zi, et);
    ep = __ffma2_rn(lo2(c1), zr, ep);
    ep = __ffma2_rn(hi2(c1), zi, ep);
    ft = __ffma2_rn(lo2(c2), zi, ft);
    ft = __ffma2_rn(hi2(c2), zr, ft);
    fp = __ffma2_rn(lo2(c3), zi, fp);
    fp = __ffma2_rn(hi2(c3), zr, fp);
  }
};

// tau = q + (1 - cos theta) z - n_x x - n_y y of one step record, double-float.
__device__ __forceinline__ df record_tau(const float4 *r, const float4 &d0, const float4 &d1) {
  const float4 r0 = r[0], r1 = r[1];
  df tau = df{r0.x, r0.y};
  tau = df_add(tau, df_mul(df{d0.x, d0.y}, df{r1.z, r1.w}));
  const df nx = df_mul(df{d0.z, d0.w}, df{r0.z, r0.w});
  const df ny = df_mul(df{d1.x, d1.y}, df{r1.x, r1.y});
  tau = df_add(tau, df{-nx.hi, -nx.lo});
  return df_add(tau, df{-ny.hi, -ny.lo});
}

template <int W>
__global__ void __launch_bounds__(W * 32, 2) adj_far_kernel(AdjParams a) {
  const FarMixedParams &p = a.f;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  AdjSmem &sm = *reinterpret_cast<AdjSmem *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ls = (uint32_t)(warp * 32 + lane);  // this lane's step within the item
  if (threadIdx.x == 0) {
    mbar_init(&sm.bar, 1);
    fence_mbar_init();
  }
  __syncthreads();

  const AdjGlobals G = *a.glob;
  const uint32_t nO = p.n_omega, nT = p.n_theta;
  const uint32_t nOp = (nO + kARS - 1) / kARS * kARS;  // padded omega slots per direction
  const uint64_t P = (uint64_t)nO * nT * p.n_phi;
  const uint64_t Pp = (uint64_t)nOp * nT * p.n_phi;
  const int64_t n_items = a.item_off[p.n_tracks];
  const df d_dw = df{G.dw_h, G.dw_l};
  uint32_t it_no = 0;

  for (int64_t item = blockIdx.x; item < n_items; item += gridDim.x, ++it_no) {
    uint32_t lo = 0, hi = p.n_tracks;  // last track with item_off[t] <= item
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (a.item_off[mid] <= item) lo = mid; else hi = mid;
    }
    const uint32_t t = lo;
    const int64_t base = p.offsets[t];
    const uint32_t n_body = track_body(p, t);
    SnapSegment seg{0, 0, 0, 0};
    track_segments(p, t, (uint32_t)kASteps, (uint32_t)(item - a.item_off[t]), &seg);
    const uint32_t r0 = seg.r0, r1 = seg.r1;  // the steps enter snapshots seg.k0 .. seg.k1
    const uint32_t has_prev = r0 > 0 ? 1u : 0u;
    const uint32_t n_rec = r1 - r0 + has_prev;
    if (threadIdx.x == 0) {  // the item's records in one bulk copy
      fence_proxy_async();
      mbar_arrive_expect_tx(&sm.bar, n_rec * kRecBytes);
      bulk_g2s(sm.rec[0], p.records + (base + r0 - has_prev) * kRecF4, n_rec * kRecBytes,
               &sm.bar);
    }
    const bool ok = mbar_wait_bounded(&sm.bar, it_no & 1u, kWaitLimitNs);
    if (__syncthreads_or(!ok)) {
      if (threadIdx.x == 0) {
        atomicExch(p.status, STATUS_WAIT_TIMEOUT);
        mbar_wait_bounded(&sm.bar, it_no & 1u, kWaitLimitNs);
      }
      __syncthreads();
      return;
    }

    const uint32_t s = r0 + ls;
    const bool valid = s < r1;
    const uint32_t si = min(has_prev + ls, n_rec - 1);  // record index of step s
    // record 0 is step 0 of the track (no previous phase) or, for lanes past
    // the end of a one-step item, the only record loaded
    const bool first = (si == 0);
    const float wt = (float)p.weight[t];
    const float swt = (float)sqrt(p.weight[t]);
    const uint32_t it_start = p.it_start[t];
    double gD[kAG];
#pragma unroll
    for (int c = 0; c < kAG; ++c) gD[c] = 0.0;

    // per (direction, step) state, kept across constants stages
    float th = 0.f, tl = 0.f, rc = 1.f, rs = 0.f, adt = 0.f;
    float2 r2c = make_float2(1.f, 1.f), r2s = make_float2(0.f, 0.f), nr2s = r2s;
    int mode = 1;  // 0: every omega included, 1: none, 2: per point
    EF2 ef;
    ef.et = ef.ep = ef.ft = ef.fp = make_float2(0.f, 0.f);

    for (uint64_t f0 = 0; f0 < Pp; f0 += kAStage) {
      const uint32_t nf = (Pp - f0 < (uint64_t)kAStage) ? (uint32_t)(Pp - f0) : (uint32_t)kAStage;
      __syncthreads();  // the previous stage's constants are no longer read
      for (uint32_t j = threadIdx.x; j < nf / 2; j += blockDim.x) {
        const uint64_t f = f0 + 2 * j;
        const uint64_t dj = f / nOp;
        const uint32_t m = (uint32_t)(f - dj * nOp);
        float4 u[2], w[2], wv[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          if (m + e < nO) {
            const uint64_t gi = dj * nO + m + e;
            wv[e] = a.wtab[m + e];
            // U summed over the snapshots these steps enter
            u[e] = make_float4(0.f, 0.f, 0.f, 0.f);
            for (uint32_t k = seg.k0; k <= seg.k1; ++k) {
              const float4 C = a.gcst[(uint64_t)k * P + gi];
              if (a.linear) {
                u[e].x += swt * C.x; u[e].y += swt * C.y;
                u[e].z += swt * C.z; u[e].w += swt * C.w;
              } else {
                const float4 A = a.save_A[((uint64_t)t * p.n_snaps + k) * P + gi];
                u[e].x += wt * (C.x * A.x + C.y * A.z);
                u[e].y += wt * (C.x * A.y + C.y * A.w);
                u[e].z += wt * (C.y * A.x + C.z * A.z);
                u[e].w += wt * (C.y * A.y + C.z * A.w);
              }
            }
            w[e] = make_float4(wv[e].z * u[e].x, -wv[e].z * u[e].y, wv[e].z * u[e].z,
                               -wv[e].z * u[e].w);
          } else {
            u[e] = w[e] = wv[e] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
        }
        float4 *o = sm.cst[j];
        o[0] = make_float4(u[0].x, u[1].x, u[0].y, u[1].y);
        o[1] = make_float4(u[0].z, u[1].z, u[0].w, u[1].w);
        o[2] = make_float4(w[0].x, w[1].x, w[0].y, w[1].y);
        o[3] = make_float4(w[0].z, w[1].z, w[0].w, w[1].w);
        o[4] = make_float4(wv[0].x, wv[0].y, wv[1].x, wv[1].y);
        o[5] = make_float4(wv[0].w, wv[1].w, 0.f, 0.f);
      }
      __syncthreads();
      float gF[kAG];
#pragma unroll
      for (int c = 0; c < kAG; ++c) gF[c] = 0.f;

      uint32_t d = (uint32_t)(f0 / nOp);
      for (uint64_t fd = (uint64_t)d * nOp; fd < f0 + nf; fd += nOp, ++d) {
        const uint32_t m_lo = (uint32_t)(max(fd, f0) - fd);
        const uint32_t m_hi = (uint32_t)(min(fd + nOp, f0 + nf) - fd);
        // slot m of direction d sits at stage index fd + m - f0 >= 0 for m >= m_lo
        const int64_t seg = (int64_t)fd - (int64_t)f0;
        if (m_lo == 0) {  // a new direction: phase, rotation and mask of step s
          const float4 d0 = a.dirtab[4 * (uint64_t)d], d1 = a.dirtab[4 * (uint64_t)d + 1];
          const df tau = record_tau(sm.rec[si], d0, d1);
          float dtau = tau.hi + tau.lo;
          if (!first) {
            const df tp = record_tau(sm.rec[si - 1], d0, d1);
            dtau = (tau.hi - tp.hi) + (tau.lo - tp.lo);
          }
          th = tau.hi;
          tl = tau.lo;
          adt = fabsf(dtau);
          mode = (!valid || G.wabs_min * adt > kPiHi) ? 1 : (G.wabs_max * adt < kPiLo ? 0 : 2);
          const df rp = df_mul_raw(d_dw, tau);
          sincosf(reduce_2pi(rp.hi, rp.lo), &rs, &rc);
          float c2r, s2r;
          cmul(rc, rs, rc, rs, c2r, s2r);
          r2c = make_float2(c2r, c2r);
          r2s = make_float2(s2r, s2r);
          nr2s = make_float2(-s2r, -s2r);
          ef.et = ef.ep = ef.ft = ef.fp = make_float2(0.f, 0.f);
        }
        if (!__all_sync(0xffffffffu, mode == 1)) {
          if (G.uniform && __all_sync(0xffffffffu, mode != 2)) {
            // every point of the segment included (lanes with mode 1 are
            // discarded below): per block of kARS slots one reseed, then
            // pairs rotated by R^2
#pragma unroll 1
            for (uint32_t m = m_lo; m < m_hi; m += kARS) {
              const float4 *cp = sm.cst[(seg + (int64_t)m) >> 1];
              float zs, zc;
              phasor_rev(cp[4].x, cp[4].y, th, tl, zs, zc);
              float2 zr = make_float2(zc, zc * rc - zs * rs);
              float2 zi = make_float2(zs, zc * rs + zs * rc);
#pragma unroll
              for (int q = 0; q < kARS / 2; ++q) {
                ef.add(cp + 6 * q, zr, zi);
                if (q + 1 < kARS / 2) rot2p(zr, zi, r2c, r2s, nr2s, zr, zi);
              }
            }
          } else {
            // per-point mask (and one reseed per point on a non-uniform axis)
            double n0 = 0.0, n1 = 0.0, cT = 0.0;
            bool have_n = false;
#pragma unroll 1
            for (uint32_t m = m_lo; m < m_hi; m += kARS) {
              const float4 *cp = sm.cst[(seg + (int64_t)m) >> 1];
              float2 zr, zi;
              {
                float zs, zc;
                phasor_rev(cp[4].x, cp[4].y, th, tl, zs, zc);
                zr = make_float2(zc, zc * rc - zs * rs);
                zi = make_float2(zs, zc * rs + zs * rc);
              }
#pragma unroll 1
              for (int q = 0; q < kARS / 2; ++q) {
                const float4 *c = cp + 6 * q;
                if (!G.uniform) {
                  float zs, zc;
                  phasor_rev(c[4].x, c[4].y, th, tl, zs, zc);
                  zr.x = zc;
                  zi.x = zs;
                  phasor_rev(c[4].z, c[4].w, th, tl, zs, zc);
                  zr.y = zc;
                  zi.y = zs;
                }
                const float4 aw = c[5];
                bool inc[2] = {aw.x * adt < kPiLo, aw.y * adt < kPiLo};
                if (mode == 2) {
#pragma unroll
                  for (int e = 0; e < 2; ++e) {
                    const float ph = (e ? aw.y : aw.x) * adt;
                    const uint32_t mm = m + 2 * q + e;
                    if (!inc[e] && !(ph > kPiHi) && mm < nO) {
                      if (!have_n) {
                        const uint32_t iT = d % nT, iP = d / nT;
                        n0 = p.sin_theta[iT] * p.cos_phi[iP];
                        n1 = p.sin_theta[iT] * p.sin_phi[iP];
                        cT = p.cos_theta[iT];
                        have_n = true;
                      }
                      inc[e] = exact_mask(p, base, s, it_start, p.omega[mm], n0, n1, cT);
                    }
                  }
                }
                const float2 g = make_float2(inc[0] ? 1.f : 0.f, inc[1] ? 1.f : 0.f);
                ef.add(c, __fmul2_rn(zr, g), __fmul2_rn(zi, g));
                if (G.uniform) rot2p(zr, zi, r2c, r2s, nr2s, zr, zi);
              }
            }
          }
        }
        if (m_hi == nOp && mode != 1) {  // the direction is complete: chain rule
          const float et = ef.et.x + ef.et.y, ep = ef.ep.x + ef.ep.y;
          const float ft = ef.ft.x + ef.ft.y, fp = ef.fp.x + ef.fp.y;
          const float4 d1 = a.dirtab[4 * (uint64_t)d + 1], d2 = a.dirtab[4 * (uint64_t)d + 2],
                       d3 = a.dirtab[4 * (uint64_t)d + 3];
          const float4 q2 = sm.rec[si][2], q3 = sm.rec[si][3];
          const float f_c = d1.z, f_sx = d1.w, f_sy = d2.x, f_cz = d2.y;
          const float thx = d2.z, thy = d2.w, thz = d3.x, phx = d3.y, phy = d3.z;
          const float D = q2.w + f_c * q2.z - f_sx * q2.x - f_sy * q2.y;
          const float c2 = __frcp_rn(D);
          const float an = f_sx * q3.x + f_sy * q3.y + f_cz * q3.z;
          const float c22 = c2 * c2;
          const float c1 = an * c22;
          const float tb = thx * q2.x + thy * q2.y + thz * q2.z;
          const float ta = thx * q3.x + thy * q3.y + thz * q3.z;
          const float pb = phx * q2.x + phy * q2.y;
          const float pa = phx * q3.x + phy * q3.y;
          const float amp_t = -(c1 * tb + c2 * ta);
          const float amp_p = -(c1 * pb + c2 * pa);
          // x: n (amp_t F_t + amp_p F_p)
          const float fx = amp_t * ft + amp_p * fp;
          // bbar: -(2 an c2^3 e.b + c2^2 e.a) n E - c1 e E;  a: -(c2^2 e.b) n E - c2 e E
          const float kb = -(et * (2.f * an * c22 * c2 * tb + c22 * ta) +
                             ep * (2.f * an * c22 * c2 * pb + c22 * pa));
          const float ka = -(et * c22 * tb + ep * c22 * pb);
          const float nv3[3] = {f_sx, f_sy, f_cz};
          const float ev3[3] = {et * thx + ep * phx, et * thy + ep * phy, et * thz};
#pragma unroll
          for (int c = 0; c < 3; ++c) {
            gF[c] += nv3[c] * fx;
            gF[3 + c] += kb * nv3[c] - c1 * ev3[c];
            gF[6 + c] += ka * nv3[c] - c2 * ev3[c];
          }
        }
      }
#pragma unroll
      for (int c = 0; c < kAG; ++c) gD[c] += (double)gF[c];
    }
    if (valid) {
#pragma unroll
      for (int c = 0; c < kAG; ++c) a.gstep[(uint64_t)(base + s) * kAG + c] = gD[c];
    }
    __syncthreads();  // records of this item no longer read
  }
}

size_t adj_smem_bytes() { return sizeof(AdjSmem); }

struct AdjLayout {
  size_t records, gcst, wtab, dirtab, glob, item_off, gstep, wpart, total;
  uint32_t w_chunks;
};

AdjLayout adj_layout(int64_t total_steps, uint64_t P, uint32_t n_omega, uint64_t n_dirs,
                     uint32_t n_tracks, uint32_t n_snaps) {
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  AdjLayout l;
  l.w_chunks = adj_weight_chunks(P, n_tracks, device_sm_count());
  l.records = 256;
  l.gcst = l.records + up((size_t)total_steps * kRecBytes);
  l.wtab = l.gcst + up((size_t)P * 16 * (n_snaps ? n_snaps : 1));
  l.dirtab = l.wtab + up((size_t)n_omega * 16);
  l.glob = l.dirtab + up((size_t)n_dirs * 64);
  l.item_off = l.glob + 256;
  l.gstep = l.item_off + up(((size_t)n_tracks + 1) * 8);
  l.wpart = l.gstep + up((size_t)total_steps * kAG * 8);
  l.total = l.wpart + up((size_t)n_tracks * l.w_chunks * 8);
  return l;
}

int check_adjoint_args(const sr_tracks *t, const sr_grid *g, void *const *out,
                       int comp = SR_COMP_TOTAL) {
  int rc = validate_spectrum_args(t, g, comp, SR_PREC_MIXED, out);
  if (rc) return rc;
  if (g->mode != SR_MODE_FAR) return fail(SR_ERR_UNSUPPORTED, "the adjoint is far field only");
  if (t->n_snaps < 1)
    return fail(SR_ERR_UNSUPPORTED, "the adjoint needs at least one snapshot (n_snaps >= 1)");
  return SR_OK;
}

}  // namespace
}  // namespace sr

using namespace sr;

extern "C" int sr_far_forward_saved(const sr_tracks *t, const sr_grid *g, int comp,
                                    int precision, void *const *out, float *saved_A,
                                    void *workspace, size_t workspace_bytes, void *stream) {
  clear_error();
  int rc = check_adjoint_args(t, g, out, comp);
  if (rc) return rc;
  if (precision != SR_PREC_MIXED && precision != SR_PREC_DF)
    return fail(SR_ERR_INVALID, "precision %d (SR_PREC_MIXED or SR_PREC_DF)", precision);
  if (!saved_A) return fail(SR_ERR_INVALID, "saved_A is NULL");
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  if (P == 0 || t->n_tracks == 0) return SR_OK;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(saved_A, 0, (size_t)t->n_tracks * t->n_snaps * P * 16, s);
  if (e != cudaSuccess) return cuda_fail(e, "saved_A reset");
  FarMixedParams p = make_far_mixed_params(t, g, comp, out);
  p.save_A = saved_A;
  if (precision == SR_PREC_DF) {
    const FarMixedConfig cfg =
        far_df_choose(g->n_omega, g->n_theta * g->n_phi, t->n_tracks, device_sm_count());
    return launch_far_df(p, cfg, workspace, workspace_bytes, s);
  }
  return launch_far_mixed(p, mixed_config(t, g, comp), workspace, workspace_bytes, s);
}

extern "C" int sr_far_total_forward_saved(const sr_tracks *t, const sr_grid *g, double *spectrum,
                                          float *saved_A, void *workspace,
                                          size_t workspace_bytes, void *stream) {
  void *out[6] = {spectrum};
  return sr_far_forward_saved(t, g, SR_COMP_TOTAL, SR_PREC_MIXED, out, saved_A, workspace,
                              workspace_bytes, stream);
}

extern "C" int sr_far_total_forward_saved_df(const sr_tracks *t, const sr_grid *g,
                                             double *spectrum, float *saved_A, void *workspace,
                                             size_t workspace_bytes, void *stream) {
  void *out[6] = {spectrum};
  return sr_far_forward_saved(t, g, SR_COMP_TOTAL, SR_PREC_DF, out, saved_A, workspace,
                              workspace_bytes, stream);
}

extern "C" int64_t sr_far_backward_workspace_bytes(const sr_tracks *t, const sr_grid *g) {
  if (!t || !g) return -1;
  const uint64_t n_dirs = (uint64_t)g->n_theta * g->n_phi;
  return (int64_t)adj_layout(t->total_steps, n_dirs * g->n_omega, g->n_omega, n_dirs,
                             t->n_tracks, t->n_snaps)
      .total;
}

extern "C" int64_t sr_far_total_backward_workspace_bytes(const sr_tracks *t, const sr_grid *g) {
  return sr_far_backward_workspace_bytes(t, g);
}

extern "C" int sr_far_total_backward(const sr_tracks *t, const sr_grid *g,
                                     const double *grad_spectrum, const float *saved_A,
                                     double *const *grad_track, double *grad_weight,
                                     void *workspace, size_t workspace_bytes, void *stream) {
  const double *grad_out[6] = {grad_spectrum};
  return sr_far_backward(t, g, SR_COMP_TOTAL, grad_out, saved_A, grad_track, grad_weight,
                         workspace, workspace_bytes, stream);
}

extern "C" int sr_far_backward(const sr_tracks *t, const sr_grid *g, int comp,
                               const double *const *grad_out, const float *saved_A,
                               double *const *grad_track, double *grad_weight, void *workspace,
                               size_t workspace_bytes, void *stream) {
  clear_error();
  if (!grad_out) return fail(SR_ERR_INVALID, "grad_out must not be NULL");
  int rc = check_adjoint_args(t, g, (void *const *)grad_out, comp);
  if (rc) return rc;
  if (!saved_A || !grad_track || !grad_weight)
    return fail(SR_ERR_INVALID, "saved_A, grad_track and grad_weight must not be NULL");
  for (int i = 0; i < 6; ++i)
    if (!grad_track[i]) return fail(SR_ERR_INVALID, "grad_track[%d] is NULL", i);
  if (t->n_tracks == 0) return SR_OK;
  const uint64_t n_dirs = (uint64_t)g->n_theta * g->n_phi;
  const uint64_t P = n_dirs * g->n_omega;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e;
  if (P == 0) {  // no spectrum: every gradient is zero
    for (int i = 0; i < 6; ++i) {
      e = cudaMemsetAsync(grad_track[i], 0, (size_t)t->total_steps * 8, s);
      if (e != cudaSuccess) return cuda_fail(e, "gradient reset");
    }
    e = cudaMemsetAsync(grad_weight, 0, (size_t)t->n_tracks * 8, s);
    return e == cudaSuccess ? SR_OK : cuda_fail(e, "gradient reset");
  }
  const AdjLayout lay = adj_layout(t->total_steps, P, g->n_omega, n_dirs, t->n_tracks, t->n_snaps);
  if (!workspace || workspace_bytes < lay.total)
    return fail(SR_ERR_WORKSPACE, "workspace of %zu bytes needed, %zu given", lay.total,
                workspace_bytes);
  if (((uintptr_t)workspace & 255u) != 0)
    return fail(SR_ERR_WORKSPACE, "workspace not 256-byte aligned");
  unsigned char *w = (unsigned char *)workspace;

  AdjParams a;
  memset(&a, 0, sizeof(a));
  a.f = make_far_mixed_params(t, g, comp, (void *const *)grad_out);
  a.f.status = (int *)w;
  a.f.records = (float4 *)(w + lay.records);
  for (int i = 0; i < n_outputs(comp); ++i) a.grad_out[i] = grad_out[i];
  a.linear = (comp == SR_COMP_CARTESIAN_COMPLEX || comp == SR_COMP_SPHERIC_COMPLEX) ? 1 : 0;
  a.save_A = (const float4 *)saved_A;
  a.gcst = (float4 *)(w + lay.gcst);
  a.wtab = (float4 *)(w + lay.wtab);
  a.dirtab = (float4 *)(w + lay.dirtab);
  a.glob = (AdjGlobals *)(w + lay.glob);
  a.item_off = (int64_t *)(w + lay.item_off);
  a.gstep = (double *)(w + lay.gstep);
  for (int i = 0; i < 6; ++i) a.grad[i] = grad_track[i];
  a.grad_w = grad_weight;

  e = cudaMemsetAsync(w, 0, 256, s);
  if (e != cudaSuccess) return cuda_fail(e, "status reset");
  // steps that enter no snapshot (after the last one written) are not visited
  e = cudaMemsetAsync(a.gstep, 0, (size_t)t->total_steps * kAG * 8, s);
  if (e != cudaSuccess) return cuda_fail(e, "gradient reset");
  const int n_sm = device_sm_count();
  const int64_t step_blocks = std::max<int64_t>(
      1, std::min<int64_t>((t->total_steps + 255) / 256, (int64_t)n_sm * 128));
  if (t->total_steps > 0) launch_far_prepass(a.f, (int)step_blocks, s);
  adj_globals_kernel<<<1, 256, 0, s>>>(a.f, a.wtab, a.glob);
  {
    const uint64_t work = std::max<uint64_t>(P, n_dirs);
    const uint64_t nb = std::min<uint64_t>((work + 255) / 256, (uint64_t)n_sm * 64);
    adj_prep_kernel<<<(unsigned)nb, 256, 0, s>>>(a);
  }
  adj_items_kernel<<<1, 1024, 0, s>>>(a.f, a.item_off, (uint32_t)kASteps);
  {
    double *wpart = (double *)(w + lay.wpart);
    adj_weight_partial_far_kernel<<<t->n_tracks * lay.w_chunks, kWeightThreads, 0, s>>>(
        a, P, lay.w_chunks, wpart);
    adj_weight_final_far_kernel<<<(t->n_tracks + 255) / 256, 256, 0, s>>>(
        wpart, t->n_tracks, lay.w_chunks, a.linear, t->weight, grad_weight);
  }
  rc = cuda_fail(cudaGetLastError(), "adjoint prep launch");
  if (rc) return rc;
  const size_t smem = adj_smem_bytes();
  e = cudaFuncSetAttribute(adj_far_kernel<kAW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "adjoint smem attribute");
  // upper bound of the work items (sum over tracks of ceil(n_body / 256))
  const int64_t items_max = t->total_steps / kASteps + (int64_t)t->n_tracks;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(items_max, 2 * (int64_t)n_sm));
  void *tok = nullptr;
  timing_record(s, true, &tok);
  adj_far_kernel<kAW><<<grid, kAW * 32, smem, s>>>(a);
  timing_record(s, false, &tok);
  rc = cuda_fail(cudaGetLastError(), "adjoint kernel launch");
  if (rc) return rc;
  if (t->total_steps > 0) {
    if (a.f.track_f32)
      adj_final_kernel<float><<<(int)step_blocks, 256, 0, s>>>(a);
    else
      adj_final_kernel<double><<<(int)step_blocks, 256, 0, s>>>(a);
  }
  return cuda_fail(cudaGetLastError(), "adjoint final launch");
}
