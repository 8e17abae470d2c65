// Adjoint of the mixed-precision near field (every comp, one snapshot).
//
// Forward (sr_near_mixed.cu, the reference's synchrad/kernel_nearfield.cl:58-102):
//   S(p) = sum_t w_t dt^2 |A_t(p)|^2,   A = sum_s a_s e^{i phi_s},
//   a = n/r^2 + i omega (beta - n)/r,   phi = omega (t + r),
//   r = |P - x_s|, n = (P - x_s)/r, beta at step s.
// With g(p) = dL/dS(p), U = 2 g w dt^2 conj(A) and z = e^{i phi}:
//   dL/dw_t  = sum_p g dt^2 |A_t|^2,
//   dL/dbeta = -I1/r,
//   dL/dx    = (-R0 + 3 n (n.R0))/r^3 - (I1 + n ((beta-n).I1) - 2 n (n.I1))/r^2
//              + n ((beta-n).R2)/r,
// per step and screen point, with the omega sums (per component k)
//   R0_k = sum Re(U_k z),  I1_k = sum omega Im(U_k z),  R2_k = sum omega^2 Re(U_k z)
// (from d phi/dx = -omega n, dn/dx = -(I - n n^T)/r, dr/dx = -n), then
// dL/du = dL/dbeta / gamma - u (u . dL/dbeta) / gamma^3.  The comps differ in
// U_k only: total and cartesian (outputs w dt^2 |A_k|^2 summed or apart) give
// U_k = 2 g_k w dt^2 A_k (g_k = g for total); cartesian_complex (outputs sqrt(w)
// dt Re/Im(e^{i omega L} A_k)) gives U_k = sqrt(w) dt (g_k,re + i g_k,im)
// e^{-i omega L}; with dL = Re(conj(U) . dA), dL/dw = sum_p Re(conj(U) . A)/(2w).
// beta - n is formed
// as in the forward ((1 - n_z) - (1 - beta_z) along z).  The |dphase| < pi
// mask is held fixed (its decisions are the forward's).
//
// Layout as in the far-field adjoint (sr_far_adjoint.cu): a lane owns one
// step and walks a screen point's omega axis (rotation recurrence reseeded
// every 8 points, pairs of points in packed FP32), the U/W/Y constants of a
// block of (screen point, omega) slots are built in shared memory from the
// saved amplitudes, and a CTA owns 256 steps of one track and loops over
// every screen point, so each step's gradient is written once.
#include <algorithm>
#include <cmath>

#include "sr_common.cuh"
#include "sr_internal.h"
#include "sr_mixed_common.cuh"
#include "sr_adjoint_common.cuh"

namespace sr {
namespace {

constexpr int kNAW = 8;               // warps per CTA
constexpr int kNASteps = kNAW * 32;   // steps per work item (one per lane)
constexpr int kNAStage = 512;         // (screen point, omega) slots per constants stage
constexpr int kNARS = 8;              // omega slots per phasor reseed
constexpr int kNAG = 6;               // per-step gradient components: x (3), beta (3)
constexpr int kNARecS = kRecF4;       // record stride in shared memory (80 bytes, as in HBM)
constexpr int kNAPair = 11;           // float4 per pair of slots in the constants

struct NearAdjParams {
  FarMixedParams f;            // tracks, grid (n_theta = radii), records, status
  const double *grad_out[6];   // [P] dL/dS_k per output of the comp, device layout
  int linear;                  // cartesian_complex: U does not depend on A
  const float4 *save_A;        // [n_tracks][P][2] (A_x re, im, A_y re, im), (A_z re, im, 0, 0)
  float4 *gcst;                // [P][2] point sensitivity in FP32: quadratic comps
                               // (2 dt^2 g_x, g_y, g_z, 0), 0; linear (V_x re, im,
                               // V_y re, im), (V_z re, im, 0, 0)
  float4 *wtab;                // [nO] (omega/2pi hi, lo, omega, |omega|) in FP32
  float4 *sctab;               // [n_screen] (X hi, lo, Y hi, lo) of the screen point
  AdjGlobals *glob;
  int64_t *item_off;           // [n_tracks + 1] first work item of each track
  double *gstep;               // [total_steps][kNAG] per-step gradients (x, beta)
  double *grad[6];             // x, y, z, ux, uy, uz  [total_steps]
  double *grad_w;              // [n_tracks]
};

// Point sensitivity (FP64) of the loss to (A_x, A_y, A_z) at point gi for the
// output gradients g_k: quadratic comps 2 dt^2 (g_x, g_y, g_z) in v[0..2];
// cartesian_complex V_k = dt (g_k,re + i g_k,im) e^{-i omega L} in v[0..5].
__device__ __forceinline__ void near_point_sens(const NearAdjParams &a, uint32_t ksnap,
                                                uint64_t gi, double v[6]) {
  const FarMixedParams &p = a.f;
  const double s2 = 2.0 * p.dt * p.dt;
  const uint64_t gk = (uint64_t)ksnap * p.n_omega * p.n_theta * p.n_phi + gi;  // snapshot slot
  for (int k = 0; k < 6; ++k) v[k] = 0.0;
  if (p.comp == SR_COMP_TOTAL) {
    v[0] = v[1] = v[2] = s2 * a.grad_out[0][gk];
  } else if (p.comp == SR_COMP_CARTESIAN) {
    for (int k = 0; k < 3; ++k) v[k] = s2 * a.grad_out[k][gk];
  } else {  // cartesian_complex (FormFactor not applied, as the reference)
    const double w = p.omega[gi % p.n_omega];
    double sL, cL;
    sincos(w * p.L_screen, &sL, &cL);
    for (int k = 0; k < 3; ++k) {
      const double gr = a.grad_out[2 * k][gk], gim = a.grad_out[2 * k + 1][gk];
      v[2 * k] = p.dt * (gr * cL + gim * sL);
      v[2 * k + 1] = p.dt * (gim * cL - gr * sL);
    }
  }
}

// dL/dw_t = sum_p Re(conj(U) . A_t) / (2 w_t): chunk sums in FP64 from the
// FP64 point sensitivities, then one thread per track adds its chunks.
__global__ void nadj_weight_partial_kernel(NearAdjParams a, uint64_t P, uint32_t n_chunks,
                                           double *wpart) {
  const uint32_t t = blockIdx.x / n_chunks, b = blockIdx.x % n_chunks;
  const uint64_t chunk = (P + n_chunks - 1) / n_chunks;
  const uint64_t g0 = (uint64_t)b * chunk, g1 = min(P, g0 + chunk);
  double acc = 0.0;
  for (uint64_t g = g0 + threadIdx.x; g < g1; g += blockDim.x) {
    for (uint32_t ks = 0; ks < a.f.n_snaps; ++ks) {  // a snapshot that never fired has A = 0
      double v[6];
      near_point_sens(a, ks, g, v);
      const uint64_t ia = 2 * (((uint64_t)t * a.f.n_snaps + ks) * P + g);
      const float4 A0 = a.save_A[ia], A1 = a.save_A[ia + 1];
      const double re[3] = {A0.x, A0.z, A1.x}, im[3] = {A0.y, A0.w, A1.y};
      for (int k = 0; k < 3; ++k)
        acc += a.linear ? v[2 * k] * re[k] + v[2 * k + 1] * im[k]
                        : v[k] * (re[k] * re[k] + im[k] * im[k]);
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

__global__ void nadj_weight_final_kernel(const double *wpart, uint32_t n_tracks,
                                         uint32_t n_chunks, int linear, const double *weight,
                                         double *grad_w) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n_tracks) return;
  double s = 0.0;
  for (uint32_t b = 0; b < n_chunks; ++b) s += wpart[(uint64_t)t * n_chunks + b];
  grad_w[t] = linear ? (weight[t] > 0.0 ? s / (2.0 * sqrt(weight[t])) : 0.0) : 0.5 * s;
}

// Point sensitivities in FP32 and the screen table.
__global__ void nadj_prep_kernel(NearAdjParams a) {
  const FarMixedParams &p = a.f;
  const uint32_t nR = p.n_theta;
  const uint64_t n_scr = (uint64_t)nR * p.n_phi;
  const uint64_t P = n_scr * p.n_omega;
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < P * p.n_snaps;
       i += stride) {
    double v[6];
    near_point_sens(a, (uint32_t)(i / P), i % P, v);
    a.gcst[2 * i] = make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]);
    a.gcst[2 * i + 1] = make_float4((float)v[4], (float)v[5], 0.f, 0.f);
  }
  for (uint64_t d = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; d < n_scr; d += stride) {
    const uint32_t iR = (uint32_t)(d % nR), iP = (uint32_t)(d / nR);
    const df X = df_from_double(p.sin_theta[iR] * p.cos_phi[iP]);  // radius * cos(phi)
    const df Y = df_from_double(p.sin_theta[iR] * p.sin_phi[iP]);  // radius * sin(phi)
    a.sctab[d] = make_float4(X.hi, X.lo, Y.hi, Y.lo);
  }
}

// dL/du_s from dL/dbeta_s (beta = u / gamma at the same step).
template <typename TT>
__global__ void nadj_final_kernel(NearAdjParams a) {
  const FarMixedParams &p = a.f;
  const TT *UX = (const TT *)p.ux, *UY = (const TT *)p.uy, *UZ = (const TT *)p.uz;
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < p.total_steps;
       g += (int64_t)gridDim.x * blockDim.x) {
    uint32_t lo = 0, hi = p.n_tracks;
    while (hi - lo > 1) {
      const uint32_t mid = (lo + hi) >> 1;
      if (p.offsets[mid] <= g) lo = mid; else hi = mid;
    }
    const uint32_t t = lo;
    const int64_t s = g - p.offsets[t];
    double v[kNAG] = {0, 0, 0, 0, 0, 0};
    if (s < (int64_t)track_body(p, t))
      for (int c = 0; c < kNAG; ++c) v[c] = a.gstep[g * kNAG + c];
    a.grad[0][g] = v[0];
    a.grad[1][g] = v[1];
    a.grad[2][g] = v[2];
    const double ux = (double)UX[g], uy = (double)UY[g], uz = (double)UZ[g];
    const double gam = sqrt(1.0 + (ux * ux + uy * uy + uz * uz));
    const double ug = (ux * v[3] + uy * v[4] + uz * v[5]) / (gam * gam * gam);
    a.grad[3][g] = v[3] / gam - ux * ug;
    a.grad[4][g] = v[4] / gam - uy * ug;
    a.grad[5][g] = v[5] / gam - uz * ug;
  }
}

// Shared memory of one CTA.  Constants per pair of omega slots (m, m+1) of a
// screen point whose omega axis is padded to a multiple of kNARS slots:
//   [0..2] U_k (G Re A_k m, m+1, G Im A_k m, m+1)          k = x, y, z
//   [3..5] W_k (omega G Re A_k ..., -omega G Im A_k ...)
//   [6..8] Y_k (omega^2 G Re A_k ..., omega^2 G Im A_k ...)
//   [9]  (omega/2pi hi, lo of m, of m+1)    [10] (|omega| of m, m+1, 0, 0)
struct NearAdjSmem {
  float4 rec[kNASteps + 1][kNARecS];
  float4 cst[kNAStage / 2][kNAPair];
  uint64_t bar;
  uint64_t pad_;
};

__device__ __forceinline__ float2 lo2(const float4 &v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(const float4 &v) { return make_float2(v.z, v.w); }

// R0 += Re(U z), I1 += omega Im(U z), R2 += omega^2 Re(U z), per component,
// for a pair of points.
struct NearSums {
  float2 r0[3], i1[3], r2[3];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int k = 0; k < 3; ++k) r0[k] = i1[k] = r2[k] = make_float2(0.f, 0.f);
  }
  __device__ __forceinline__ void add(const float4 *c, float2 zr, float2 zi) {
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      const float4 u = c[k], w = c[3 + k], y = c[6 + k];
      r0[k] = __ffma2_rn(lo2(u), zr, r0[k]);
      r0[k] = __ffma2_rn(hi2(u), zi, r0[k]);
      i1[k] = __ffma2_rn(lo2(w), zi, i1[k]);
      i1[k] = __ffma2_rn(hi2(w), zr, i1[k]);
      r2[k] = __ffma2_rn(lo2(y), zr, r2[k]);
      r2[k] = __ffma2_rn(hi2(y), zi, r2[k]);
    }
  }
};

// Geometry of one step and screen point from the step record: the retarded
// time tau' = t + r - L = (t - z) + rho^2/(r + L - z) (double-float), the
// distance r and n (FP32), and 1 - n_z.
struct NearGeo {
  df tau;
  float r, nx, ny, nz, omn;
};

__device__ __forceinline__ NearGeo near_geo(const float4 *rec, const float4 &sc, const df &dL) {
  const float4 r0 = rec[0], r1 = rec[1];
  const df ddx = df_sub(df{sc.x, sc.y}, df{r0.z, r0.w});
  const df ddy = df_sub(df{sc.z, sc.w}, df{r1.x, r1.y});
  const df D = df_sub(dL, df{r1.z, r1.w});
  const df rho2 = df_add(df_mul(ddx, ddx), df_mul(ddy, ddy));
  const df r = df_sqrt(df_add(rho2, df_mul(D, D)));
  const df F = (D.hi > 0.f) ? df_div(rho2, df_add(r, D)) : df_sub(r, D);
  NearGeo g;
  g.tau = df_add(df{r0.x, r0.y}, F);
  g.r = r.hi + r.lo;
  const float rinv = __frcp_rn(g.r);
  g.nx = (ddx.hi + ddx.lo) * rinv;
  g.ny = (ddy.hi + ddy.lo) * rinv;
  g.nz = (D.hi + D.lo) * rinv;
  g.omn = (F.hi + F.lo) * rinv;
  return g;
}

template <int W>
__global__ void __launch_bounds__(W * 32, 2) nadj_kernel(NearAdjParams a) {
  const FarMixedParams &p = a.f;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  NearAdjSmem &sm = *reinterpret_cast<NearAdjSmem *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t ls = (uint32_t)(warp * 32 + lane);  // this lane's step within the item
  if (threadIdx.x == 0) {
    mbar_init(&sm.bar, 1);
    fence_mbar_init();
  }
  __syncthreads();

  const AdjGlobals G = *a.glob;
  const uint32_t nO = p.n_omega, nR = p.n_theta;
  const uint32_t nOp = (nO + kNARS - 1) / kNARS * kNARS;  // padded omega slots per point
  const uint64_t P = (uint64_t)nO * nR * p.n_phi;
  const uint64_t Pp = (uint64_t)nOp * nR * p.n_phi;
  const int64_t n_items = a.item_off[p.n_tracks];
  const df d_dw = df{G.dw_h, G.dw_l};
  const df dL = df_from_double(p.L_screen);
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
    track_segments(p, t, (uint32_t)kNASteps, (uint32_t)(item - a.item_off[t]), &seg);
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
    double gD[kNAG];
#pragma unroll
    for (int c = 0; c < kNAG; ++c) gD[c] = 0.0;

    // per (screen point, step) state, kept across constants stages
    float th = 0.f, tl = 0.f, rc = 1.f, rs = 0.f, adt = 0.f;
    float gr = 1.f, gnx = 0.f, gny = 0.f, gnz = 1.f, gomn = 0.f;
    float2 r2c = make_float2(1.f, 1.f), r2s = make_float2(0.f, 0.f), nr2s = r2s;
    int mode = 1;  // 0: every omega included, 1: none, 2: per point
    NearSums ns;
    ns.zero();

    for (uint64_t f0 = 0; f0 < Pp; f0 += kNAStage) {
      const uint32_t nf =
          (Pp - f0 < (uint64_t)kNAStage) ? (uint32_t)(Pp - f0) : (uint32_t)kNAStage;
      __syncthreads();  // the previous stage's constants are no longer read
      for (uint32_t j = threadIdx.x; j < nf / 2; j += blockDim.x) {
        const uint64_t f = f0 + 2 * j;
        const uint64_t dj = f / nOp;
        const uint32_t m = (uint32_t)(f - dj * nOp);
        float ar[2][3], ai[2][3], om[2];
        float4 wv[2];
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          if (m + e < nO) {
            const uint64_t gi = dj * nO + m + e;
#pragma unroll
            for (int k = 0; k < 3; ++k) ar[e][k] = ai[e][k] = 0.f;
            // U summed over the snapshots these steps enter
            for (uint32_t ks = seg.k0; ks <= seg.k1; ++ks) {
              const uint64_t ic = 2 * ((uint64_t)ks * P + gi);
              const float4 C0 = a.gcst[ic], C1 = a.gcst[ic + 1];
              if (a.linear) {  // U_k = sqrt(w) V_k
                ar[e][0] += swt * C0.x; ai[e][0] += swt * C0.y;
                ar[e][1] += swt * C0.z; ai[e][1] += swt * C0.w;
                ar[e][2] += swt * C1.x; ai[e][2] += swt * C1.y;
              } else {         // U_k = w g'_k A_k
                const uint64_t ia = 2 * (((uint64_t)t * p.n_snaps + ks) * P + gi);
                const float4 A0 = a.save_A[ia], A1 = a.save_A[ia + 1];
                ar[e][0] += wt * C0.x * A0.x; ai[e][0] += wt * C0.x * A0.y;
                ar[e][1] += wt * C0.y * A0.z; ai[e][1] += wt * C0.y * A0.w;
                ar[e][2] += wt * C0.z * A1.x; ai[e][2] += wt * C0.z * A1.y;
              }
            }
            wv[e] = a.wtab[m + e];
          } else {
#pragma unroll
            for (int k = 0; k < 3; ++k) ar[e][k] = ai[e][k] = 0.f;
            wv[e] = make_float4(0.f, 0.f, 0.f, 0.f);
          }
          om[e] = wv[e].z;
        }
        float4 *o = sm.cst[j];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
          const float u0r = ar[0][k], u1r = ar[1][k];
          const float u0i = ai[0][k], u1i = ai[1][k];
          o[k] = make_float4(u0r, u1r, u0i, u1i);
          o[3 + k] = make_float4(om[0] * u0r, om[1] * u1r, -om[0] * u0i, -om[1] * u1i);
          o[6 + k] = make_float4(om[0] * om[0] * u0r, om[1] * om[1] * u1r, om[0] * om[0] * u0i,
                                 om[1] * om[1] * u1i);
        }
        o[9] = make_float4(wv[0].x, wv[0].y, wv[1].x, wv[1].y);
        o[10] = make_float4(wv[0].w, wv[1].w, 0.f, 0.f);
      }
      __syncthreads();
      float gF[kNAG];
#pragma unroll
      for (int c = 0; c < kNAG; ++c) gF[c] = 0.f;

      uint32_t d = (uint32_t)(f0 / nOp);
      for (uint64_t fd = (uint64_t)d * nOp; fd < f0 + nf; fd += nOp, ++d) {
        const uint32_t m_lo = (uint32_t)(max(fd, f0) - fd);
        const uint32_t m_hi = (uint32_t)(min(fd + nOp, f0 + nf) - fd);
        // slot m of screen point d sits at stage index fd + m - f0 >= 0 for m >= m_lo
        const int64_t seg = (int64_t)fd - (int64_t)f0;
        if (m_lo == 0) {  // a new screen point: phase, rotation and mask of step s
          const float4 sc = a.sctab[d];
          const NearGeo gs = near_geo(sm.rec[si], sc, dL);
          // the track's first step compares the whole phase omega (t + r) with zero
          float dtau = (gs.tau.hi + gs.tau.lo) + (dL.hi + dL.lo);
          if (!first) {
            const NearGeo gp = near_geo(sm.rec[si - 1], sc, dL);
            dtau = (gs.tau.hi - gp.tau.hi) + (gs.tau.lo - gp.tau.lo);
          }
          th = gs.tau.hi;
          tl = gs.tau.lo;
          gr = gs.r;
          gnx = gs.nx;
          gny = gs.ny;
          gnz = gs.nz;
          gomn = gs.omn;
          adt = fabsf(dtau);
          mode = (!valid || G.wabs_min * adt > kPiHi) ? 1 : (G.wabs_max * adt < kPiLo ? 0 : 2);
          const df rp = df_mul_raw(d_dw, gs.tau);
          sincosf(reduce_2pi(rp.hi, rp.lo), &rs, &rc);
          float c2r, s2r;
          cmul(rc, rs, rc, rs, c2r, s2r);
          r2c = make_float2(c2r, c2r);
          r2s = make_float2(s2r, s2r);
          nr2s = make_float2(-s2r, -s2r);
          ns.zero();
        }
        if (!__all_sync(0xffffffffu, mode == 1)) {
          if (G.uniform && __all_sync(0xffffffffu, mode != 2)) {
            // every point included (lanes with mode 1 are discarded below)
#pragma unroll 1
            for (uint32_t m = m_lo; m < m_hi; m += kNARS) {
              const float4 *cp = sm.cst[(seg + (int64_t)m) >> 1];
              float zs, zc;
              phasor_rev(cp[9].x, cp[9].y, th, tl, zs, zc);
              float2 zr = make_float2(zc, zc * rc - zs * rs);
              float2 zi = make_float2(zs, zc * rs + zs * rc);
#pragma unroll
              for (int q = 0; q < kNARS / 2; ++q) {
                ns.add(cp + kNAPair * q, zr, zi);
                if (q + 1 < kNARS / 2) rot2p(zr, zi, r2c, r2s, nr2s, zr, zi);
              }
            }
          } else {
            // per-point mask (and one reseed per point on a non-uniform axis)
            double P0 = 0.0, P1 = 0.0;
            bool have_p = false;
#pragma unroll 1
            for (uint32_t m = m_lo; m < m_hi; m += kNARS) {
              const float4 *cp = sm.cst[(seg + (int64_t)m) >> 1];
              float2 zr, zi;
              {
                float zs, zc;
                phasor_rev(cp[9].x, cp[9].y, th, tl, zs, zc);
                zr = make_float2(zc, zc * rc - zs * rs);
                zi = make_float2(zs, zc * rs + zs * rc);
              }
#pragma unroll 1
              for (int q = 0; q < kNARS / 2; ++q) {
                const float4 *c = cp + kNAPair * q;
                if (!G.uniform) {
                  float zs, zc;
                  phasor_rev(c[9].x, c[9].y, th, tl, zs, zc);
                  zr.x = zc;
                  zi.x = zs;
                  phasor_rev(c[9].z, c[9].w, th, tl, zs, zc);
                  zr.y = zc;
                  zi.y = zs;
                }
                const float4 aw = c[10];
                bool inc[2] = {aw.x * adt < kPiLo, aw.y * adt < kPiLo};
                if (mode == 2) {
#pragma unroll
                  for (int e = 0; e < 2; ++e) {
                    const float ph = (e ? aw.y : aw.x) * adt;
                    const uint32_t mm = m + 2 * q + e;
                    if (!inc[e] && !(ph > kPiHi) && mm < nO) {
                      if (!have_p) {
                        const uint32_t iR = d % nR, iP = d / nR;
                        P0 = p.sin_theta[iR] * p.cos_phi[iP];
                        P1 = p.sin_theta[iR] * p.sin_phi[iP];
                        have_p = true;
                      }
                      inc[e] = exact_mask_near(p, base, s, it_start, p.omega[mm], P0, P1);
                    }
                  }
                }
                const float2 gm = make_float2(inc[0] ? 1.f : 0.f, inc[1] ? 1.f : 0.f);
                ns.add(c, __fmul2_rn(zr, gm), __fmul2_rn(zi, gm));
                if (G.uniform) rot2p(zr, zi, r2c, r2s, nr2s, zr, zi);
              }
            }
          }
        }
        if (m_hi == nOp && mode != 1) {  // the screen point is complete: chain rule
          const float4 q2 = sm.rec[si][2];  // (beta_x, beta_y, beta_z, 1 - beta_z)
          float R0[3], I1[3], R2[3];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            R0[k] = ns.r0[k].x + ns.r0[k].y;
            I1[k] = ns.i1[k].x + ns.i1[k].y;
            R2[k] = ns.r2[k].x + ns.r2[k].y;
          }
          const float n[3] = {gnx, gny, gnz};
          const float bmn[3] = {q2.x - gnx, q2.y - gny, gomn - q2.w};  // beta - n
          const float ir = __frcp_rn(gr);
          const float ir2 = ir * ir, ir3 = ir2 * ir;
          const float nR0 = n[0] * R0[0] + n[1] * R0[1] + n[2] * R0[2];
          const float nI1 = n[0] * I1[0] + n[1] * I1[1] + n[2] * I1[2];
          const float bI1 = bmn[0] * I1[0] + bmn[1] * I1[1] + bmn[2] * I1[2];
          const float bR2 = bmn[0] * R2[0] + bmn[1] * R2[1] + bmn[2] * R2[2];
#pragma unroll
          for (int k = 0; k < 3; ++k) {
            gF[k] += (3.f * n[k] * nR0 - R0[k]) * ir3 -
                     (I1[k] + n[k] * bI1 - 2.f * n[k] * nI1) * ir2 + n[k] * bR2 * ir;
            gF[3 + k] -= I1[k] * ir;
          }
        }
      }
#pragma unroll
      for (int c = 0; c < kNAG; ++c) gD[c] += (double)gF[c];
    }
    if (valid) {
#pragma unroll
      for (int c = 0; c < kNAG; ++c) a.gstep[(uint64_t)(base + s) * kNAG + c] = gD[c];
    }
    __syncthreads();  // records of this item no longer read
  }
}

size_t nadj_smem_bytes() { return sizeof(NearAdjSmem); }

struct NearAdjLayout {
  size_t records, gcst, wtab, sctab, glob, item_off, gstep, wpart, total;
  uint32_t w_chunks;
};

NearAdjLayout nadj_layout(int64_t total_steps, uint64_t P, uint32_t n_omega, uint64_t n_scr,
                          uint32_t n_tracks, uint32_t n_snaps) {
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  NearAdjLayout l;
  l.w_chunks = adj_weight_chunks(P, n_tracks, device_sm_count());
  l.records = 256;
  l.gcst = l.records + up((size_t)total_steps * kRecBytes);
  l.wtab = l.gcst + up((size_t)P * 32 * (n_snaps ? n_snaps : 1));
  l.sctab = l.wtab + up((size_t)n_omega * 16);
  l.glob = l.sctab + up((size_t)n_scr * 16);
  l.item_off = l.glob + 256;
  l.gstep = l.item_off + up(((size_t)n_tracks + 1) * 8);
  l.wpart = l.gstep + up((size_t)total_steps * kNAG * 8);
  l.total = l.wpart + up((size_t)n_tracks * l.w_chunks * 8);
  return l;
}

int check_near_adjoint_args(const sr_tracks *t, const sr_grid *g, void *const *out,
                            int comp = SR_COMP_TOTAL) {
  int rc = validate_spectrum_args(t, g, comp, SR_PREC_MIXED, out);
  if (rc) return rc;
  if (g->mode != SR_MODE_NEAR) return fail(SR_ERR_UNSUPPORTED, "near-field adjoint: mode near");
  if (t->n_snaps < 1)
    return fail(SR_ERR_UNSUPPORTED, "the adjoint needs at least one snapshot (n_snaps >= 1)");
  return SR_OK;
}

}  // namespace
}  // namespace sr

using namespace sr;

extern "C" int sr_near_forward_saved(const sr_tracks *t, const sr_grid *g, int comp,
                                     void *const *out, float *saved_A, void *workspace,
                                     size_t workspace_bytes, void *stream) {
  clear_error();
  int rc = check_near_adjoint_args(t, g, out, comp);
  if (rc) return rc;
  if (!saved_A) return fail(SR_ERR_INVALID, "saved_A is NULL");
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  if (P == 0 || t->n_tracks == 0) return SR_OK;
  cudaStream_t s = (cudaStream_t)stream;
  cudaError_t e = cudaMemsetAsync(saved_A, 0, (size_t)t->n_tracks * t->n_snaps * P * 32, s);
  if (e != cudaSuccess) return cuda_fail(e, "saved_A reset");
  FarMixedParams p = make_far_mixed_params(t, g, comp, out);
  p.save_A = saved_A;
  return launch_near_mixed(p, mixed_config(t, g, comp), workspace, workspace_bytes, s);
}

extern "C" int sr_near_total_forward_saved(const sr_tracks *t, const sr_grid *g, double *spectrum,
                                           float *saved_A, void *workspace,
                                           size_t workspace_bytes, void *stream) {
  void *out[6] = {spectrum};
  return sr_near_forward_saved(t, g, SR_COMP_TOTAL, out, saved_A, workspace, workspace_bytes,
                               stream);
}

extern "C" int64_t sr_near_total_backward_workspace_bytes(const sr_tracks *t, const sr_grid *g) {
  return sr_near_backward_workspace_bytes(t, g);
}

extern "C" int64_t sr_near_backward_workspace_bytes(const sr_tracks *t, const sr_grid *g) {
  if (!t || !g) return -1;
  const uint64_t n_scr = (uint64_t)g->n_theta * g->n_phi;
  return (int64_t)nadj_layout(t->total_steps, n_scr * g->n_omega, g->n_omega, n_scr,
                              t->n_tracks, t->n_snaps)
      .total;
}

extern "C" int sr_near_total_backward(const sr_tracks *t, const sr_grid *g,
                                      const double *grad_spectrum, const float *saved_A,
                                      double *const *grad_track, double *grad_weight,
                                      void *workspace, size_t workspace_bytes, void *stream) {
  const double *grad_out[6] = {grad_spectrum};
  return sr_near_backward(t, g, SR_COMP_TOTAL, grad_out, saved_A, grad_track, grad_weight,
                          workspace, workspace_bytes, stream);
}

extern "C" int sr_near_backward(const sr_tracks *t, const sr_grid *g, int comp,
                                const double *const *grad_out, const float *saved_A,
                                double *const *grad_track, double *grad_weight, void *workspace,
                                size_t workspace_bytes, void *stream) {
  clear_error();
  if (!grad_out) return fail(SR_ERR_INVALID, "grad_out must not be NULL");
  int rc = check_near_adjoint_args(t, g, (void *const *)grad_out, comp);
  if (rc) return rc;
  if (!saved_A || !grad_track || !grad_weight)
    return fail(SR_ERR_INVALID, "saved_A, grad_track and grad_weight must not be NULL");
  for (int i = 0; i < 6; ++i)
    if (!grad_track[i]) return fail(SR_ERR_INVALID, "grad_track[%d] is NULL", i);
  if (t->n_tracks == 0) return SR_OK;
  const uint64_t n_scr = (uint64_t)g->n_theta * g->n_phi;
  const uint64_t P = n_scr * g->n_omega;
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
  const NearAdjLayout lay =
      nadj_layout(t->total_steps, P, g->n_omega, n_scr, t->n_tracks, t->n_snaps);
  if (!workspace || workspace_bytes < lay.total)
    return fail(SR_ERR_WORKSPACE, "workspace of %zu bytes needed, %zu given", lay.total,
                workspace_bytes);
  if (((uintptr_t)workspace & 255u) != 0)
    return fail(SR_ERR_WORKSPACE, "workspace not 256-byte aligned");
  unsigned char *w = (unsigned char *)workspace;

  NearAdjParams a;
  memset(&a, 0, sizeof(a));
  a.f = make_far_mixed_params(t, g, comp, (void *const *)grad_out);
  a.f.status = (int *)w;
  a.f.records = (float4 *)(w + lay.records);
  for (int i = 0; i < n_outputs(comp); ++i) a.grad_out[i] = grad_out[i];
  a.linear = comp == SR_COMP_CARTESIAN_COMPLEX ? 1 : 0;
  a.save_A = (const float4 *)saved_A;
  a.gcst = (float4 *)(w + lay.gcst);
  a.wtab = (float4 *)(w + lay.wtab);
  a.sctab = (float4 *)(w + lay.sctab);
  a.glob = (AdjGlobals *)(w + lay.glob);
  a.item_off = (int64_t *)(w + lay.item_off);
  a.gstep = (double *)(w + lay.gstep);
  for (int i = 0; i < 6; ++i) a.grad[i] = grad_track[i];
  a.grad_w = grad_weight;

  e = cudaMemsetAsync(w, 0, 256, s);
  if (e != cudaSuccess) return cuda_fail(e, "status reset");
  // steps that enter no snapshot (after the last one written) are not visited
  e = cudaMemsetAsync(a.gstep, 0, (size_t)t->total_steps * kNAG * 8, s);
  if (e != cudaSuccess) return cuda_fail(e, "gradient reset");
  const int n_sm = device_sm_count();
  const int64_t step_blocks = std::max<int64_t>(
      1, std::min<int64_t>((t->total_steps + 255) / 256, (int64_t)n_sm * 128));
  if (t->total_steps > 0) launch_near_prepass(a.f, (int)step_blocks, s);
  adj_globals_kernel<<<1, 256, 0, s>>>(a.f, a.wtab, a.glob);
  {
    const uint64_t work = std::max<uint64_t>(P, n_scr);
    const uint64_t nb = std::min<uint64_t>((work + 255) / 256, (uint64_t)n_sm * 64);
    nadj_prep_kernel<<<(unsigned)nb, 256, 0, s>>>(a);
  }
  adj_items_kernel<<<1, 1024, 0, s>>>(a.f, a.item_off, (uint32_t)kNASteps);
  {
    double *wpart = (double *)(w + lay.wpart);
    nadj_weight_partial_kernel<<<t->n_tracks * lay.w_chunks, kWeightThreads, 0, s>>>(
        a, P, lay.w_chunks, wpart);
    nadj_weight_final_kernel<<<(t->n_tracks + 255) / 256, 256, 0, s>>>(
        wpart, t->n_tracks, lay.w_chunks, a.linear, t->weight, grad_weight);
  }
  rc = cuda_fail(cudaGetLastError(), "near adjoint prep launch");
  if (rc) return rc;
  const size_t smem = nadj_smem_bytes();
  e = cudaFuncSetAttribute(nadj_kernel<kNAW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "near adjoint smem attribute");
  const int64_t items_max = t->total_steps / kNASteps + (int64_t)t->n_tracks;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(items_max, 2 * (int64_t)n_sm));
  void *tok = nullptr;
  timing_record(s, true, &tok);
  nadj_kernel<kNAW><<<grid, kNAW * 32, smem, s>>>(a);
  timing_record(s, false, &tok);
  rc = cuda_fail(cudaGetLastError(), "near adjoint kernel launch");
  if (rc) return rc;
  if (t->total_steps > 0) {
    if (a.f.track_f32)
      nadj_final_kernel<float><<<(int)step_blocks, 256, 0, s>>>(a);
    else
      nadj_final_kernel<double><<<(int)step_blocks, 256, 0, s>>>(a);
  }
  return cuda_fail(cudaGetLastError(), "near adjoint final launch");
}
