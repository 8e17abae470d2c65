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
//    rotation recurrence z_{j+1} = z_j R, R = exp(i domega tau), with an exact
//    double-float reseed of the first point at every step; two points are
//    advanced at once with packed FFMA2/FMUL2.
//  * the |dphase| < pi mask is decided per step from |omega| |dtau| with a
//    guard band; inside the band the reference's FP64 expression is evaluated
//    bit for bit from the original track data.
//  * sums are FP32 inside a TMA stage of steps and folded into compensated
//    (Knuth TwoSum) FP32 pairs in shared memory; per-track results are formed
//    and accumulated in FP64.
//
// Work decomposition: a warp owns one direction and an omega tile of 32*K
// points (lane l: points tile*32K + l*K .. +K-1); a CTA of W warps owns W
// consecutive warp tasks and loops over a contiguous subset of the tracks.
// Track records are streamed through shared memory by 1-D bulk TMA copies
// (cp.async.bulk + mbarrier, double buffered) and reused by every warp.  Each
// (task group, track subset) item writes its own partial spectrum; a final
// kernel adds the subsets in fixed order, so results are deterministic.
#include <cmath>

#include "sr_common.cuh"
#include "sr_internal.h"

namespace sr {
namespace {

constexpr int kStage = 128;         // steps per TMA stage
constexpr int kRecF4 = 4;           // float4 per step record (64 bytes)
constexpr float kPiLo = 3.14159265358979f * (1.0f - 4e-6f);
constexpr float kPiHi = 3.14159265358979f * (1.0f + 4e-6f);

// ------------------------------------------------------------------------
// Pre-pass: per-step records in FP64, stored as floats / double-floats.
//   r0 = (q.hi, q.lo, x.hi, x.lo)   q = t - z, t = (itStart + s) dt
//   r1 = (y.hi, y.lo, z.hi, z.lo)
//   r2 = (bbar_x, bbar_y, bbar_z, 1 - bbar_z)
//   r3 = (a_x, a_y, a_z, 0)
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
      rec[0] = zero; rec[1] = zero; rec[2] = zero; rec[3] = zero;
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
  }
}

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

template <int K, int W>
struct Smem {
  float4 stage[2][kStage * kRecF4];    // 2 x 8 KB
  uint64_t bar[2];
  uint64_t pad_[2];
  float4 setup[W][32][3];              // per-step broadcast values
  float kahan[W][K][8][32];            // (sum, comp) x (th re, th im, ph re, ph im)
  float2 omega_df[W][32 * K];          // omega table for non-uniform lanes
};

template <int K, int W>
__global__ void __launch_bounds__(W * 32, 1) far_mixed_kernel(FarMixedParams p) {
  static_assert(K % 2 == 0 && K >= 2 && K <= 16, "K");
  extern __shared__ __align__(128) unsigned char smem_raw[];
  Smem<K, W> &sm = *reinterpret_cast<Smem<K, W> *>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int KP = K / 2;

  if (threadIdx.x == 0) {
    mbar_init(&sm.bar[0], 1);
    mbar_init(&sm.bar[1], 1);
    fence_mbar_init();
  }
  __syncthreads();

  const uint32_t nO = p.n_omega, nT = p.n_theta;
  const uint32_t n_dirs = nT * p.n_phi;
  const uint64_t P = (uint64_t)nO * n_dirs;
  const uint32_t n_wt = n_dirs * p.n_wtiles;
  const double dw_glob = (nO > 1) ? (p.omega[nO - 1] - p.omega[0]) / (double)(nO - 1) : 0.0;
  const df d_dw = df_from_double(dw_glob);

  uint32_t stage_no = 0;  // running stage counter (mbarrier phase bookkeeping)
  bool pending = false;   // a copy for stage_no is in flight

  for (uint32_t item = blockIdx.x; item < p.n_items; item += gridDim.x) {
    const uint32_t sub = item / p.n_groups, grp = item % p.n_groups;
    const uint32_t wt = grp * W + warp;
    const bool active = wt < n_wt;
    const uint32_t dir = active ? wt / p.n_wtiles : 0u;
    const uint32_t tile = active ? wt % p.n_wtiles : 0u;
    const uint32_t iT = dir % nT, iP = dir / nT;
    const int j0 = (int)(tile * 32u * K) + lane * K;
    const int nv = active ? max(0, min(K, (int)nO - j0)) : 0;

    // Direction constants: n = (sinT cosP, sinT sinP, cosT) as the reference
    // rounds them, theta-hat, phi-hat.
    const double sT = p.sin_theta[iT], cT = p.cos_theta[iT];
    const double sPh = p.sin_phi[iP], cPh = p.cos_phi[iP];
    const double n0d = sT * cPh, n1d = sT * sPh, n2d = cT;
    const df d_c = df_from_double(1.0 - cT), d_sx = df_from_double(n0d),
             d_sy = df_from_double(n1d);
    const float f_c = (float)(1.0 - cT), f_sx = (float)n0d, f_sy = (float)n1d,
                f_cz = (float)cT;
    const float thx = (float)(cT * cPh), thy = (float)(cT * sPh), thz = (float)(-sT);
    const float phx = (float)(-sPh), phy = (float)cPh;

    // Lane omega constants and uniformity of its chunk.
    const double w0d = nv > 0 ? p.omega[j0] : 0.0;
    const df d_w0 = df_from_double(w0d);
    bool uniform = true;
    float wabs_min = 3.0e38f, wabs_max = 0.f;
    for (int m = 0; m < K; ++m) {
      if (m < nv) {
        const double wm = p.omega[j0 + m];
        const double pred = w0d + (double)m * dw_glob;
        if (fabs(wm - pred) > 1e-12 * fabs(wm) + 1e-300) uniform = false;
        const float a = (float)fabs(wm);
        wabs_min = fminf(wabs_min, a);
        wabs_max = fmaxf(wabs_max, a);
        const df dm = df_from_double(wm);
        sm.omega_df[warp][lane * K + m] = make_float2(dm.hi, dm.lo);
      } else {
        sm.omega_df[warp][lane * K + m] = make_float2(0.f, 0.f);
      }
    }
    if (nv == 0) { wabs_min = 0.f; wabs_max = 0.f; }

    uint32_t t0, t1;
    subset_tracks(p, sub, t0, t1);

    // First stage of this item.
    uint32_t cur_t = t0;
    while (cur_t < t1 && track_body(p, cur_t) == 0) ++cur_t;
    if (threadIdx.x == 0 && cur_t < t1) {
      const uint32_t nb = track_body(p, cur_t);
      const uint32_t cnt = min((uint32_t)kStage, nb);
      const int b = stage_no & 1;
      fence_proxy_async();
      mbar_arrive_expect_tx(&sm.bar[b], cnt * 64u);
      bulk_g2s(sm.stage[b], p.records + (p.offsets[cur_t]) * kRecF4, cnt * 64u, &sm.bar[b]);
    }
    pending = cur_t < t1;

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
      for (int q = 0; q < KP; ++q) {
        aTr[q] = aTi[q] = aPr[q] = aPi[q] = make_float2(0.f, 0.f);
      }
#pragma unroll
      for (int m = 0; m < K; ++m)
#pragma unroll
        for (int v = 0; v < 8; ++v) sm.kahan[warp][m][v][lane] = 0.f;

      // Snapshot write: A = compensated outer sum + inner sum, per comp, FP64.
      auto flush = [&](uint32_t ksnap) {
        if (!active) return;
        const double wpdt2 = wp * p.dt * p.dt;
        const double wpdt = sqrt(wp) * p.dt;
        const double thxd = cT * cPh, thyd = cT * sPh, thzd = -sT;
        const double phxd = -sPh, phyd = cPh;
#pragma unroll
        for (int m = 0; m < K; ++m) {
          if (m >= nv) continue;
          const int q = m >> 1;
          const float itr = (m & 1) ? aTr[q].y : aTr[q].x;
          const float iti = (m & 1) ? aTi[q].y : aTi[q].x;
          const float ipr = (m & 1) ? aPr[q].y : aPr[q].x;
          const float ipi = (m & 1) ? aPi[q].y : aPi[q].x;
          const float *kh = &sm.kahan[warp][m][0][lane];
          const double Ar = (double)kh[0 * 32] + (double)kh[4 * 32] + (double)itr;
          const double Ai = (double)kh[1 * 32] + (double)kh[5 * 32] + (double)iti;
          const double Br = (double)kh[2 * 32] + (double)kh[6 * 32] + (double)ipr;
          const double Bi = (double)kh[3 * 32] + (double)kh[7 * 32] + (double)ipi;
          const uint64_t gti = (uint64_t)(j0 + m) + (uint64_t)nO * dir;
          double *part = p.partial + ((uint64_t)sub * p.n_out * p.n_snaps) * P;
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

      df tprev = {0.f, 0.f};  // tau of the previous step (track start: 0 phase)
      for (uint32_t s0 = 0; s0 < n_body; s0 += kStage) {
        const uint32_t cnt = min((uint32_t)kStage, n_body - s0);
        const int b = stage_no & 1;
        // Issue the next stage (this track or the next non-empty one of the item).
        if (threadIdx.x == 0) {
          uint32_t nt = t, ns0 = s0 + kStage;
          if (ns0 >= n_body) {
            nt = t + 1;
            ns0 = 0;
            while (nt < t1 && track_body(p, nt) == 0) ++nt;
          }
          if (nt < t1) {
            const uint32_t nb = track_body(p, nt);
            const uint32_t ncnt = min((uint32_t)kStage, nb - ns0);
            const int nbuf = (stage_no + 1) & 1;
            fence_proxy_async();
            mbar_arrive_expect_tx(&sm.bar[nbuf], ncnt * 64u);
            bulk_g2s(sm.stage[nbuf], p.records + (p.offsets[nt] + ns0) * kRecF4,
                     ncnt * 64u, &sm.bar[nbuf]);
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
        const float4 *stg = sm.stage[b];

        if (active) {
          for (uint32_t c0 = 0; c0 < cnt; c0 += 32) {
            const uint32_t mcnt = min(32u, cnt - c0);
            // ---- per-step setup: lane l -> step s0 + c0 + l ----
            {
              const uint32_t l = (uint32_t)lane < mcnt ? (uint32_t)lane : mcnt - 1;
              const float4 r0 = stg[(c0 + l) * kRecF4 + 0];
              const float4 r1 = stg[(c0 + l) * kRecF4 + 1];
              const float4 r2 = stg[(c0 + l) * kRecF4 + 2];
              const float4 r3 = stg[(c0 + l) * kRecF4 + 3];
              // tau = q + (1 - cos th) z - n_x x - n_y y   (double-float)
              df tau = df{r0.x, r0.y};
              tau = df_add(tau, df_mul(d_c, df{r1.z, r1.w}));
              df nx = df_mul(d_sx, df{r0.z, r0.w});
              df ny = df_mul(d_sy, df{r1.x, r1.y});
              tau = df_add(tau, df{-nx.hi, -nx.lo});
              tau = df_add(tau, df{-ny.hi, -ny.lo});
              // previous step's tau (lane 0: carried, or 0-phase at track start)
              float ph = __shfl_up_sync(0xffffffffu, tau.hi, 1);
              float pl = __shfl_up_sync(0xffffffffu, tau.lo, 1);
              if (lane == 0) { ph = tprev.hi; pl = tprev.lo; }
              const bool first = (s0 + c0 + l) == 0;
              const float dtau = first ? (tau.hi + tau.lo) : ((tau.hi - ph) + (tau.lo - pl));
              // amplitude on theta-hat / phi-hat
              const float D = r2.w + f_c * r2.z - f_sx * r2.x - f_sy * r2.y;
              const float c2 = __frcp_rn(D);
              const float an = f_sx * r3.x + f_sy * r3.y + f_cz * r3.z;
              const float c1 = an * c2 * c2;
              const float tb = thx * r2.x + thy * r2.y + thz * r2.z;
              const float ta = thx * r3.x + thy * r3.y + thz * r3.z;
              const float pb = phx * r2.x + phy * r2.y;
              const float pa = phx * r3.x + phy * r3.y;
              const float amp_t = -(c1 * tb + c2 * ta);
              const float amp_p = -(c1 * pb + c2 * pa);
              // rotation between neighbouring omega points
              const df rp = df_mul_raw(d_dw, tau);
              const float rr = reduce_2pi(rp.hi, rp.lo);
              float Rs, Rc;
              sincosf(rr, &Rs, &Rc);
              const float R2c = Rc * Rc - Rs * Rs, R2s = 2.f * Rc * Rs;
              sm.setup[warp][lane][0] = make_float4(tau.hi, tau.lo, amp_t, amp_p);
              sm.setup[warp][lane][1] = make_float4(Rc, Rs, R2c, R2s);
              sm.setup[warp][lane][2] = make_float4(fabsf(dtau), 0.f, 0.f, 0.f);
              const float th_last = __shfl_sync(0xffffffffu, tau.hi, mcnt - 1);
              const float tl_last = __shfl_sync(0xffffffffu, tau.lo, mcnt - 1);
              tprev = df{th_last, tl_last};
            }
            __syncwarp();
            // ---- the points: K per lane, two at a time ----
            for (uint32_t i = 0; i < mcnt; ++i) {
              const float4 A = sm.setup[warp][i][0];
              const float4 B = sm.setup[warp][i][1];
              const float adt = sm.setup[warp][i][2].x;
              const uint32_t s = s0 + c0 + i;
              const bool all_in = wabs_max * adt < kPiLo;
              const bool all_out = wabs_min * adt > kPiHi;
              if (uniform && all_in) {
                const df pz = df_mul_raw(d_w0, df{A.x, A.y});
                const float r = reduce_2pi(pz.hi, pz.lo);
                float zs, zc;
                __sincosf(r, &zs, &zc);
                float2 Zr = make_float2(zc, zc * B.x - zs * B.y);
                float2 Zi = make_float2(zs, zc * B.y + zs * B.x);
                const float2 at = make_float2(A.z, A.z), ap = make_float2(A.w, A.w);
                const float2 r2c = make_float2(B.z, B.z), r2s = make_float2(B.w, B.w);
                const float2 nr2s = make_float2(-B.w, -B.w);
#pragma unroll
                for (int q = 0; q < KP; ++q) {
                  aTr[q] = __ffma2_rn(Zr, at, aTr[q]);
                  aTi[q] = __ffma2_rn(Zi, at, aTi[q]);
                  aPr[q] = __ffma2_rn(Zr, ap, aPr[q]);
                  aPi[q] = __ffma2_rn(Zi, ap, aPi[q]);
                  if (q + 1 < KP) {
                    const float2 u = __fmul2_rn(Zi, nr2s);
                    const float2 v = __fmul2_rn(Zr, r2s);
                    Zr = __ffma2_rn(Zr, r2c, u);
                    Zi = __ffma2_rn(Zi, r2c, v);
                  }
                }
              } else if (!all_out) {
                // Slow path: per-point mask and/or non-uniform omega.
                uint32_t mask = 0;
                for (int m = 0; m < nv; ++m) {
                  const float2 wd = sm.omega_df[warp][lane * K + m];
                  const float ph = fabsf(wd.x) * adt;
                  bool inc;
                  if (ph < kPiLo) inc = true;
                  else if (ph > kPiHi) inc = false;
                  else inc = exact_mask(p, base, s, it_start, p.omega[j0 + m], n0d, n1d, n2d);
                  mask |= (uint32_t)inc << m;
                }
                float zc = 1.f, zs = 0.f;
#pragma unroll
                for (int m = 0; m < K; ++m) {
                  if (!uniform || m == 0) {
                    const float2 wd = sm.omega_df[warp][lane * K + m];
                    const df pz = df_mul_raw(df{wd.x, wd.y}, df{A.x, A.y});
                    const float r = reduce_2pi(pz.hi, pz.lo);
                    __sincosf(r, &zs, &zc);
                  } else {
                    const float nc = zc * B.x - zs * B.y;
                    zs = zc * B.y + zs * B.x;
                    zc = nc;
                  }
                  if ((mask >> m) & 1u) {
                    const int q = m >> 1;
                    if (m & 1) {
                      aTr[q].y = __fmaf_rn(zc, A.z, aTr[q].y);
                      aTi[q].y = __fmaf_rn(zs, A.z, aTi[q].y);
                      aPr[q].y = __fmaf_rn(zc, A.w, aPr[q].y);
                      aPi[q].y = __fmaf_rn(zs, A.w, aPi[q].y);
                    } else {
                      aTr[q].x = __fmaf_rn(zc, A.z, aTr[q].x);
                      aTi[q].x = __fmaf_rn(zs, A.z, aTi[q].x);
                      aPr[q].x = __fmaf_rn(zc, A.w, aPr[q].x);
                      aPi[q].x = __fmaf_rn(zs, A.w, aPi[q].x);
                    }
                  }
                }
              }
              if ((int64_t)s == snap.fire_it) {  // uniform over the CTA
                flush(snap.k);
                snap.advance(it_start, it_end, snaps, p.n_snaps);
              }
            }
            __syncwarp();
          }
          // ---- fold the stage's FP32 sums into the compensated pairs ----
#pragma unroll
          for (int m = 0; m < K; ++m) {
            const int q = m >> 1;
            const float v[4] = {(m & 1) ? aTr[q].y : aTr[q].x, (m & 1) ? aTi[q].y : aTi[q].x,
                                (m & 1) ? aPr[q].y : aPr[q].x, (m & 1) ? aPi[q].y : aPi[q].x};
#pragma unroll
            for (int c = 0; c < 4; ++c) {
              float &S = sm.kahan[warp][m][c][lane];
              float &C = sm.kahan[warp][m][c + 4][lane];
              const df e = two_sum(S, v[c]);
              S = e.hi;
              C += e.lo;
            }
          }
#pragma unroll
          for (int q = 0; q < KP; ++q) {
            aTr[q] = aTi[q] = aPr[q] = aPi[q] = make_float2(0.f, 0.f);
          }
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
    }
    (void)pending;
  }
}

// out[c][k*P + g] += sum over subsets (fixed order) of partial[sub][c][k][g]
__global__ void far_reduce_kernel(FarMixedParams p) {
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

template <int K, int W>
int launch_main(const FarMixedParams &p, int grid, cudaStream_t s) {
  const size_t smem = sizeof(Smem<K, W>);
  cudaError_t e = cudaFuncSetAttribute(far_mixed_kernel<K, W>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_fail(e, "far_mixed smem attribute");
  far_mixed_kernel<K, W><<<grid, W * 32, smem, s>>>(p);
  return cuda_fail(cudaGetLastError(), "far_mixed kernel launch");
}

template <int W>
int dispatch_k(int K, const FarMixedParams &p, int grid, cudaStream_t s) {
  switch (K) {
    case 2: return launch_main<2, W>(p, grid, s);
    case 4: return launch_main<4, W>(p, grid, s);
    case 6: return launch_main<6, W>(p, grid, s);
    case 8: return launch_main<8, W>(p, grid, s);
    case 10: return launch_main<10, W>(p, grid, s);
    case 12: return launch_main<12, W>(p, grid, s);
    case 14: return launch_main<14, W>(p, grid, s);
    case 16: return launch_main<16, W>(p, grid, s);
    default: return fail(SR_ERR_INVALID, "unsupported points per lane %d", K);
  }
}

template <int K, int W>
int occupancy_of() {
  int n = 0;
  const size_t smem = sizeof(Smem<K, W>);
  cudaFuncSetAttribute(far_mixed_kernel<K, W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)smem);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, far_mixed_kernel<K, W>, W * 32, smem) !=
      cudaSuccess)
    n = 1;
  return n > 0 ? n : 1;
}

int occupancy(int K, int W) {
  if (W != 8) return 1;
  switch (K) {
    case 2: return occupancy_of<2, 8>();
    case 4: return occupancy_of<4, 8>();
    case 6: return occupancy_of<6, 8>();
    case 8: return occupancy_of<8, 8>();
    case 10: return occupancy_of<10, 8>();
    case 12: return occupancy_of<12, 8>();
    case 14: return occupancy_of<14, 8>();
    default: return occupancy_of<16, 8>();
  }
}

}  // namespace

FarMixedConfig far_mixed_choose(uint32_t n_omega, uint32_t n_dirs, uint32_t n_tracks,
                                int n_sm) {
  FarMixedConfig c;
  int k = (int)((n_omega + 31) / 32);
  k += k & 1;
  c.K = k < 2 ? 2 : (k > 16 ? 16 : k);
  c.W = 8;
  c.ctas_per_sm = 1;
  const uint64_t n_wtiles = (n_omega + 32u * c.K - 1) / (32u * c.K);
  const uint64_t groups = (n_dirs * n_wtiles + c.W - 1) / c.W;
  const uint64_t capacity = (uint64_t)n_sm * c.ctas_per_sm;
  uint64_t nsub = (16 * capacity + groups - 1) / (groups ? groups : 1);
  if (nsub > n_tracks) nsub = n_tracks;
  if (nsub < 1) nsub = 1;
  if (nsub > 64) nsub = 64;
  c.n_sub = (int)nsub;
  return c;
}

size_t far_mixed_workspace(int64_t total_steps, uint64_t n_points, int n_out, uint32_t n_snaps,
                           const FarMixedConfig &cfg) {
  size_t b = 256;                                          // status word
  b += ((size_t)total_steps * 64 + 255) / 256 * 256;       // step records
  b += (size_t)cfg.n_sub * n_out * n_snaps * n_points * 8; // partial spectra
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
  p.status = (int *)w;
  p.records = (float4 *)(w + 256);
  p.partial = (double *)(w + 256 + ((size_t)p.total_steps * 64 + 255) / 256 * 256);
  p.n_wtiles = (p.n_omega + 32u * cfg.K - 1) / (32u * cfg.K);
  const uint32_t n_dirs = p.n_theta * p.n_phi;
  p.n_groups = (uint32_t)(((uint64_t)n_dirs * p.n_wtiles + cfg.W - 1) / cfg.W);
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
      far_prepass_kernel<float><<<(int)nb, blk, 0, stream>>>(p);
    else
      far_prepass_kernel<double><<<(int)nb, blk, 0, stream>>>(p);
    int rc = cuda_fail(cudaGetLastError(), "far prepass launch");
    if (rc) return rc;
  }
  const int occ = occupancy(cfg.K, cfg.W);
  int grid = n_sm * occ;
  if ((uint32_t)grid > p.n_items) grid = (int)p.n_items;
  void *tok = nullptr;
  timing_record(stream, true, &tok);
  int rc = dispatch_k<8>(cfg.K, p, grid, stream);
  timing_record(stream, false, &tok);
  if (rc) return rc;
  const uint64_t total = (uint64_t)p.n_out * p.n_snaps * P;
  uint64_t nb = (total + 255) / 256;
  if (nb > (uint64_t)n_sm * 64) nb = (uint64_t)n_sm * 64;
  far_reduce_kernel<<<(unsigned)nb, 256, 0, stream>>>(p);
  return cuda_fail(cudaGetLastError(), "far reduce launch");
}

}  // namespace sr
