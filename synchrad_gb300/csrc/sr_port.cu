// Plain ports of the reference kernels: one thread per spectral point, every
// track of the batch in sequence, the reference's arithmetic in FP64 or FP32.
//
// This translation unit is compiled with --fmad=false so that, like the
// reference built without contraction, every product and sum is rounded on its
// own; the FP64 results then differ from the CPU oracle only through the last
// bits of sin/cos.  These kernels are the SR_PREC_DOUBLE path (the "plain FP64"
// baseline), and SR_PREC_FLOAT / SR_PREC_FLOAT_NATIVE (dtype='float').
#include <cmath>

#include "sr_common.cuh"
#include "sr_internal.h"

namespace sr {
namespace {

template <typename T, bool NATIVE>
struct Math;
template <bool NATIVE>
struct Math<double, NATIVE> {
  static __device__ __forceinline__ double rsq(double v) { return 1.0 / sqrt(v); }
  static __device__ __forceinline__ double sqr(double v) { return sqrt(v); }
  static __device__ __forceinline__ double sn(double v) { return sin(v); }
  static __device__ __forceinline__ double cs(double v) { return cos(v); }
};
template <>
struct Math<float, false> {
  static __device__ __forceinline__ float rsq(float v) { return 1.0f / sqrtf(v); }
  static __device__ __forceinline__ float sqr(float v) { return sqrtf(v); }
  static __device__ __forceinline__ float sn(float v) { return sinf(v); }
  static __device__ __forceinline__ float cs(float v) { return cosf(v); }
};
template <>
struct Math<float, true> {  // OpenCL native_* counterparts
  static __device__ __forceinline__ float rsq(float v) { return rsqrtf(v); }
  static __device__ __forceinline__ float sqr(float v) { return sqrtf(v); }
  static __device__ __forceinline__ float sn(float v) { return __sinf(v); }
  static __device__ __forceinline__ float cs(float v) { return __cosf(v); }
};

struct TrackView {
  uint64_t base;
  uint32_t n_steps, it_start, it_end;
  double wp;
  const uint32_t *snaps;
};

__device__ __forceinline__ TrackView track_view(const PortParams &p, uint32_t t) {
  TrackView v;
  if (p.offsets == nullptr) {
    v.base = 0;
    v.n_steps = p.n_steps1;
    v.it_start = p.it_start1;
    v.it_end = p.it_end1;
    v.wp = p.wp1;
    v.snaps = p.snap_its;
  } else {
    v.base = (uint64_t)p.offsets[t];
    v.n_steps = (uint32_t)(p.offsets[t + 1] - p.offsets[t]);
    v.it_start = p.it_start[t];
    v.it_end = p.it_end[t];
    v.wp = p.weight[t];
    v.snaps = p.snap_its + (size_t)t * p.snap_stride;
  }
  return v;
}

// Far field (synchrad/kernel_farfield.cl, all five kernels).
// COMP: 0 total, 1 cartesian, 2 cartesian_complex, 3 spheric, 4 spheric_complex.
template <typename T, int COMP, bool NATIVE>
__global__ void __launch_bounds__(256) port_far_kernel(PortParams p) {
  using M = Math<T, NATIVE>;
  const uint32_t nO = p.n_omega, nT = p.n_1, nP = p.n_phi;
  const uint64_t nTotal = (uint64_t)nO * nT * nP;
  const T *om = (const T *)p.omega, *sT = (const T *)p.axis1,
          *cT = (const T *)p.axis2, *sP = (const T *)p.sin_phi,
          *cP = (const T *)p.cos_phi, *ffa = (const T *)p.form_factor;
  const T *X = (const T *)p.x, *Y = (const T *)p.y, *Z = (const T *)p.z;
  const T *UX = (const T *)p.ux, *UY = (const T *)p.uy, *UZ = (const T *)p.uz;
  const T dt = (T)p.dt;
  const T dtInv = (T)1. / dt;
  const uint32_t n_tr = p.offsets ? p.n_tracks : 1u;

  for (uint64_t gti = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
       gti < nTotal; gti += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t iP = (uint32_t)(gti / ((uint64_t)nO * nT));
    const uint32_t iT = (uint32_t)((gti - (uint64_t)iP * nO * nT) / nO);
    const uint32_t iO = (uint32_t)(gti - (uint64_t)iP * nO * nT - (uint64_t)iT * nO);
    const T w = om[iO];
    const T n0 = sT[iT] * cP[iP], n1 = sT[iT] * sP[iP], n2 = cT[iT];
    const T t0 = cT[iT] * cP[iP], t1 = cT[iT] * sP[iP], t2 = -sT[iT];
    const T p0 = -sP[iP], p1 = cP[iP], p2 = (T)0.0;
    const T ffl = (COMP == 2) ? ffa[iO] : (T)1.0;

    for (uint32_t tr = 0; tr < n_tr; ++tr) {
      const TrackView tv = track_view(p, tr);
      if (tv.it_end == 0 || tv.n_steps == 0) continue;  // rejected on the host
      const T wp = (T)tv.wp;
      const T wpdt2 = wp * dt * dt;
      const T wpdt = M::sqr(wp) * dt;
      const T *x = X + tv.base, *y = Y + tv.base, *z = Z + tv.base;
      const T *ux = UX + tv.base, *uy = UY + tv.base, *uz = UZ + tv.base;
      T phasePrev = (T)0.;
      T re0 = 0, re1 = 0, re2 = 0, im0 = 0, im1 = 0, im2 = 0;
      SnapState snap;
      snap.init(tv.it_start, tv.it_end, tv.snaps, p.n_snaps);
      // Body steps; snapshot writes due after the last body step (the
      // reference keeps iterating up to itEnd - 2 without changing A) are
      // issued by the second phase of the loop without empty iterations.
      const uint32_t n_body = min(tv.it_end - 1u, tv.n_steps - 1u);
      for (int64_t it64 = 0; it64 < (int64_t)n_body || snap.fire_it != SnapState::NEVER;
           it64 = (it64 < (int64_t)n_body) ? it64 + 1 : snap.fire_it) {
        const uint32_t it = (uint32_t)it64;
        if (it64 < (int64_t)n_body) {
          const uint32_t itg = tv.it_start + it;
          const T time = (T)itg * dt;
          const T phase = w * (time - (x[it] * n0 + y[it] * n1 + z[it] * n2));
          const T dPhase = fabs(phase - phasePrev);
          phasePrev = phase;
          if (dPhase < (T)M_PI) {
            T g = M::rsq((T)1. + (ux[it] * ux[it] + uy[it] * uy[it] + uz[it] * uz[it]));
            const T b0 = ux[it] * g, b1 = uy[it] * g, b2 = uz[it] * g;
            g = M::rsq((T)1. + (ux[it + 1] * ux[it + 1] + uy[it + 1] * uy[it + 1] +
                                uz[it + 1] * uz[it + 1]));
            const T bn0 = ux[it + 1] * g, bn1 = uy[it + 1] * g, bn2 = uz[it + 1] * g;
            const T a0 = (bn0 - b0) * dtInv, a1 = (bn1 - b1) * dtInv, a2 = (bn2 - b2) * dtInv;
            const T m0 = (T)0.5 * (bn0 + b0), m1 = (T)0.5 * (bn1 + b1),
                    m2 = (T)0.5 * (bn2 + b2);
            T c1 = a0 * n0 + a1 * n1 + a2 * n2;
            T c2 = (T)1. - (m0 * n0 + m1 * n1 + m2 * n2);
            c2 = (T)1. / c2;
            c1 = c1 * c2 * c2;
            const T sn = M::sn(phase), cs = M::cs(phase);
            T A0 = c1 * (n0 - m0) - c2 * a0;
            T A1 = c1 * (n1 - m1) - c2 * a1;
            T A2 = c1 * (n2 - m2) - c2 * a2;
            if (COMP == 3 || COMP == 4) {
              const T r = n0 * A0 + n1 * A1 + n2 * A2;
              const T th = t0 * A0 + t1 * A1 + t2 * A2;
              const T ph = p0 * A0 + p1 * A1 + p2 * A2;
              A0 = r; A1 = th; A2 = ph;
            }
            if (COMP == 2) {
              re0 += A0 * cs * ffl; re1 += A1 * cs * ffl; re2 += A2 * cs * ffl;
              im0 += A0 * sn * ffl; im1 += A1 * sn * ffl; im2 += A2 * sn * ffl;
            } else {
              re0 += A0 * cs; re1 += A1 * cs; re2 += A2 * cs;
              im0 += A0 * sn; im1 += A1 * sn; im2 += A2 * sn;
            }
          }
        }
        if (it64 == snap.fire_it) {
          const uint64_t o = gti + nTotal * snap.k;
          T **out = (T **)p.out;
          if (COMP == 0) {
            out[0][o] += wpdt2 * ((re0 * re0 + re1 * re1 + re2 * re2) +
                                  (im0 * im0 + im1 * im1 + im2 * im2));
          } else if (COMP == 1 || COMP == 3) {
            out[0][o] += wpdt2 * (re0 * re0 + im0 * im0);
            out[1][o] += wpdt2 * (re1 * re1 + im1 * im1);
            out[2][o] += wpdt2 * (re2 * re2 + im2 * im2);
          } else {
            out[0][o] += wpdt * re0; out[1][o] += wpdt * im0;
            out[2][o] += wpdt * re1; out[3][o] += wpdt * im1;
            out[4][o] += wpdt * re2; out[5][o] += wpdt * im2;
          }
          snap.advance(tv.it_start, tv.it_end, tv.snaps, p.n_snaps);
        }
      }
    }
  }
}

// Near field (synchrad/kernel_nearfield.cl, all three kernels).
// COMP: 0 total, 1 cartesian, 2 cartesian_complex (FormFactor not applied).
template <typename T, int COMP, bool NATIVE>
__global__ void __launch_bounds__(256) port_near_kernel(PortParams p) {
  using M = Math<T, NATIVE>;
  const uint32_t nO = p.n_omega, nR = p.n_1, nP = p.n_phi;
  const uint64_t nTotal = (uint64_t)nO * nR * nP;
  const T *om = (const T *)p.omega, *rad = (const T *)p.axis1,
          *sP = (const T *)p.sin_phi, *cP = (const T *)p.cos_phi;
  const T *X = (const T *)p.x, *Y = (const T *)p.y, *Z = (const T *)p.z;
  const T *UX = (const T *)p.ux, *UY = (const T *)p.uy, *UZ = (const T *)p.uz;
  const T dt = (T)p.dt;
  const T L = (T)p.L;
  const uint32_t n_tr = p.offsets ? p.n_tracks : 1u;

  for (uint64_t gti = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
       gti < nTotal; gti += (uint64_t)gridDim.x * blockDim.x) {
    const uint32_t iP = (uint32_t)(gti / ((uint64_t)nO * nR));
    const uint32_t iR = (uint32_t)((gti - (uint64_t)iP * nO * nR) / nO);
    const uint32_t iO = (uint32_t)(gti - (uint64_t)iP * nO * nR - (uint64_t)iR * nO);
    const T w = om[iO];
    const T P0 = rad[iR] * cP[iP], P1 = rad[iR] * sP[iP], P2 = L;

    for (uint32_t tr = 0; tr < n_tr; ++tr) {
      const TrackView tv = track_view(p, tr);
      if (tv.it_end == 0 || tv.n_steps == 0) continue;  // rejected on the host
      const T wp = (T)tv.wp;
      const T wpdt2 = wp * dt * dt;
      const T wpdt = M::sqr(wp) * dt;
      const T *x = X + tv.base, *y = Y + tv.base, *z = Z + tv.base;
      const T *ux = UX + tv.base, *uy = UY + tv.base, *uz = UZ + tv.base;
      T phasePrev = (T)0.;
      T re0 = 0, re1 = 0, re2 = 0, im0 = 0, im1 = 0, im2 = 0;
      SnapState snap;
      snap.init(tv.it_start, tv.it_end, tv.snaps, p.n_snaps);
      // Body steps; snapshot writes due after the last body step (the
      // reference keeps iterating up to itEnd - 2 without changing A) are
      // issued by the second phase of the loop without empty iterations.
      const uint32_t n_body = min(tv.it_end - 1u, tv.n_steps - 1u);
      for (int64_t it64 = 0; it64 < (int64_t)n_body || snap.fire_it != SnapState::NEVER;
           it64 = (it64 < (int64_t)n_body) ? it64 + 1 : snap.fire_it) {
        const uint32_t it = (uint32_t)it64;
        if (it64 < (int64_t)n_body) {
          const uint32_t itg = tv.it_start + it;
          const T time = (T)itg * dt;
          const T d0 = P0 - x[it], d1 = P1 - y[it], d2 = P2 - z[it];
          const T r = M::sqr(d0 * d0 + d1 * d1 + d2 * d2);
          const T phase = w * (time + r);
          const T dPhase = fabs(phase - phasePrev);
          phasePrev = phase;
          if (dPhase < (T)M_PI) {
            const T rInv = (T)1. / r;
            const T n0 = rInv * d0, n1 = rInv * d1, n2 = rInv * d2;
            const T g = M::rsq((T)1. + (ux[it] * ux[it] + uy[it] * uy[it] + uz[it] * uz[it]));
            const T b0 = ux[it] * g, b1 = uy[it] * g, b2 = uz[it] * g;
            const T sn = M::sn(phase), cs = M::cs(phase);
            const T wr = w * rInv, rr = rInv * rInv;
            const T c10 = wr * (b0 - n0), c11 = wr * (b1 - n1), c12 = wr * (b2 - n2);
            const T c20 = rr * n0, c21 = rr * n1, c22 = rr * n2;
            re0 += -c10 * sn + c20 * cs; re1 += -c11 * sn + c21 * cs;
            re2 += -c12 * sn + c22 * cs;
            im0 += c10 * cs + c20 * sn; im1 += c11 * cs + c21 * sn;
            im2 += c12 * cs + c22 * sn;
          }
        }
        if (it64 == snap.fire_it) {
          const uint64_t o = gti + nTotal * snap.k;
          T **out = (T **)p.out;
          if (COMP == 0) {
            out[0][o] += wpdt2 * ((re0 * re0 + re1 * re1 + re2 * re2) +
                                  (im0 * im0 + im1 * im1 + im2 * im2));
          } else if (COMP == 1) {
            out[0][o] += wpdt2 * (re0 * re0 + im0 * im0);
            out[1][o] += wpdt2 * (re1 * re1 + im1 * im1);
            out[2][o] += wpdt2 * (re2 * re2 + im2 * im2);
          } else {
            out[0][o] += wpdt * re0; out[1][o] += wpdt * im0;
            out[2][o] += wpdt * re1; out[3][o] += wpdt * im1;
            out[4][o] += wpdt * re2; out[5][o] += wpdt * im2;
          }
          snap.advance(tv.it_start, tv.it_end, tv.snaps, p.n_snaps);
        }
      }
    }
  }
}

template <typename T, bool NATIVE>
int launch_typed(const PortParams &p, int mode, int comp, cudaStream_t s) {
  const uint64_t n = (uint64_t)p.n_omega * p.n_1 * p.n_phi;
  const int block = 256;
  uint64_t blocks = (n + block - 1) / block;
  if (blocks > (1u << 30)) blocks = 1u << 30;
  const dim3 grid((unsigned)blocks);
  if (mode == 0) {
    switch (comp) {
      case 0: port_far_kernel<T, 0, NATIVE><<<grid, block, 0, s>>>(p); break;
      case 1: port_far_kernel<T, 1, NATIVE><<<grid, block, 0, s>>>(p); break;
      case 2: port_far_kernel<T, 2, NATIVE><<<grid, block, 0, s>>>(p); break;
      case 3: port_far_kernel<T, 3, NATIVE><<<grid, block, 0, s>>>(p); break;
      case 4: port_far_kernel<T, 4, NATIVE><<<grid, block, 0, s>>>(p); break;
      default: return fail(SR_ERR_INVALID, "unknown comp %d", comp);
    }
  } else {
    switch (comp) {
      case 0: port_near_kernel<T, 0, NATIVE><<<grid, block, 0, s>>>(p); break;
      case 1: port_near_kernel<T, 1, NATIVE><<<grid, block, 0, s>>>(p); break;
      case 2: port_near_kernel<T, 2, NATIVE><<<grid, block, 0, s>>>(p); break;
      default: return fail(SR_ERR_UNSUPPORTED, "near field has no comp %d", comp);
    }
  }
  return cuda_fail(cudaGetLastError(), "port kernel launch");
}

}  // namespace

int launch_port(const PortParams &p, int mode, int comp, int dtype, bool native,
                cudaStream_t stream) {
  if ((uint64_t)p.n_omega * p.n_1 * p.n_phi == 0) return SR_OK;
  void *tok = nullptr;
  timing_record(stream, true, &tok);
  int rc;
  if (dtype == SR_DTYPE_F64)
    rc = launch_typed<double, false>(p, mode, comp, stream);
  else if (native)
    rc = launch_typed<float, true>(p, mode, comp, stream);
  else
    rc = launch_typed<float, false>(p, mode, comp, stream);
  timing_record(stream, false, &tok);
  return rc;
}

}  // namespace sr
