/*
 * Host driver for the reference's own OpenCL kernels compiled as C++
 * (see oracle/ref_shim.hpp and oracle/build_ref.sh).
 *
 * TEST INFRASTRUCTURE ONLY.  It plays the role of the OpenCL NDRange of
 * synchrad/calc.py:324-353: one call per track, one work-item per spectral
 * point (gti = iOmega + nOmega*(iTheta + nTheta*iPhi)), here an OpenMP loop
 * over points.  The kernels themselves are the reference's, unmodified apart
 * from the Mako substitution of ${my_dtype} and ${f_native}
 * (synchrad/calc.py:605-624).
 *
 * The reference kernels read itSnaps[nSnaps] once every snapshot has been
 * written (synchrad/kernel_farfield.cl:100 after iSnap reaches nSnaps).  The
 * driver passes a copy of itSnaps with one extra slot holding 0, a value that
 * `it_glob + 2` never equals, so that read stays in bounds and never fires.
 */
#include <cstdint>
#include <vector>

thread_local unsigned int sr_cl_gid = 0;

typedef unsigned int uint;

#define SR_FAR_TAIL(T)                                                       \
  T *, T *, T *, T *, T *, T *, T, uint, uint, uint, T *, T *, T *, T *, T *, \
      uint, uint, uint, T, uint, uint *
#define SR_NEAR_TAIL(T)                                                      \
  T *, T *, T *, T *, T *, T *, T, uint, uint, uint, T *, T *, T *, T *, T,   \
      uint, uint, uint, T, uint, uint *

#define SR_DECLARE_FAR(NS, T)                                                \
  namespace NS {                                                             \
  void total(T *, SR_FAR_TAIL(T));                                           \
  void cartesian_comps(T *, T *, T *, SR_FAR_TAIL(T));                       \
  void cartesian_comps_complex(T *, T *, T *, T *, T *, T *, SR_FAR_TAIL(T), \
                               T *);                                         \
  void spheric_comps(T *, T *, T *, SR_FAR_TAIL(T));                         \
  void spheric_comps_complex(T *, T *, T *, T *, T *, T *, SR_FAR_TAIL(T),   \
                             T *);                                           \
  }
#define SR_DECLARE_NEAR(NS, T)                                               \
  namespace NS {                                                             \
  void total(T *, SR_NEAR_TAIL(T));                                          \
  void cartesian_comps(T *, T *, T *, SR_NEAR_TAIL(T));                      \
  void cartesian_comps_complex(T *, T *, T *, T *, T *, T *,                 \
                               SR_NEAR_TAIL(T), T *);                        \
  }

SR_DECLARE_FAR(sr_ref_far_double, double)
SR_DECLARE_FAR(sr_ref_far_float, float)
SR_DECLARE_NEAR(sr_ref_near_double, double)
SR_DECLARE_NEAR(sr_ref_near_float, float)

namespace {

template <typename T>
struct FarKernels;
template <>
struct FarKernels<double> {
  static constexpr auto total = &sr_ref_far_double::total;
  static constexpr auto cart = &sr_ref_far_double::cartesian_comps;
  static constexpr auto cart_c = &sr_ref_far_double::cartesian_comps_complex;
  static constexpr auto sph = &sr_ref_far_double::spheric_comps;
  static constexpr auto sph_c = &sr_ref_far_double::spheric_comps_complex;
};
template <>
struct FarKernels<float> {
  static constexpr auto total = &sr_ref_far_float::total;
  static constexpr auto cart = &sr_ref_far_float::cartesian_comps;
  static constexpr auto cart_c = &sr_ref_far_float::cartesian_comps_complex;
  static constexpr auto sph = &sr_ref_far_float::spheric_comps;
  static constexpr auto sph_c = &sr_ref_far_float::spheric_comps_complex;
};
template <typename T>
struct NearKernels;
template <>
struct NearKernels<double> {
  static constexpr auto total = &sr_ref_near_double::total;
  static constexpr auto cart = &sr_ref_near_double::cartesian_comps;
  static constexpr auto cart_c = &sr_ref_near_double::cartesian_comps_complex;
};
template <>
struct NearKernels<float> {
  static constexpr auto total = &sr_ref_near_float::total;
  static constexpr auto cart = &sr_ref_near_float::cartesian_comps;
  static constexpr auto cart_c = &sr_ref_near_float::cartesian_comps_complex;
};

template <typename T>
int run_far(int comp, void *const *sp, const void *const *trk, double wp,
            uint itStart, uint itEnd, uint nSteps, const void *const *ax,
            uint nO, uint nT, uint nP, double dt, uint nSnaps,
            const uint *itSnaps, const void *ff, int nthreads) {
  std::vector<uint> snaps(itSnaps, itSnaps + nSnaps);
  snaps.push_back(0u);
  T *s[6];
  for (int i = 0; i < 6; ++i) s[i] = (T *)sp[i];
  T *x = (T *)trk[0], *y = (T *)trk[1], *z = (T *)trk[2];
  T *ux = (T *)trk[3], *uy = (T *)trk[4], *uz = (T *)trk[5];
  T *om = (T *)ax[0], *sT = (T *)ax[1], *cT = (T *)ax[2], *sP = (T *)ax[3],
    *cP = (T *)ax[4];
  T *F = (T *)ff;
  const long long n = (long long)nO * nT * nP;
  if (comp < 0 || comp > 4) return -1;
  if ((comp == 2 || comp == 4) && !F) return -1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (long long g = 0; g < n; ++g) {
    sr_cl_gid = (unsigned int)g;
    uint *isn = const_cast<uint *>(snaps.data());
    switch (comp) {
      case 0:
        FarKernels<T>::total(s[0], x, y, z, ux, uy, uz, (T)wp, itStart, itEnd,
                             nSteps, om, sT, cT, sP, cP, nO, nT, nP, (T)dt,
                             nSnaps, isn);
        break;
      case 1:
        FarKernels<T>::cart(s[0], s[1], s[2], x, y, z, ux, uy, uz, (T)wp,
                            itStart, itEnd, nSteps, om, sT, cT, sP, cP, nO, nT,
                            nP, (T)dt, nSnaps, isn);
        break;
      case 2:
        FarKernels<T>::cart_c(s[0], s[1], s[2], s[3], s[4], s[5], x, y, z, ux,
                              uy, uz, (T)wp, itStart, itEnd, nSteps, om, sT,
                              cT, sP, cP, nO, nT, nP, (T)dt, nSnaps, isn, F);
        break;
      case 3:
        FarKernels<T>::sph(s[0], s[1], s[2], x, y, z, ux, uy, uz, (T)wp,
                           itStart, itEnd, nSteps, om, sT, cT, sP, cP, nO, nT,
                           nP, (T)dt, nSnaps, isn);
        break;
      case 4:
        FarKernels<T>::sph_c(s[0], s[1], s[2], s[3], s[4], s[5], x, y, z, ux,
                             uy, uz, (T)wp, itStart, itEnd, nSteps, om, sT, cT,
                             sP, cP, nO, nT, nP, (T)dt, nSnaps, isn, F);
        break;
    }
  }
  return 0;
}

template <typename T>
int run_near(int comp, void *const *sp, const void *const *trk, double wp,
             uint itStart, uint itEnd, uint nSteps, const void *const *ax,
             double L, uint nO, uint nR, uint nP, double dt, uint nSnaps,
             const uint *itSnaps, const void *ff, int nthreads) {
  std::vector<uint> snaps(itSnaps, itSnaps + nSnaps);
  snaps.push_back(0u);
  T *s[6];
  for (int i = 0; i < 6; ++i) s[i] = (T *)sp[i];
  T *x = (T *)trk[0], *y = (T *)trk[1], *z = (T *)trk[2];
  T *ux = (T *)trk[3], *uy = (T *)trk[4], *uz = (T *)trk[5];
  T *om = (T *)ax[0], *rad = (T *)ax[1], *sP = (T *)ax[2], *cP = (T *)ax[3];
  T *F = (T *)ff;
  const long long n = (long long)nO * nR * nP;
  if (comp < 0 || comp > 2) return -1;
  if (comp == 2 && !F) return -1;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (long long g = 0; g < n; ++g) {
    sr_cl_gid = (unsigned int)g;
    uint *isn = const_cast<uint *>(snaps.data());
    switch (comp) {
      case 0:
        NearKernels<T>::total(s[0], x, y, z, ux, uy, uz, (T)wp, itStart,
                              itEnd, nSteps, om, rad, sP, cP, (T)L, nO, nR, nP,
                              (T)dt, nSnaps, isn);
        break;
      case 1:
        NearKernels<T>::cart(s[0], s[1], s[2], x, y, z, ux, uy, uz, (T)wp,
                             itStart, itEnd, nSteps, om, rad, sP, cP, (T)L, nO,
                             nR, nP, (T)dt, nSnaps, isn);
        break;
      case 2:
        NearKernels<T>::cart_c(s[0], s[1], s[2], s[3], s[4], s[5], x, y, z,
                               ux, uy, uz, (T)wp, itStart, itEnd, nSteps, om,
                               rad, sP, cP, (T)L, nO, nR, nP, (T)dt, nSnaps,
                               isn, F);
        break;
    }
  }
  return 0;
}

}  // namespace

extern "C" int sr_ref_far(int dtype, int comp, void *const *spectra,
                          const void *const *track, double wp, uint itStart,
                          uint itEnd, uint nSteps, const void *const *axes,
                          uint nOmega, uint nTheta, uint nPhi, double dt,
                          uint nSnaps, const uint *itSnaps,
                          const void *formFactor, int nthreads) {
  if (dtype == 0)
    return run_far<double>(comp, spectra, track, wp, itStart, itEnd, nSteps,
                           axes, nOmega, nTheta, nPhi, dt, nSnaps, itSnaps,
                           formFactor, nthreads);
  if (dtype == 1)
    return run_far<float>(comp, spectra, track, wp, itStart, itEnd, nSteps,
                          axes, nOmega, nTheta, nPhi, dt, nSnaps, itSnaps,
                          formFactor, nthreads);
  return -1;
}

extern "C" int sr_ref_near(int dtype, int comp, void *const *spectra,
                           const void *const *track, double wp, uint itStart,
                           uint itEnd, uint nSteps, const void *const *axes,
                           double L, uint nOmega, uint nR, uint nPhi,
                           double dt, uint nSnaps, const uint *itSnaps,
                           const void *formFactor, int nthreads) {
  if (dtype == 0)
    return run_near<double>(comp, spectra, track, wp, itStart, itEnd, nSteps,
                            axes, L, nOmega, nR, nPhi, dt, nSnaps, itSnaps,
                            formFactor, nthreads);
  if (dtype == 1)
    return run_near<float>(comp, spectra, track, wp, itStart, itEnd, nSteps,
                           axes, L, nOmega, nR, nPhi, dt, nSnaps, itSnaps,
                           formFactor, nthreads);
  return -1;
}
