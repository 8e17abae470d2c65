/*
 * SynchRad radiation integral: CPU oracle (plain C, FP64 and FP32).
 *
 * TEST INFRASTRUCTURE ONLY.  This is a restatement of the reference's device
 * kernels, synchrad/kernel_farfield.cl (5 kernels) and
 * synchrad/kernel_nearfield.cl (3 kernels), used as the parity checker for
 * the CUDA library and as the timed CPU baseline.  Only tests/, the smoke
 * check and bench.py's CPU-baseline leg may load it; the product never does.
 *
 * Pinning: tests/test_oracle.py checks it bit-for-bit against the reference's
 * own kernel source compiled for the CPU (oracle/build_ref.sh ->
 * oracle/_ref/libsr_ref.so) where that source is available, and against the
 * golden vectors in tests/golden/ (generated from oracle/_ref by
 * tests/golden/make_golden.py) everywhere else.
 *
 * ABI (same as oracle/ref_driver.cpp, so both are interchangeable):
 *   dtype 0 = double, 1 = float: the element type of every array argument
 *   comp  0 total, 1 cartesian, 2 cartesian_complex, 3 spheric,
 *         4 spheric_complex (near field: 0, 1, 2)
 *   spectra[]: device-order arrays [nSnaps][nPhi][nTheta|nR][nOmega],
 *              accumulated in place (+=) as the reference kernels do
 *   track[] = {x, y, z, ux, uy, uz}, axes[] = {omega*2pi, sinTheta, cosTheta,
 *   sinPhi, cosPhi} (far) or {omega*2pi, radius, sinPhi, cosPhi} (near).
 * Returns 0, or -1 for arguments the reference cannot handle either
 * (itEnd == 0 or nSteps == 0 make its unsigned loop bounds wrap).
 */
#include <math.h>
#include <stdint.h>
#include <stddef.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

#define REAL double
#define SFX f64
#define R_SQRT(v) sqrt(v)
#define R_SIN(v) sin(v)
#define R_COS(v) cos(v)
#define R_FABS(v) fabs(v)
#include "sr_oracle_impl.h"
#undef REAL
#undef SFX
#undef R_SQRT
#undef R_SIN
#undef R_COS
#undef R_FABS

#define REAL float
#define SFX f32
#define R_SQRT(v) sqrtf(v)
#define R_SIN(v) sinf(v)
#define R_COS(v) cosf(v)
#define R_FABS(v) fabsf(v)
#include "sr_oracle_impl.h"
#undef REAL
#undef SFX
#undef R_SQRT
#undef R_SIN
#undef R_COS
#undef R_FABS

int sro_far(int dtype, int comp, void *const *spectra, const void *const *track,
            double wp, uint32_t itStart, uint32_t itEnd, uint32_t nSteps,
            const void *const *axes, uint32_t nOmega, uint32_t nTheta,
            uint32_t nPhi, double dt, uint32_t nSnaps, const uint32_t *itSnaps,
            const void *formFactor, int nthreads) {
  if (itEnd == 0 || nSteps == 0 || comp < 0 || comp > 4) return -1;
  if (comp == 2 && formFactor == NULL) return -1;
  if (nthreads < 1) nthreads = 1;
  if (dtype == 0)
    return far_f64(comp, spectra, track, wp, itStart, itEnd, nSteps, axes,
                   nOmega, nTheta, nPhi, dt, nSnaps, itSnaps, formFactor,
                   nthreads);
  if (dtype == 1)
    return far_f32(comp, spectra, track, wp, itStart, itEnd, nSteps, axes,
                   nOmega, nTheta, nPhi, dt, nSnaps, itSnaps, formFactor,
                   nthreads);
  return -1;
}

int sro_near(int dtype, int comp, void *const *spectra,
             const void *const *track, double wp, uint32_t itStart,
             uint32_t itEnd, uint32_t nSteps, const void *const *axes,
             double L, uint32_t nOmega, uint32_t nR, uint32_t nPhi, double dt,
             uint32_t nSnaps, const uint32_t *itSnaps, const void *formFactor,
             int nthreads) {
  (void)formFactor; /* passed but not applied, synchrad/kernel_nearfield.cl:244 */
  if (itEnd == 0 || nSteps == 0 || comp < 0 || comp > 2) return -1;
  if (nthreads < 1) nthreads = 1;
  if (dtype == 0)
    return near_f64(comp, spectra, track, wp, itStart, itEnd, nSteps, axes, L,
                    nOmega, nR, nPhi, dt, nSnaps, itSnaps, nthreads);
  if (dtype == 1)
    return near_f32(comp, spectra, track, wp, itStart, itEnd, nSteps, axes, L,
                    nOmega, nR, nPhi, dt, nSnaps, itSnaps, nthreads);
  return -1;
}
