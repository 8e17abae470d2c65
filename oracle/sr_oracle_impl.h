/*
 * Body of the CPU oracle, included twice by oracle/sr_oracle.c with
 *   REAL = double, SFX = f64   and   REAL = float, SFX = f32.
 *
 * TEST INFRASTRUCTURE ONLY (see the header of oracle/sr_oracle.c).
 *
 * Every expression keeps the operand order of the reference kernels so that,
 * built with -ffp-contract=off, the results are bit-identical to the
 * reference source compiled through oracle/ref_shim.hpp.
 */

#define SR_CAT2(a, b) a##_##b
#define SR_CAT(a, b) SR_CAT2(a, b)
#define SR_FN(name) SR_CAT(name, SFX)

/* First snapshot index whose iteration lies after itStart
 * (synchrad/kernel_farfield.cl:53-57). */
static uint32_t SR_FN(first_snap)(uint32_t itStart, uint32_t nSnaps,
                                  const uint32_t *itSnaps) {
  uint32_t k = 0;
  while (k < nSnaps && !(itStart < itSnaps[k])) ++k;
  return k;
}

/*
 * Far field, one spectral point, one track: the loop of
 * synchrad/kernel_farfield.cl:59-107 (total), :166-223 (cartesian_comps),
 * :287-342 (cartesian_comps_complex), :405-467 (spheric_comps) and
 * :534-592 (spheric_comps_complex).
 *   amp = c1 (n - bbar) - c2 a,  c2 = 1/(1 - n.bbar),  c1 = (a.n) c2^2
 *   A  += amp exp(i w (t - n.x))   while |phase - phasePrev| < pi
 * The snapshot write fires when itStart + it + 2 == itSnaps[k]; the k < nSnaps
 * guard replaces the reference's read of itSnaps[nSnaps] once all snapshots
 * are written (that read never matches in the cases the reference handles).
 */
static void SR_FN(far_point)(int comp, uint64_t gti, REAL *const *sp,
                             const REAL *x, const REAL *y, const REAL *z,
                             const REAL *ux, const REAL *uy, const REAL *uz,
                             REAL wp, uint32_t itStart, uint32_t itEnd,
                             uint32_t nSteps, const REAL *omega,
                             const REAL *sinT, const REAL *cosT,
                             const REAL *sinP, const REAL *cosP, uint32_t nO,
                             uint32_t nT, uint32_t nP, REAL dt,
                             uint32_t nSnaps, const uint32_t *itSnaps,
                             const REAL *ff) {
  const uint64_t nTotal = (uint64_t)nO * nT * nP;
  const uint32_t iP = (uint32_t)(gti / ((uint64_t)nO * nT));
  const uint32_t iT = (uint32_t)((gti - (uint64_t)iP * nO * nT) / nO);
  const uint32_t iO = (uint32_t)(gti - (uint64_t)iP * nO * nT - (uint64_t)iT * nO);

  const REAL w = omega[iO];
  const REAL n0 = sinT[iT] * cosP[iP], n1 = sinT[iT] * sinP[iP], n2 = cosT[iT];
  /* theta-hat and phi-hat of synchrad/kernel_farfield.cl:385-388 */
  const REAL t0 = cosT[iT] * cosP[iP], t1 = cosT[iT] * sinP[iP], t2 = -sinT[iT];
  const REAL p0 = -sinP[iP], p1 = cosP[iP], p2 = (REAL)0.0;
  const REAL ffl = (comp == 2) ? ff[iO] : (REAL)1.0;

  const REAL dtInv = (REAL)1. / dt;
  const REAL wpdt2 = wp * dt * dt;
  const REAL wpdt = R_SQRT(wp) * dt;
  REAL phasePrev = (REAL)0.;
  REAL re0 = 0, re1 = 0, re2 = 0, im0 = 0, im1 = 0, im2 = 0;

  uint32_t k = SR_FN(first_snap)(itStart, nSnaps, itSnaps);
  for (uint32_t it = 0; it < itEnd - 1; it++) {
    const uint32_t itg = itStart + it;
    if (it < nSteps - 1) {
      const REAL time = (REAL)itg * dt;
      const REAL phase = w * (time - (x[it] * n0 + y[it] * n1 + z[it] * n2));
      const REAL dPhase = R_FABS(phase - phasePrev);
      phasePrev = phase;
      if (dPhase < (REAL)M_PI) {
        REAL g = (REAL)1. / R_SQRT((REAL)1. + (ux[it] * ux[it] + uy[it] * uy[it] +
                                               uz[it] * uz[it]));
        const REAL b0 = ux[it] * g, b1 = uy[it] * g, b2 = uz[it] * g;
        g = (REAL)1. / R_SQRT((REAL)1. + (ux[it + 1] * ux[it + 1] +
                                          uy[it + 1] * uy[it + 1] +
                                          uz[it + 1] * uz[it + 1]));
        const REAL bn0 = ux[it + 1] * g, bn1 = uy[it + 1] * g, bn2 = uz[it + 1] * g;
        const REAL a0 = (bn0 - b0) * dtInv, a1 = (bn1 - b1) * dtInv,
                   a2 = (bn2 - b2) * dtInv;
        const REAL m0 = (REAL)0.5 * (bn0 + b0), m1 = (REAL)0.5 * (bn1 + b1),
                   m2 = (REAL)0.5 * (bn2 + b2);
        REAL c1 = a0 * n0 + a1 * n1 + a2 * n2;
        REAL c2 = (REAL)1. - (m0 * n0 + m1 * n1 + m2 * n2);
        c2 = (REAL)1. / c2;
        c1 = c1 * c2 * c2;
        const REAL sn = R_SIN(phase), cs = R_COS(phase);
        REAL A0 = c1 * (n0 - m0) - c2 * a0;
        REAL A1 = c1 * (n1 - m1) - c2 * a1;
        REAL A2 = c1 * (n2 - m2) - c2 * a2;
        if (comp == 3 || comp == 4) {
          const REAL r = n0 * A0 + n1 * A1 + n2 * A2;
          const REAL th = t0 * A0 + t1 * A1 + t2 * A2;
          const REAL ph = p0 * A0 + p1 * A1 + p2 * A2;
          A0 = r; A1 = th; A2 = ph;
        }
        if (comp == 2) {
          re0 += A0 * cs * ffl; re1 += A1 * cs * ffl; re2 += A2 * cs * ffl;
          im0 += A0 * sn * ffl; im1 += A1 * sn * ffl; im2 += A2 * sn * ffl;
        } else {
          re0 += A0 * cs; re1 += A1 * cs; re2 += A2 * cs;
          im0 += A0 * sn; im1 += A1 * sn; im2 += A2 * sn;
        }
      }
    }
    if (k < nSnaps && itg + 2 == itSnaps[k]) {
      const uint64_t o = gti + nTotal * k;
      switch (comp) {
        case 0:
          sp[0][o] += wpdt2 * ((re0 * re0 + re1 * re1 + re2 * re2) +
                               (im0 * im0 + im1 * im1 + im2 * im2));
          break;
        case 1:
        case 3:
          sp[0][o] += wpdt2 * (re0 * re0 + im0 * im0);
          sp[1][o] += wpdt2 * (re1 * re1 + im1 * im1);
          sp[2][o] += wpdt2 * (re2 * re2 + im2 * im2);
          break;
        default: /* 2, 4: coherent components */
          sp[0][o] += wpdt * re0; sp[1][o] += wpdt * im0;
          sp[2][o] += wpdt * re1; sp[3][o] += wpdt * im1;
          sp[4][o] += wpdt * re2; sp[5][o] += wpdt * im2;
          break;
      }
      ++k;
    }
  }
}

/*
 * Near field, one screen point, one track: the loop of
 * synchrad/kernel_nearfield.cl:58-102 (total), :161-212 (cartesian_comps) and
 * :271-323 (cartesian_comps_complex, FormFactor passed but not applied).
 *   r = |P - x|,  phase = w (t + r),  n = (P - x)/r,  beta at step it
 *   A += (n/r^2 + i w (beta - n)/r) exp(i phase)
 */
static void SR_FN(near_point)(int comp, uint64_t gti, REAL *const *sp,
                              const REAL *x, const REAL *y, const REAL *z,
                              const REAL *ux, const REAL *uy, const REAL *uz,
                              REAL wp, uint32_t itStart, uint32_t itEnd,
                              uint32_t nSteps, const REAL *omega,
                              const REAL *radius, const REAL *sinP,
                              const REAL *cosP, REAL L, uint32_t nO,
                              uint32_t nR, uint32_t nP, REAL dt,
                              uint32_t nSnaps, const uint32_t *itSnaps) {
  const uint64_t nTotal = (uint64_t)nO * nR * nP;
  const uint32_t iP = (uint32_t)(gti / ((uint64_t)nO * nR));
  const uint32_t iR = (uint32_t)((gti - (uint64_t)iP * nO * nR) / nO);
  const uint32_t iO = (uint32_t)(gti - (uint64_t)iP * nO * nR - (uint64_t)iR * nO);

  const REAL w = omega[iO];
  const REAL P0 = radius[iR] * cosP[iP], P1 = radius[iR] * sinP[iP], P2 = L;
  const REAL wpdt2 = wp * dt * dt;
  const REAL wpdt = R_SQRT(wp) * dt;
  REAL phasePrev = (REAL)0.;
  REAL re0 = 0, re1 = 0, re2 = 0, im0 = 0, im1 = 0, im2 = 0;

  uint32_t k = SR_FN(first_snap)(itStart, nSnaps, itSnaps);
  for (uint32_t it = 0; it < itEnd - 1; it++) {
    const uint32_t itg = itStart + it;
    if (it < nSteps - 1) {
      const REAL time = (REAL)itg * dt;
      const REAL d0 = P0 - x[it], d1 = P1 - y[it], d2 = P2 - z[it];
      const REAL r = R_SQRT(d0 * d0 + d1 * d1 + d2 * d2);
      const REAL phase = w * (time + r);
      const REAL dPhase = R_FABS(phase - phasePrev);
      phasePrev = phase;
      if (dPhase < (REAL)M_PI) {
        const REAL rInv = (REAL)1. / r;
        const REAL n0 = rInv * d0, n1 = rInv * d1, n2 = rInv * d2;
        const REAL g = (REAL)1. / R_SQRT((REAL)1. + (ux[it] * ux[it] +
                                                     uy[it] * uy[it] +
                                                     uz[it] * uz[it]));
        const REAL b0 = ux[it] * g, b1 = uy[it] * g, b2 = uz[it] * g;
        const REAL sn = R_SIN(phase), cs = R_COS(phase);
        const REAL wr = w * rInv, rr = rInv * rInv;
        const REAL c10 = wr * (b0 - n0), c11 = wr * (b1 - n1), c12 = wr * (b2 - n2);
        const REAL c20 = rr * n0, c21 = rr * n1, c22 = rr * n2;
        re0 += -c10 * sn + c20 * cs; re1 += -c11 * sn + c21 * cs;
        re2 += -c12 * sn + c22 * cs;
        im0 += c10 * cs + c20 * sn; im1 += c11 * cs + c21 * sn;
        im2 += c12 * cs + c22 * sn;
      }
    }
    if (k < nSnaps && itg + 2 == itSnaps[k]) {
      const uint64_t o = gti + nTotal * k;
      switch (comp) {
        case 0:
          sp[0][o] += wpdt2 * ((re0 * re0 + re1 * re1 + re2 * re2) +
                               (im0 * im0 + im1 * im1 + im2 * im2));
          break;
        case 1:
          sp[0][o] += wpdt2 * (re0 * re0 + im0 * im0);
          sp[1][o] += wpdt2 * (re1 * re1 + im1 * im1);
          sp[2][o] += wpdt2 * (re2 * re2 + im2 * im2);
          break;
        default:
          sp[0][o] += wpdt * re0; sp[1][o] += wpdt * im0;
          sp[2][o] += wpdt * re1; sp[3][o] += wpdt * im1;
          sp[4][o] += wpdt * re2; sp[5][o] += wpdt * im2;
          break;
      }
      ++k;
    }
  }
}

static int SR_FN(far)(int comp, void *const *spectra, const void *const *trk,
                      double wp, uint32_t itStart, uint32_t itEnd,
                      uint32_t nSteps, const void *const *ax, uint32_t nO,
                      uint32_t nT, uint32_t nP, double dt, uint32_t nSnaps,
                      const uint32_t *itSnaps, const void *ff, int nthreads) {
  REAL *sp[6];
  for (int i = 0; i < 6; ++i) sp[i] = (REAL *)spectra[i];
  const REAL *x = (const REAL *)trk[0], *y = (const REAL *)trk[1],
             *z = (const REAL *)trk[2], *ux = (const REAL *)trk[3],
             *uy = (const REAL *)trk[4], *uz = (const REAL *)trk[5];
  const REAL *om = (const REAL *)ax[0], *sT = (const REAL *)ax[1],
             *cT = (const REAL *)ax[2], *sP = (const REAL *)ax[3],
             *cP = (const REAL *)ax[4];
  const int64_t n = (int64_t)nO * nT * nP;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t g = 0; g < n; ++g)
    SR_FN(far_point)(comp, (uint64_t)g, sp, x, y, z, ux, uy, uz, (REAL)wp,
                     itStart, itEnd, nSteps, om, sT, cT, sP, cP, nO, nT, nP,
                     (REAL)dt, nSnaps, itSnaps, (const REAL *)ff);
  return 0;
}

static int SR_FN(near)(int comp, void *const *spectra, const void *const *trk,
                       double wp, uint32_t itStart, uint32_t itEnd,
                       uint32_t nSteps, const void *const *ax, double L,
                       uint32_t nO, uint32_t nR, uint32_t nP, double dt,
                       uint32_t nSnaps, const uint32_t *itSnaps, int nthreads) {
  REAL *sp[6];
  for (int i = 0; i < 6; ++i) sp[i] = (REAL *)spectra[i];
  const REAL *x = (const REAL *)trk[0], *y = (const REAL *)trk[1],
             *z = (const REAL *)trk[2], *ux = (const REAL *)trk[3],
             *uy = (const REAL *)trk[4], *uz = (const REAL *)trk[5];
  const REAL *om = (const REAL *)ax[0], *rad = (const REAL *)ax[1],
             *sP = (const REAL *)ax[2], *cP = (const REAL *)ax[3];
  const int64_t n = (int64_t)nO * nR * nP;
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (int64_t g = 0; g < n; ++g)
    SR_FN(near_point)(comp, (uint64_t)g, sp, x, y, z, ux, uy, uz, (REAL)wp,
                      itStart, itEnd, nSteps, om, rad, sP, cP, (REAL)L, nO, nR,
                      nP, (REAL)dt, nSnaps, itSnaps);
  return 0;
}

#undef SR_FN
#undef SR_CAT
#undef SR_CAT2
