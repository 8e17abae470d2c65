// C ABI of synchrad_gb300 (declared in include/synchrad_gb300.h): argument
// validation, error reporting and dispatch to the kernels.
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "sr_common.cuh"
#include "sr_internal.h"

namespace sr {

namespace {
thread_local char g_err[1024] = "";
}

int fail(int code, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  if (e == cudaSuccess) return SR_OK;
  return fail(SR_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

void clear_error() { g_err[0] = '\0'; }

namespace {

int n_sm_of_current_device() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 148;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 148;
  return n;
}

int check_common(const sr_tracks *t, const sr_grid *g, int comp, int precision,
                 void *const *out) {
  if (!t || !g) return fail(SR_ERR_INVALID, "tracks and grid must not be NULL");
  if (g->mode != SR_MODE_FAR && g->mode != SR_MODE_NEAR)
    return fail(SR_ERR_INVALID, "unknown grid mode %u", g->mode);
  const int nout = n_outputs(comp);
  if (nout == 0) return fail(SR_ERR_INVALID, "unknown comp %d", comp);
  if (g->mode == SR_MODE_NEAR && comp > SR_COMP_CARTESIAN_COMPLEX)
    return fail(SR_ERR_INVALID, "comp %d is far-field only (spheric components)", comp);
  if (precision < SR_PREC_DOUBLE || precision > SR_PREC_DF)
    return fail(SR_ERR_INVALID, "unknown precision %d", precision);
  if (t->dtype > SR_DTYPE_F32 || g->dtype > SR_DTYPE_F32)
    return fail(SR_ERR_INVALID, "unknown dtype");
  if (precision == SR_PREC_DOUBLE && (t->dtype != SR_DTYPE_F64 || g->dtype != SR_DTYPE_F64))
    return fail(SR_ERR_INVALID, "SR_PREC_DOUBLE needs FP64 tracks and grid");
  if ((precision == SR_PREC_FLOAT || precision == SR_PREC_FLOAT_NATIVE) &&
      (t->dtype != SR_DTYPE_F32 || g->dtype != SR_DTYPE_F32))
    return fail(SR_ERR_INVALID, "SR_PREC_FLOAT needs FP32 tracks and grid");
  if (precision == SR_PREC_MIXED && g->dtype != SR_DTYPE_F64)
    return fail(SR_ERR_INVALID, "SR_PREC_MIXED needs an FP64 grid");
  if (precision == SR_PREC_DF && g->dtype != SR_DTYPE_F64)
    return fail(SR_ERR_INVALID, "SR_PREC_DF needs an FP64 grid");
  if (precision == SR_PREC_DF && g->mode != SR_MODE_FAR)
    return fail(SR_ERR_UNSUPPORTED, "SR_PREC_DF evaluates the far field only");
  if (!out) return fail(SR_ERR_INVALID, "out must not be NULL");
  for (int i = 0; i < nout; ++i)
    if (!out[i]) return fail(SR_ERR_INVALID, "output array %d is NULL", i);
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  if (P > 0xffffffffull)
    return fail(SR_ERR_INVALID, "grid of %llu points exceeds 32-bit point indices",
                (unsigned long long)P);
  if (P > 0 && (!g->omega || !g->axis1 || !g->sin_phi || !g->cos_phi ||
                (g->mode == SR_MODE_FAR && !g->axis2)))
    return fail(SR_ERR_INVALID, "grid axis pointer is NULL");
  if (comp == SR_COMP_CARTESIAN_COMPLEX && g->mode == SR_MODE_FAR && P > 0 && !g->form_factor)
    return fail(SR_ERR_INVALID, "cartesian_complex needs form_factor");
  if (t->n_tracks > 0) {
    if (!t->offsets || !t->x || !t->y || !t->z || !t->ux || !t->uy || !t->uz || !t->weight ||
        !t->it_start || !t->it_end)
      return fail(SR_ERR_INVALID, "track pointer is NULL");
    if (t->n_snaps > 0 && !t->snap_its) return fail(SR_ERR_INVALID, "snap_its is NULL");
    if (t->total_steps < 0) return fail(SR_ERR_INVALID, "negative total_steps");
    if (!(t->dt > 0.0) && !(t->dt < 0.0)) return fail(SR_ERR_INVALID, "dt must be non-zero");
  }
  return SR_OK;
}

FarMixedParams far_mixed_params(const sr_tracks *t, const sr_grid *g, int comp,
                                void *const *out) {
  FarMixedParams p;
  memset(&p, 0, sizeof(p));
  p.n_tracks = t->n_tracks;
  p.track_f32 = t->dtype == SR_DTYPE_F32;
  p.total_steps = t->total_steps;
  p.offsets = t->offsets;
  p.x = t->x; p.y = t->y; p.z = t->z;
  p.ux = t->ux; p.uy = t->uy; p.uz = t->uz;
  p.weight = t->weight;
  p.it_start = t->it_start; p.it_end = t->it_end; p.snap_its = t->snap_its;
  p.snap_stride = t->snap_stride; p.n_snaps = t->n_snaps;
  p.dt = t->dt;
  p.n_omega = g->n_omega; p.n_theta = g->n_theta; p.n_phi = g->n_phi;
  p.omega = (const double *)g->omega;
  p.sin_theta = (const double *)g->axis1;
  p.cos_theta = (const double *)g->axis2;
  p.sin_phi = (const double *)g->sin_phi;
  p.cos_phi = (const double *)g->cos_phi;
  p.form_factor = (const double *)g->form_factor;
  p.L_screen = g->L_screen;
  p.comp = comp;
  p.n_out = n_outputs(comp);
  for (int i = 0; i < p.n_out; ++i) p.out[i] = (double *)out[i];
  return p;
}

}  // namespace

// The checks and parameter packing of sr_spectrum, for other entry points of
// the library that evaluate the same mixed-precision far field.
int validate_spectrum_args(const sr_tracks *t, const sr_grid *g, int comp, int precision,
                           void *const *out) {
  return check_common(t, g, comp, precision, out);
}
FarMixedParams make_far_mixed_params(const sr_tracks *t, const sr_grid *g, int comp,
                                     void *const *out) {
  return far_mixed_params(t, g, comp, out);
}
int device_sm_count() { return n_sm_of_current_device(); }

}  // namespace sr

using namespace sr;

extern "C" const char *sr_last_error(void) { return g_err; }

extern "C" int sr_version(void) { return 100; }

extern "C" int64_t sr_workspace_bytes(const sr_tracks *t, const sr_grid *g, int comp,
                                      int precision) {
  clear_error();
  if (!t || !g) return fail(SR_ERR_INVALID, "tracks and grid must not be NULL");
  if (g->mode != SR_MODE_FAR && g->mode != SR_MODE_NEAR)
    return fail(SR_ERR_INVALID, "unknown grid mode %u", g->mode);
  const int nout = n_outputs(comp);
  if (nout == 0) return fail(SR_ERR_INVALID, "unknown comp %d", comp);
  if (g->mode == SR_MODE_NEAR && comp > SR_COMP_CARTESIAN_COMPLEX)
    return fail(SR_ERR_INVALID, "comp %d is far-field only (spheric components)", comp);
  if (precision < SR_PREC_DOUBLE || precision > SR_PREC_DF)
    return fail(SR_ERR_INVALID, "unknown precision %d", precision);
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  if (precision == SR_PREC_DF) {
    if (g->mode != SR_MODE_FAR)
      return fail(SR_ERR_UNSUPPORTED, "SR_PREC_DF evaluates the far field only");
    const FarMixedConfig cfg =
        far_df_choose(g->n_omega, g->n_theta * g->n_phi, t->n_tracks, device_sm_count());
    return (int64_t)far_df_workspace(t->total_steps, P, nout, t->n_snaps ? t->n_snaps : 1, cfg);
  }
  if (precision != SR_PREC_MIXED) return 0;
  const FarMixedConfig cfg = mixed_config(t, g, comp);
  if (g->mode == SR_MODE_FAR)
    return (int64_t)far_mixed_workspace(t->total_steps, P, nout, t->n_snaps ? t->n_snaps : 1, cfg);
  return (int64_t)near_mixed_workspace(t->total_steps, P, nout, t->n_snaps ? t->n_snaps : 1, cfg);
}

extern "C" int sr_workspace_status(const void *workspace, void *stream) {
  clear_error();
  if (!workspace) return fail(SR_ERR_INVALID, "workspace is NULL");
  cudaError_t e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "stream synchronize");
  int status = 0;
  e = cudaMemcpy(&status, workspace, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "status read");
  if (status == STATUS_WAIT_TIMEOUT)
    return fail(SR_ERR_TIMEOUT, "a kernel wait on a staged copy ran out of time");
  return SR_OK;
}

extern "C" int sr_spectrum(const sr_tracks *t, const sr_grid *g, int comp, int precision,
                           void *const *out, void *workspace, size_t workspace_bytes,
                           void *stream) {
  clear_error();
  int rc = check_common(t, g, comp, precision, out);
  if (rc) return rc;
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  if (P == 0 || t->n_tracks == 0 || t->n_snaps == 0) return SR_OK;
  cudaStream_t s = (cudaStream_t)stream;

  if (precision == SR_PREC_DF) {
    const FarMixedConfig cfg =
        far_df_choose(g->n_omega, g->n_theta * g->n_phi, t->n_tracks, device_sm_count());
    return launch_far_df(far_mixed_params(t, g, comp, out), cfg, workspace, workspace_bytes, s);
  }
  if (precision == SR_PREC_MIXED) {
    const FarMixedConfig cfg = mixed_config(t, g, comp);
    if (g->mode == SR_MODE_FAR)
      return launch_far_mixed(far_mixed_params(t, g, comp, out), cfg, workspace,
                              workspace_bytes, s);
    return launch_near_mixed(far_mixed_params(t, g, comp, out), cfg, workspace,
                             workspace_bytes, s);
  }

  PortParams p;
  memset(&p, 0, sizeof(p));
  p.n_tracks = t->n_tracks;
  p.offsets = t->offsets;
  p.x = t->x; p.y = t->y; p.z = t->z;
  p.ux = t->ux; p.uy = t->uy; p.uz = t->uz;
  p.weight = t->weight;
  p.it_start = t->it_start; p.it_end = t->it_end; p.snap_its = t->snap_its;
  p.snap_stride = t->snap_stride; p.n_snaps = t->n_snaps;
  p.dt = t->dt;
  p.n_omega = g->n_omega; p.n_1 = g->n_theta; p.n_phi = g->n_phi;
  p.omega = g->omega; p.axis1 = g->axis1; p.axis2 = g->axis2;
  p.sin_phi = g->sin_phi; p.cos_phi = g->cos_phi; p.form_factor = g->form_factor;
  p.L = g->L_screen;
  for (int i = 0; i < n_outputs(comp); ++i) p.out[i] = out[i];
  return launch_port(p, g->mode == SR_MODE_FAR ? 0 : 1, comp,
                     precision == SR_PREC_DOUBLE ? SR_DTYPE_F64 : SR_DTYPE_F32,
                     precision == SR_PREC_FLOAT_NATIVE, s);
}

// ---------------------------------------------------------------------------
// Per-track entry points (the reference kernels' argument lists).
// ---------------------------------------------------------------------------
namespace {

int per_track(int mode, int comp, int dtype, int native, void *const *spectra, const void *x,
              const void *y, const void *z, const void *ux, const void *uy, const void *uz,
              double wp, uint32_t itStart, uint32_t itEnd, uint32_t nSteps, const void *omega,
              const void *axis1, const void *axis2, const void *sinPhi, const void *cosPhi,
              double L, uint32_t nOmega, uint32_t n1, uint32_t nPhi, double dt, uint32_t nSnaps,
              const uint32_t *itSnaps, const void *formFactor, void *stream) {
  clear_error();
  if (dtype != SR_DTYPE_F64 && dtype != SR_DTYPE_F32)
    return fail(SR_ERR_INVALID, "dtype must be SR_DTYPE_F64 or SR_DTYPE_F32");
  if (itEnd == 0 || nSteps == 0)
    return fail(SR_ERR_INVALID,
                "itEnd and nSteps must be >= 1 (the reference's unsigned loop bounds wrap)");
  const uint64_t P = (uint64_t)nOmega * n1 * nPhi;
  if (P > 0xffffffffull) return fail(SR_ERR_INVALID, "grid exceeds 32-bit point indices");
  if (!x || !y || !z || !ux || !uy || !uz || !omega || !axis1 || !sinPhi || !cosPhi ||
      (mode == 0 && !axis2))
    return fail(SR_ERR_INVALID, "array argument is NULL");
  if (nSnaps > 0 && !itSnaps) return fail(SR_ERR_INVALID, "itSnaps is NULL");
  for (int i = 0; i < n_outputs(comp); ++i)
    if (!spectra[i]) return fail(SR_ERR_INVALID, "spectrum array %d is NULL", i);
  if (comp == SR_COMP_CARTESIAN_COMPLEX && mode == 0 && !formFactor)
    return fail(SR_ERR_INVALID, "FormFactor is NULL");
  PortParams p;
  memset(&p, 0, sizeof(p));
  p.n_tracks = 1;
  p.offsets = nullptr;
  p.x = x; p.y = y; p.z = z; p.ux = ux; p.uy = uy; p.uz = uz;
  p.wp1 = wp; p.it_start1 = itStart; p.it_end1 = itEnd; p.n_steps1 = nSteps;
  p.snap_its = itSnaps; p.snap_stride = 0; p.n_snaps = nSnaps;
  p.dt = dt;
  p.n_omega = nOmega; p.n_1 = n1; p.n_phi = nPhi;
  p.omega = omega; p.axis1 = axis1; p.axis2 = axis2; p.sin_phi = sinPhi; p.cos_phi = cosPhi;
  p.form_factor = formFactor;
  p.L = L;
  for (int i = 0; i < n_outputs(comp); ++i) p.out[i] = spectra[i];
  if (P == 0 || nSnaps == 0) return SR_OK;
  return launch_port(p, mode, comp, dtype, native != 0, (cudaStream_t)stream);
}

}  // namespace

#define SR_FAR_ARGS                                                                    \
  x, y, z, ux, uy, uz, wp, itStart, itEnd, nSteps, omega, sinTheta, cosTheta, sinPhi, \
      cosPhi, 0.0, nOmega, nTheta, nPhi, dt, nSnaps, itSnaps

extern "C" int sr_far_total(int dtype, int native, void *spectrum, const void *x,
                            const void *y, const void *z, const void *ux, const void *uy,
                            const void *uz, double wp, uint32_t itStart, uint32_t itEnd,
                            uint32_t nSteps, const void *omega, const void *sinTheta,
                            const void *cosTheta, const void *sinPhi, const void *cosPhi,
                            uint32_t nOmega, uint32_t nTheta, uint32_t nPhi, double dt,
                            uint32_t nSnaps, const uint32_t *itSnaps, void *stream) {
  void *sp[6] = {spectrum};
  return per_track(0, SR_COMP_TOTAL, dtype, native, sp, SR_FAR_ARGS, nullptr, stream);
}

extern "C" int sr_far_cartesian_comps(int dtype, int native, void *s1, void *s2, void *s3,
                                      const void *x, const void *y, const void *z,
                                      const void *ux, const void *uy, const void *uz,
                                      double wp, uint32_t itStart, uint32_t itEnd,
                                      uint32_t nSteps, const void *omega,
                                      const void *sinTheta, const void *cosTheta,
                                      const void *sinPhi, const void *cosPhi, uint32_t nOmega,
                                      uint32_t nTheta, uint32_t nPhi, double dt,
                                      uint32_t nSnaps, const uint32_t *itSnaps, void *stream) {
  void *sp[6] = {s1, s2, s3};
  return per_track(0, SR_COMP_CARTESIAN, dtype, native, sp, SR_FAR_ARGS, nullptr, stream);
}

extern "C" int sr_far_cartesian_comps_complex(
    int dtype, int native, void *s1r, void *s1i, void *s2r, void *s2i, void *s3r, void *s3i,
    const void *x, const void *y, const void *z, const void *ux, const void *uy, const void *uz,
    double wp, uint32_t itStart, uint32_t itEnd, uint32_t nSteps, const void *omega,
    const void *sinTheta, const void *cosTheta, const void *sinPhi, const void *cosPhi,
    uint32_t nOmega, uint32_t nTheta, uint32_t nPhi, double dt, uint32_t nSnaps,
    const uint32_t *itSnaps, const void *FormFactor, void *stream) {
  void *sp[6] = {s1r, s1i, s2r, s2i, s3r, s3i};
  return per_track(0, SR_COMP_CARTESIAN_COMPLEX, dtype, native, sp, SR_FAR_ARGS, FormFactor,
                   stream);
}

extern "C" int sr_far_spheric_comps(int dtype, int native, void *s1, void *s2, void *s3,
                                    const void *x, const void *y, const void *z, const void *ux,
                                    const void *uy, const void *uz, double wp, uint32_t itStart,
                                    uint32_t itEnd, uint32_t nSteps, const void *omega,
                                    const void *sinTheta, const void *cosTheta,
                                    const void *sinPhi, const void *cosPhi, uint32_t nOmega,
                                    uint32_t nTheta, uint32_t nPhi, double dt, uint32_t nSnaps,
                                    const uint32_t *itSnaps, void *stream) {
  void *sp[6] = {s1, s2, s3};
  return per_track(0, SR_COMP_SPHERIC, dtype, native, sp, SR_FAR_ARGS, nullptr, stream);
}

extern "C" int sr_far_spheric_comps_complex(
    int dtype, int native, void *s1r, void *s1i, void *s2r, void *s2i, void *s3r, void *s3i,
    const void *x, const void *y, const void *z, const void *ux, const void *uy, const void *uz,
    double wp, uint32_t itStart, uint32_t itEnd, uint32_t nSteps, const void *omega,
    const void *sinTheta, const void *cosTheta, const void *sinPhi, const void *cosPhi,
    uint32_t nOmega, uint32_t nTheta, uint32_t nPhi, double dt, uint32_t nSnaps,
    const uint32_t *itSnaps, const void *FormFactor, void *stream) {
  (void)FormFactor;  // accepted, not applied (synchrad/kernel_farfield.cl:499, 576-577)
  void *sp[6] = {s1r, s1i, s2r, s2i, s3r, s3i};
  return per_track(0, SR_COMP_SPHERIC_COMPLEX, dtype, native, sp, SR_FAR_ARGS, nullptr, stream);
}

#define SR_NEAR_ARGS                                                                      \
  x, y, z, ux, uy, uz, wp, itStart, itEnd, nSteps, omega, radius, nullptr, sinPhi, cosPhi, \
      distanceToScreen, nOmega, nRadius, nPhi, dt, nSnaps, itSnaps

extern "C" int sr_near_total(int dtype, int native, void *spectrum, const void *x,
                             const void *y, const void *z, const void *ux, const void *uy,
                             const void *uz, double wp, uint32_t itStart, uint32_t itEnd,
                             uint32_t nSteps, const void *omega, const void *radius,
                             const void *sinPhi, const void *cosPhi, double distanceToScreen,
                             uint32_t nOmega, uint32_t nRadius, uint32_t nPhi, double dt,
                             uint32_t nSnaps, const uint32_t *itSnaps, void *stream) {
  void *sp[6] = {spectrum};
  return per_track(1, SR_COMP_TOTAL, dtype, native, sp, SR_NEAR_ARGS, nullptr, stream);
}

extern "C" int sr_near_cartesian_comps(int dtype, int native, void *s1, void *s2, void *s3,
                                       const void *x, const void *y, const void *z,
                                       const void *ux, const void *uy, const void *uz,
                                       double wp, uint32_t itStart, uint32_t itEnd,
                                       uint32_t nSteps, const void *omega, const void *radius,
                                       const void *sinPhi, const void *cosPhi,
                                       double distanceToScreen, uint32_t nOmega,
                                       uint32_t nRadius, uint32_t nPhi, double dt,
                                       uint32_t nSnaps, const uint32_t *itSnaps, void *stream) {
  void *sp[6] = {s1, s2, s3};
  return per_track(1, SR_COMP_CARTESIAN, dtype, native, sp, SR_NEAR_ARGS, nullptr, stream);
}

extern "C" int sr_near_cartesian_comps_complex(
    int dtype, int native, void *s1r, void *s1i, void *s2r, void *s2i, void *s3r, void *s3i,
    const void *x, const void *y, const void *z, const void *ux, const void *uy, const void *uz,
    double wp, uint32_t itStart, uint32_t itEnd, uint32_t nSteps, const void *omega,
    const void *radius, const void *sinPhi, const void *cosPhi, double distanceToScreen,
    uint32_t nOmega, uint32_t nRadius, uint32_t nPhi, double dt, uint32_t nSnaps,
    const uint32_t *itSnaps, const void *FormFactor, void *stream) {
  (void)FormFactor;  // accepted, not applied (synchrad/kernel_nearfield.cl:244, 306-307)
  void *sp[6] = {s1r, s1i, s2r, s2i, s3r, s3i};
  return per_track(1, SR_COMP_CARTESIAN_COMPLEX, dtype, native, sp, SR_NEAR_ARGS, nullptr,
                   stream);
}
