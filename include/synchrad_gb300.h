/*
 * synchrad_gb300: C ABI of the GB300 (sm_103a) radiation-integral library.
 *
 * The library evaluates SynchRad's far-field (Lienard-Wiechert spectral sum
 * over track steps, per (omega, theta, phi) point) and near-field (screen at a
 * finite distance) integrals on the GPU.  All pointers named "device" are CUDA
 * device pointers owned by the caller.  Three diagnostics and tuning calls
 * allocate: sr_autotune (device scratch and outputs for its trial runs, freed
 * before it returns), sr_probe_fp32_peak (a 16-byte stream-ordered buffer) and
 * sr_graph_create (a private stream and the graph objects); no other entry
 * point allocates device memory.
 * Every entry point is stream-ordered on `stream` (a cudaStream_t, NULL for the
 * legacy default stream), returns SR_OK or a negative SR_ERR_* code, and leaves
 * a message for sr_last_error() on failure.  Output spectra are accumulated in
 * place (+=), as the reference kernels do.
 *
 * Spectrum layout on the device (the reference's, synchrad/calc.py:455-456):
 *   out[k][iPhi][iTheta|iR][iOmega],  k < n_snaps,
 * i.e. point index gti = iOmega + nOmega*(iTheta + nTheta*iPhi).
 */
#ifndef SYNCHRAD_GB300_H
#define SYNCHRAD_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  SR_OK = 0,
  SR_ERR_INVALID = -1,     /* bad argument (null pointer, size, combination) */
  SR_ERR_UNSUPPORTED = -2, /* valid but not implemented for this mode/comp */
  SR_ERR_CUDA = -3,        /* a CUDA launch or runtime call failed */
  SR_ERR_WORKSPACE = -4,   /* workspace missing or smaller than required */
  SR_ERR_TIMEOUT = -5      /* a kernel wait ran out of time (see sr_workspace_status) */
};

enum { SR_DTYPE_F64 = 0, SR_DTYPE_F32 = 1 };
enum { SR_MODE_FAR = 0, SR_MODE_NEAR = 1 };

/* `comp` of calculate_spectrum (synchrad/calc.py:133-144, 458-465). */
enum {
  SR_COMP_TOTAL = 0,             /* 1 output:  sum_tracks w dt^2 |A|^2 */
  SR_COMP_CARTESIAN = 1,         /* 3 outputs: |A_x|^2, |A_y|^2, |A_z|^2 */
  SR_COMP_CARTESIAN_COMPLEX = 2, /* 6 outputs: sqrt(w) dt Re/Im A_{x,y,z} */
  SR_COMP_SPHERIC = 3,           /* 3 outputs: |A_r|^2, |A_theta|^2, |A_phi|^2 (far) */
  SR_COMP_SPHERIC_COMPLEX = 4    /* 6 outputs: sqrt(w) dt Re/Im A_{r,theta,phi} (far) */
};

/* Arithmetic of one evaluation. */
enum {
  SR_PREC_DOUBLE = 0,       /* FP64 throughout: the plain port of the reference kernel */
  SR_PREC_FLOAT = 1,        /* FP32 throughout: the reference's dtype='float' */
  SR_PREC_FLOAT_NATIVE = 2, /* FP32 with fast intrinsics: dtype='float' + 'native' */
  SR_PREC_MIXED = 3,        /* FP32 bulk, double-float phase, compensated sums, FP64 spectrum */
  SR_PREC_DF = 4            /* double-float throughout (~48 bits) on the FP32 pipe: FP64-class
                               spectra for losses that amplify the forward error; far field,
                               F64 grid, F64 or F32 tracks.  No counterpart in the reference. */
};

/*
 * A batch of tracks in CSR form.  Track t owns steps offsets[t] .. offsets[t+1]-1
 * of the concatenated arrays x..uz.  Per-track values mirror one reference
 * kernel launch (synchrad/calc.py:306-322): wp = weight[t], itStart =
 * it_start[t], itEnd = it_end[t], nSteps = offsets[t+1]-offsets[t], and the
 * snapshot iterations row snap_its[t*snap_stride .. + n_snaps) (snap_stride 0:
 * one row shared by every track, the it_range case).
 */
typedef struct sr_tracks {
  uint32_t n_tracks;
  uint32_t dtype;           /* SR_DTYPE_F64 | SR_DTYPE_F32: element type of x..uz */
  int64_t total_steps;      /* host copy of offsets[n_tracks] */
  const int64_t *offsets;   /* device [n_tracks + 1], offsets[0] == 0 */
  const void *x, *y, *z;    /* device [total_steps] positions (c = 1 units) */
  const void *ux, *uy, *uz; /* device [total_steps] momenta gamma*beta */
  const double *weight;     /* device [n_tracks] */
  const uint32_t *it_start; /* device [n_tracks] */
  const uint32_t *it_end;   /* device [n_tracks] */
  const uint32_t *snap_its; /* device, see above */
  uint32_t snap_stride;
  uint32_t n_snaps;
  double dt;                /* c*dt, the reference's timeStep */
} sr_tracks;

/*
 * The spectral grid as the reference uploads it (synchrad/calc.py:486-512):
 * omega already multiplied by 2*pi; far field: sinTheta, cosTheta, sinPhi,
 * cosPhi; near field: radius, sinPhi, cosPhi and the screen distance.
 */
typedef struct sr_grid {
  uint32_t mode;            /* SR_MODE_FAR | SR_MODE_NEAR */
  uint32_t dtype;           /* element type of the axis arrays */
  uint32_t n_omega;
  uint32_t n_theta;         /* n_R in near mode */
  uint32_t n_phi;
  uint32_t reserved;
  const void *omega;        /* device [n_omega] */
  const void *axis1;        /* device: far sinTheta [n_theta], near radius [n_R] */
  const void *axis2;        /* device: far cosTheta [n_theta], near unused */
  const void *sin_phi;      /* device [n_phi] */
  const void *cos_phi;      /* device [n_phi] */
  const void *form_factor;  /* device [n_omega]; used by far cartesian_complex only */
  double L_screen;          /* near mode: distance to the screen */
} sr_grid;

/* ---------------------------------------------------------------------------
 * Batched evaluation: the GB300-native entry point.
 *
 * Replaces the per-track loop of SynchRad.calculate_spectrum
 * (synchrad/calc.py:257-267) and the kernel launches it makes
 * (synchrad/calc.py:324-353): one call evaluates every track of the batch and
 * accumulates the incoherent (or coherent, for *_complex) sum into `out`.
 *   out:  n_out device arrays (1, 3 or 6 by comp), element type double for
 *         SR_PREC_DOUBLE / SR_PREC_MIXED and float for SR_PREC_FLOAT*.
 *   workspace: device scratch of at least sr_workspace_bytes(...) bytes,
 *         256-byte aligned (NULL allowed when that size is 0).
 * Track and grid element types: SR_PREC_DOUBLE needs F64 tracks and grid,
 * SR_PREC_FLOAT* need F32 tracks and grid, SR_PREC_MIXED takes F64 or F32
 * tracks with an F64 grid.
 * ------------------------------------------------------------------------- */
int sr_spectrum(const sr_tracks *tracks, const sr_grid *grid, int comp,
                int precision, void *const *out, void *workspace,
                size_t workspace_bytes, void *stream);

/* The mixed-precision far field of sr_spectrum without any device allocation.
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory themselves (code embedded in a host application that owns every
 * allocation and hands over only input and output buffers): the scratch lives
 * in a 64 MiB array compiled into this library, held by every GPU that loads
 * it until the process exits.  Sizes whose scratch (80 B per track step, 8 B
 * per point x output x snapshot, plus per-CTA sums) exceeds it are rejected
 * with SR_ERR_INVALID.  The first call on a device looks up the array's device
 * address (make it before any stream capture); that address is kept for the
 * process and does not survive cudaDeviceReset.  Calls that overlap on the GPU
 * share the array and race.  Far field only; outputs are double, accumulated.
 * A bounded kernel wait that ran out of time is reported by sr_noalloc_status,
 * not by the return code. */
int sr_spectrum_noalloc(const sr_tracks *tracks, const sr_grid *grid, int comp,
                        void *const *out, void *stream);

/* Synchronises `stream` and reads the kernels' status word of the last
 * sr_spectrum_noalloc call on the current device (it lives in the static
 * array; the next call clears it): SR_OK, or SR_ERR_TIMEOUT if a bounded wait
 * expired and that call's outputs are incomplete.  Allocates nothing.  No
 * counterpart in the reference. */
int sr_noalloc_status(void *stream);

/* Scratch bytes sr_spectrum needs for these sizes (reads host fields only):
 * 0 for SR_PREC_DOUBLE and SR_PREC_FLOAT*, which need none; SR_ERR_INVALID
 * (negative, with a message) for NULL arguments, an unknown mode, comp or
 * precision, or a spheric comp on a near-field grid. */
int64_t sr_workspace_bytes(const sr_tracks *tracks, const sr_grid *grid,
                           int comp, int precision);

/* Synchronises `stream` and reads the kernels' status word from a workspace
 * used by sr_spectrum: SR_OK, or SR_ERR_TIMEOUT if a bounded wait expired. */
int sr_workspace_status(const void *workspace, void *stream);

/* Message of the last failure on the calling thread ("" if none). */
const char *sr_last_error(void);

/* Library version, major*10000 + minor*100 + patch. */
int sr_version(void);

/* ---------------------------------------------------------------------------
 * Work shape autotuning and CUDA graphs.  No counterpart in the reference
 * (its host loop launches one OpenCL kernel per track, synchrad/calc.py:257-267).
 * ------------------------------------------------------------------------- */

/* Work shape of the persistent mixed-precision launch. */
typedef struct sr_config {
  int32_t points_per_lane;      /* omega points each lane carries (far: 8..32) */
  int32_t lanes_per_direction;  /* lanes sharing one direction's omega axis */
  int32_t steps_per_stage;      /* step records per TMA stage (far field) */
  int32_t track_subsets;        /* tracks are split into this many subsets */
  int32_t ctas;                 /* CTAs of the persistent launch */
  int32_t reserved;
  double ms;                    /* time on the tuning sample (0: not timed) */
} sr_config;

/* Times candidate work shapes (points per lane and lanes per direction, then
 * steps per stage, then track subsets) with CUDA events on a sample of the
 * problem (its leading tracks, about budget_ms / 100 of work each run) and
 * caches the fastest for problems of exactly these sizes; later sr_spectrum
 * and sr_workspace_bytes calls for such problems use it (query the workspace
 * size after tuning).  Allocates and frees its own scratch; stops starting new
 * candidates once budget_ms (<= 0: 3000) has passed.  best / dflt (either may
 * be NULL) receive the chosen and the default shape with their sample times.
 * Runs on `stream` and synchronises it: the track arrays may still be
 * arriving by copies that `stream` waits for (the offsets are read on it).
 * SR_PREC_MIXED only. */
int sr_autotune(const sr_tracks *tracks, const sr_grid *grid, int comp, int precision,
                double budget_ms, void *stream, sr_config *best, sr_config *dflt);

/* The work shape sr_spectrum uses for this problem (tuned or default). */
int sr_config_get(const sr_tracks *tracks, const sr_grid *grid, int comp, int precision,
                  sr_config *out);

/* Pins a work shape for problems of exactly these sizes (for instance one
 * tuned in an earlier process): points_per_lane (far 8/16/24/32, near 8/16),
 * lanes_per_direction (8/16/32), steps_per_stage (far: multiple of 32 in
 * [32, 512]) and track_subsets (0: default, at most 64) are used, the rest is
 * derived.  A shape whose shared memory would exceed a CTA's 227 KB is
 * refused with SR_ERR_INVALID. */
int sr_config_set(const sr_tracks *tracks, const sr_grid *grid, int comp, int precision,
                  const sr_config *config);

/* Forgets every tuned work shape. */
int sr_config_clear(void);

/* One sr_spectrum call (all its copies and kernels) captured into a CUDA graph
 * on a private stream and instantiated; sr_graph_launch replays it on any
 * stream, accumulating into the same `out` from the same device buffers (the
 * track, grid, output and workspace pointers are baked in). */
typedef struct sr_graph sr_graph;
int sr_graph_create(const sr_tracks *tracks, const sr_grid *grid, int comp, int precision,
                    void *const *out, void *workspace, size_t workspace_bytes,
                    sr_graph **graph);
int sr_graph_launch(sr_graph *graph, void *stream);
/* Kernel nodes and all nodes of the captured graph. */
int sr_graph_nodes(const sr_graph *graph, int *n_kernels, int *n_nodes);
void sr_graph_destroy(sr_graph *graph);

/* ---------------------------------------------------------------------------
 * Adjoint of the far field (mixed or double-float forward), one snapshot.
 * No counterpart in the reference (it has no gradients).  The |dphase| < pi
 * mask is held fixed; uniform and non-uniform omega axes.
 * ------------------------------------------------------------------------- */

/* sr_spectrum (SR_PREC_MIXED, far, SR_COMP_TOTAL, n_snaps = 1) that also
 * records each track's A_theta, A_phi per point in saved_A
 * ([n_tracks][P][4] float, written) for sr_far_total_backward.  Same
 * workspace as sr_spectrum. */
int sr_far_total_forward_saved(const sr_tracks *tracks, const sr_grid *grid,
                               double *spectrum, float *saved_A, void *workspace,
                               size_t workspace_bytes, void *stream);

/* The same in double-float arithmetic (SR_PREC_DF): the spectrum to FP64-class
 * accuracy, saved_A (float) as above.  Workspace: sr_workspace_bytes(...,
 * SR_COMP_TOTAL, SR_PREC_DF).  For losses that amplify the forward error, such
 * as a misfit S - T that is a small fraction of S. */
int sr_far_total_forward_saved_df(const sr_tracks *tracks, const sr_grid *grid,
                                  double *spectrum, float *saved_A, void *workspace,
                                  size_t workspace_bytes, void *stream);

/* Scratch bytes of sr_far_total_backward for these sizes. */
int64_t sr_far_total_backward_workspace_bytes(const sr_tracks *tracks,
                                              const sr_grid *grid);

/* Given dL/dS (grad_spectrum, [P] doubles in the device layout) and the
 * forward's saved_A, writes dL/dx, dL/dy, dL/dz, dL/dux, dL/duy, dL/duz
 * (grad_track[0..5], [total_steps] doubles each) and dL/dw (grad_weight,
 * [n_tracks]).  Phases are recomputed, not stored. */
int sr_far_total_backward(const sr_tracks *tracks, const sr_grid *grid,
                          const double *grad_spectrum, const float *saved_A,
                          double *const *grad_track, double *grad_weight,
                          void *workspace, size_t workspace_bytes, void *stream);

/* Every far-field comp (the reference's five far kernels,
 * synchrad/kernel_farfield.cl:6-595), one snapshot: the forward of comp `comp`
 * in `precision` (SR_PREC_MIXED or SR_PREC_DF) into its n_out outputs (double,
 * accumulated), recording saved_A as above; workspace: sr_workspace_bytes of
 * that comp and precision.  The backward takes dL/dS_k for each output
 * (grad_out[k], [P] doubles) and writes the same gradients as
 * sr_far_total_backward.  Quadratic comps (total, cartesian, spheric) and the
 * coherent *_complex comps (linear in A: their dL/dw follows sqrt(w)); the
 * spheric radial outputs are identically zero and carry no gradient.  Its
 * workspace is sr_far_backward_workspace_bytes (the same for every comp). */
int sr_far_forward_saved(const sr_tracks *tracks, const sr_grid *grid, int comp, int precision,
                         void *const *out, float *saved_A, void *workspace,
                         size_t workspace_bytes, void *stream);
int64_t sr_far_backward_workspace_bytes(const sr_tracks *tracks, const sr_grid *grid);
int sr_far_backward(const sr_tracks *tracks, const sr_grid *grid, int comp,
                    const double *const *grad_out, const float *saved_A,
                    double *const *grad_track, double *grad_weight, void *workspace,
                    size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Adjoint of the mixed-precision near field (screen at distance L), comp
 * 'total', one snapshot.  No counterpart in the reference.  Same conventions
 * as the far-field adjoint above; saved_A is [n_tracks][P][8] float
 * (A_x, A_y, A_z as re, im pairs, then two floats of padding).
 * ------------------------------------------------------------------------- */
int sr_near_total_forward_saved(const sr_tracks *tracks, const sr_grid *grid,
                                double *spectrum, float *saved_A, void *workspace,
                                size_t workspace_bytes, void *stream);
int64_t sr_near_total_backward_workspace_bytes(const sr_tracks *tracks,
                                               const sr_grid *grid);
int sr_near_total_backward(const sr_tracks *tracks, const sr_grid *grid,
                           const double *grad_spectrum, const float *saved_A,
                           double *const *grad_track, double *grad_weight,
                           void *workspace, size_t workspace_bytes, void *stream);

/* Every near-field comp (total, cartesian, cartesian_complex:
 * synchrad/kernel_nearfield.cl:5-326), one snapshot, as sr_far_forward_saved /
 * sr_far_backward: outputs and their gradients per comp; saved_A as for
 * sr_near_total_forward_saved.  cartesian_complex outputs (sqrt(w) dt Re/Im
 * of e^{i omega L} A_k) are linear in A.  No counterpart in the reference. */
int sr_near_forward_saved(const sr_tracks *tracks, const sr_grid *grid, int comp,
                          void *const *out, float *saved_A, void *workspace,
                          size_t workspace_bytes, void *stream);
int64_t sr_near_backward_workspace_bytes(const sr_tracks *tracks, const sr_grid *grid);
int sr_near_backward(const sr_tracks *tracks, const sr_grid *grid, int comp,
                     const double *const *grad_out, const float *saved_A,
                     double *const *grad_track, double *grad_weight, void *workspace,
                     size_t workspace_bytes, void *stream);

/* ---------------------------------------------------------------------------
 * Diagnostics.  These have no counterpart in the reference; the benchmark uses
 * them for its roofline figures.
 * ------------------------------------------------------------------------- */

/* While enabled, every sr_spectrum / per-track call records CUDA events around
 * its dominant kernel on the call's stream. */
int sr_timing_enable(int enable);

/* Waits for the recorded events, returns their summed duration (ms) and count,
 * and clears the record. */
int sr_timing_read(double *total_ms, int *n_launches);

/* Measures this device's FP32 fused-multiply-add throughput (TFLOP/s, 2 flops
 * per FMA) with scalar FFMA and with packed FFMA2 instructions. */
int sr_probe_fp32_peak(double *tflops_scalar, double *tflops_packed, void *stream);

/* Failure-path self-test: launches a one-warp kernel whose bounded wait (the
 * mbarrier wait every kernel of the library uses) is on a barrier nothing
 * completes, with a limit of limit_ns (1 .. 1e9); the kernel records the
 * timeout in the status word at the start of `workspace` (>= 4 bytes) as the
 * spectrum kernels do, and sr_workspace_status then returns SR_ERR_TIMEOUT.
 * With `workspace` NULL the target is the status word of sr_spectrum_noalloc's
 * static array, read back by sr_noalloc_status.
 * No copy is issued and the context stays usable. */
int sr_selftest_wait_timeout(int64_t limit_ns, void *workspace, void *stream);

/* ---------------------------------------------------------------------------
 * Per-track entry points: the reference's OpenCL kernels, one launch each.
 *
 * Same argument order and meaning as the kernels in
 * synchrad/kernel_farfield.cl and synchrad/kernel_nearfield.cl as
 * synchrad/calc.py:306-353 binds them, with `dtype` (SR_DTYPE_F64 or
 * SR_DTYPE_F32, the Mako ${my_dtype}) as the first argument and the stream as
 * the last.  Every array argument has element type `dtype`; `native` selects
 * the ${f_native} intrinsics for SR_DTYPE_F32.  No workspace is needed.
 * ------------------------------------------------------------------------- */

/* synchrad/kernel_farfield.cl:6-28 `total` */
int sr_far_total(int dtype, int native, void *spectrum, const void *x,
                 const void *y, const void *z, const void *ux, const void *uy,
                 const void *uz, double wp, uint32_t itStart, uint32_t itEnd,
                 uint32_t nSteps, const void *omega, const void *sinTheta,
                 const void *cosTheta, const void *sinPhi, const void *cosPhi,
                 uint32_t nOmega, uint32_t nTheta, uint32_t nPhi, double dt,
                 uint32_t nSnaps, const uint32_t *itSnaps, void *stream);

/* synchrad/kernel_farfield.cl:111-135 `cartesian_comps` */
int sr_far_cartesian_comps(int dtype, int native, void *spectrum1,
                           void *spectrum2, void *spectrum3, const void *x,
                           const void *y, const void *z, const void *ux,
                           const void *uy, const void *uz, double wp,
                           uint32_t itStart, uint32_t itEnd, uint32_t nSteps,
                           const void *omega, const void *sinTheta,
                           const void *cosTheta, const void *sinPhi,
                           const void *cosPhi, uint32_t nOmega,
                           uint32_t nTheta, uint32_t nPhi, double dt,
                           uint32_t nSnaps, const uint32_t *itSnaps,
                           void *stream);

/* synchrad/kernel_farfield.cl:227-255 `cartesian_comps_complex` */
int sr_far_cartesian_comps_complex(
    int dtype, int native, void *spectrum1_re, void *spectrum1_im,
    void *spectrum2_re, void *spectrum2_im, void *spectrum3_re,
    void *spectrum3_im, const void *x, const void *y, const void *z,
    const void *ux, const void *uy, const void *uz, double wp,
    uint32_t itStart, uint32_t itEnd, uint32_t nSteps, const void *omega,
    const void *sinTheta, const void *cosTheta, const void *sinPhi,
    const void *cosPhi, uint32_t nOmega, uint32_t nTheta, uint32_t nPhi,
    double dt, uint32_t nSnaps, const uint32_t *itSnaps,
    const void *FormFactor, void *stream);

/* synchrad/kernel_farfield.cl:346-370 `spheric_comps` */
int sr_far_spheric_comps(int dtype, int native, void *spectrum1,
                         void *spectrum2, void *spectrum3, const void *x,
                         const void *y, const void *z, const void *ux,
                         const void *uy, const void *uz, double wp,
                         uint32_t itStart, uint32_t itEnd, uint32_t nSteps,
                         const void *omega, const void *sinTheta,
                         const void *cosTheta, const void *sinPhi,
                         const void *cosPhi, uint32_t nOmega, uint32_t nTheta,
                         uint32_t nPhi, double dt, uint32_t nSnaps,
                         const uint32_t *itSnaps, void *stream);

/* synchrad/kernel_farfield.cl:471-499 `spheric_comps_complex`
 * (FormFactor is accepted and, as in the reference, not applied) */
int sr_far_spheric_comps_complex(
    int dtype, int native, void *spectrum1_re, void *spectrum1_im,
    void *spectrum2_re, void *spectrum2_im, void *spectrum3_re,
    void *spectrum3_im, const void *x, const void *y, const void *z,
    const void *ux, const void *uy, const void *uz, double wp,
    uint32_t itStart, uint32_t itEnd, uint32_t nSteps, const void *omega,
    const void *sinTheta, const void *cosTheta, const void *sinPhi,
    const void *cosPhi, uint32_t nOmega, uint32_t nTheta, uint32_t nPhi,
    double dt, uint32_t nSnaps, const uint32_t *itSnaps,
    const void *FormFactor, void *stream);

/* synchrad/kernel_nearfield.cl:5-27 `total` */
int sr_near_total(int dtype, int native, void *spectrum, const void *x,
                  const void *y, const void *z, const void *ux, const void *uy,
                  const void *uz, double wp, uint32_t itStart, uint32_t itEnd,
                  uint32_t nSteps, const void *omega, const void *radius,
                  const void *sinPhi, const void *cosPhi,
                  double distanceToScreen, uint32_t nOmega, uint32_t nRadius,
                  uint32_t nPhi, double dt, uint32_t nSnaps,
                  const uint32_t *itSnaps, void *stream);

/* synchrad/kernel_nearfield.cl:106-130 `cartesian_comps` */
int sr_near_cartesian_comps(int dtype, int native, void *spectrum1,
                            void *spectrum2, void *spectrum3, const void *x,
                            const void *y, const void *z, const void *ux,
                            const void *uy, const void *uz, double wp,
                            uint32_t itStart, uint32_t itEnd, uint32_t nSteps,
                            const void *omega, const void *radius,
                            const void *sinPhi, const void *cosPhi,
                            double distanceToScreen, uint32_t nOmega,
                            uint32_t nRadius, uint32_t nPhi, double dt,
                            uint32_t nSnaps, const uint32_t *itSnaps,
                            void *stream);

/* synchrad/kernel_nearfield.cl:216-244 `cartesian_comps_complex`
 * (FormFactor is accepted and, as in the reference, not applied) */
int sr_near_cartesian_comps_complex(
    int dtype, int native, void *spectrum1_re, void *spectrum1_im,
    void *spectrum2_re, void *spectrum2_im, void *spectrum3_re,
    void *spectrum3_im, const void *x, const void *y, const void *z,
    const void *ux, const void *uy, const void *uz, double wp,
    uint32_t itStart, uint32_t itEnd, uint32_t nSteps, const void *omega,
    const void *radius, const void *sinPhi, const void *cosPhi,
    double distanceToScreen, uint32_t nOmega, uint32_t nRadius, uint32_t nPhi,
    double dt, uint32_t nSnaps, const uint32_t *itSnaps,
    const void *FormFactor, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* SYNCHRAD_GB300_H */
