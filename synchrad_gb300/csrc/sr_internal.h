// Internal launch descriptors shared by the translation units of the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/synchrad_gb300.h"

namespace sr {

// Arguments of the plain-port kernels (one thread per spectral point, every
// track of the batch in sequence).  `offsets == nullptr` selects the
// single-track form of the reference kernels, with the scalars `*1` below.
struct PortParams {
  uint32_t n_tracks;
  const int64_t *offsets;
  const void *x, *y, *z, *ux, *uy, *uz;
  const double *weight;
  const uint32_t *it_start, *it_end, *snap_its;
  uint32_t snap_stride, n_snaps;
  double wp1;
  uint32_t it_start1, it_end1, n_steps1;
  double dt;
  uint32_t n_omega, n_1, n_phi;
  const void *omega, *axis1, *axis2, *sin_phi, *cos_phi, *form_factor;
  double L;
  void *out[6];
};

// Optional CUDA-event timing of the dominant kernel of a call (sr_diag.cu).
void timing_record(cudaStream_t s, bool start, void **token);

// mode: 0 far, 1 near; dtype: 0 f64, 1 f32.
int launch_port(const PortParams &p, int mode, int comp, int dtype, bool native,
                cudaStream_t stream);

// Arguments of the mixed-precision far-field path.
struct FarMixedParams {
  // tracks
  uint32_t n_tracks;
  int track_f32;
  int64_t total_steps;
  const int64_t *offsets;
  const void *x, *y, *z, *ux, *uy, *uz;
  const double *weight;
  const uint32_t *it_start, *it_end, *snap_its;
  uint32_t snap_stride, n_snaps;
  double dt;
  // grid (FP64 axes)
  uint32_t n_omega, n_theta, n_phi;
  const double *omega, *sin_theta, *cos_theta, *sin_phi, *cos_phi,
      *form_factor;
  double L_screen;     // near field: distance to the screen
  int comp;
  int n_out;
  // decomposition
  uint32_t n_wtiles;   // omega tiles of 32*K points per direction
  uint32_t n_groups;   // CTA-sized groups of warp tasks
  uint32_t n_sub;      // track subsets
  uint32_t n_items;    // n_groups * n_sub
  uint32_t dpw;        // directions per warp
  uint32_t stage_steps;  // far field: step records per TMA stage
  uint32_t fold_stages;  // far field: stages between folds of the FP32 sums
  // workspace
  float4 *records;     // [total_steps][4]
  double *partial;     // [n_sub][n_out][n_snaps][P]
  float *outer;        // [grid][W][K][8][32] compensated per-track sums
  float *save_A;       // optional per-track amplitudes for the adjoints, as each
                       // snapshot writes them: far [n_tracks][n_snaps][P][4]
                       // (A_theta, A_phi), near [n_tracks][n_snaps][P][8] (A_x, A_y,
                       // A_z complex, two floats of padding)
  int *status;
  unsigned int *queue;   // work items handed out after each CTA's first (zeroed per launch)
  // outputs
  double *out[6];
};

struct FarMixedConfig {
  int K;        // points per lane
  int W;        // warps per CTA
  int L;        // lanes per direction
  int dpw;      // directions per warp (32 / L)
  int n_sub;    // track subsets
  int ctas_per_sm;
  int grid;     // CTAs of the persistent launch
  int stage;    // step records per TMA stage (far field; multiple of 32, <= 512)
};

FarMixedConfig far_mixed_make(uint32_t n_omega, uint32_t n_dirs, uint32_t n_tracks, int n_sm,
                              int K, int L, int stage, int n_sub);
FarMixedConfig near_mixed_make(uint32_t n_omega, uint32_t n_screen, uint32_t n_tracks, int n_sm,
                               int K, int L, int n_sub);
// The configuration sr_spectrum uses for a mixed-precision problem: the
// autotuner's choice when one is cached for this problem, else the default.
FarMixedConfig mixed_config(const sr_tracks *t, const sr_grid *g, int comp);
FarMixedConfig far_mixed_choose(uint32_t n_omega, uint32_t n_dirs,
                                uint32_t n_tracks, int n_sm);
size_t far_mixed_smem_bytes(int dpw, int stage);
size_t far_mixed_workspace(int64_t total_steps, uint64_t n_points, int n_out,
                           uint32_t n_snaps, const FarMixedConfig &cfg);
int launch_far_mixed(FarMixedParams p, const FarMixedConfig &cfg,
                     void *workspace, size_t ws_bytes, cudaStream_t stream);
void launch_far_prepass(const FarMixedParams &p, int blocks, cudaStream_t stream);
void launch_near_prepass(const FarMixedParams &p, int blocks, cudaStream_t stream);

// The mixed-precision near field (same parameter block; n_theta holds n_R,
// sin_theta the radius axis, L_screen the screen distance).
FarMixedConfig near_mixed_choose(uint32_t n_omega, uint32_t n_screen, uint32_t n_tracks,
                                 int n_sm);
size_t near_mixed_workspace(int64_t total_steps, uint64_t n_points, int n_out,
                            uint32_t n_snaps, const FarMixedConfig &cfg);
int launch_near_mixed(FarMixedParams p, const FarMixedConfig &cfg, void *workspace,
                      size_t ws_bytes, cudaStream_t stream);

// The double-float far field (sr_far_df.cu, SR_PREC_DF): its work shape,
// workspace size and launch (same parameter block as the mixed far field).
FarMixedConfig far_df_choose(uint32_t n_omega, uint32_t n_dirs, uint32_t n_tracks, int n_sm);
size_t far_df_workspace(int64_t total_steps, uint64_t n_points, int n_out, uint32_t n_snaps,
                        const FarMixedConfig &cfg);
int launch_far_df(FarMixedParams p, const FarMixedConfig &cfg, void *workspace,
                  size_t ws_bytes, cudaStream_t stream);

// sr_api.cu: argument checks and parameter packing shared by entry points.
int validate_spectrum_args(const sr_tracks *t, const sr_grid *g, int comp,
                           int precision, void *const *out);
FarMixedParams make_far_mixed_params(const sr_tracks *t, const sr_grid *g,
                                     int comp, void *const *out);
int device_sm_count();

// sr_noalloc.cu: the status word of the allocation-free entry point's static
// scratch array on the current device.
int noalloc_status_word(int **word);

}  // namespace sr
