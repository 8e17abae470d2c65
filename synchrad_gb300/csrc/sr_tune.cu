// Autotuner of the mixed-precision kernels' work shape, and CUDA-graph
// capture of a whole spectrum call (no counterpart in the reference, whose
// host loop launches one OpenCL kernel per track: synchrad/calc.py:257-267).
//
// The free parameters of the persistent far-field launch are the points per
// lane K, the lanes per direction L, the step records per TMA stage and the
// number of track subsets (the near field: K, L and the subsets).  sr_autotune
// times candidates with CUDA events on a bounded sample of the problem (the
// leading tracks), by coordinate search: (K, L) first, then the stage size,
// then the subsets, and caches the fastest per problem shape; sr_spectrum and
// sr_workspace_bytes then use the cached choice for that shape.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cmath>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "sr_common.cuh"
#include "sr_internal.h"

namespace sr {
namespace {

struct TuneKey {
  int device, mode, comp, dtype;
  uint32_t n_omega, n_theta, n_phi, n_tracks, n_snaps;
  int64_t total_steps;
  auto tie() const {
    return std::tie(device, mode, comp, dtype, n_omega, n_theta, n_phi, n_tracks, n_snaps,
                    total_steps);
  }
  bool operator<(const TuneKey &o) const { return tie() < o.tie(); }
};

std::mutex g_tmu;
std::map<TuneKey, FarMixedConfig> g_cache;

TuneKey key_of(const sr_tracks *t, const sr_grid *g, int comp) {
  TuneKey k{};
  if (cudaGetDevice(&k.device) != cudaSuccess) k.device = -1;  // no device: one key space
  k.mode = g->mode;
  k.comp = comp;
  k.dtype = t->dtype;
  k.n_omega = g->n_omega;
  k.n_theta = g->n_theta;
  k.n_phi = g->n_phi;
  k.n_tracks = t->n_tracks;
  k.n_snaps = t->n_snaps;
  k.total_steps = t->total_steps;
  return k;
}

FarMixedConfig default_config(const sr_tracks *t, const sr_grid *g) {
  if (g->mode == SR_MODE_FAR)
    return far_mixed_choose(g->n_omega, g->n_theta * g->n_phi, t->n_tracks, device_sm_count());
  return near_mixed_choose(g->n_omega, g->n_theta * g->n_phi, t->n_tracks, device_sm_count());
}

void to_public(const FarMixedConfig &c, double ms, sr_config *o) {
  if (!o) return;
  o->points_per_lane = c.K;
  o->lanes_per_direction = c.L;
  o->steps_per_stage = c.stage;
  o->track_subsets = c.n_sub;
  o->ctas = c.grid;
  o->reserved = 0;
  o->ms = ms;
}

size_t workspace_of(const sr_tracks *t, const sr_grid *g, int n_out, const FarMixedConfig &c) {
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  const uint32_t ns = t->n_snaps ? t->n_snaps : 1;
  return g->mode == SR_MODE_FAR ? far_mixed_workspace(t->total_steps, P, n_out, ns, c)
                                : near_mixed_workspace(t->total_steps, P, n_out, ns, c);
}

// Best of `reps` timed runs (after one untimed run), in ms; negative on error.
double time_config(const sr_tracks *t, const sr_grid *g, int comp, const FarMixedConfig &c,
                   void *const *out, void *ws, size_t ws_bytes, cudaStream_t s, int reps) {
  const FarMixedParams p = make_far_mixed_params(t, g, comp, out);
  auto run = [&]() {
    return g->mode == SR_MODE_FAR ? launch_far_mixed(p, c, ws, ws_bytes, s)
                                  : launch_near_mixed(p, c, ws, ws_bytes, s);
  };
  if (run() != SR_OK) return -1.0;
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -1.0;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return -1.0;
  }
  double best = 1e300;
  for (int r = 0; r < reps; ++r) {
    cudaEventRecord(e0, s);
    if (run() != SR_OK) {
      best = -1.0;
      break;
    }
    cudaEventRecord(e1, s);
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      best = -1.0;
      break;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best = std::min(best, (double)ms);
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return best;
}

}  // namespace

FarMixedConfig mixed_config(const sr_tracks *t, const sr_grid *g, int comp) {
  const TuneKey k = key_of(t, g, comp);
  {
    std::lock_guard<std::mutex> lk(g_tmu);
    auto it = g_cache.find(k);
    if (it != g_cache.end()) return it->second;
  }
  return default_config(t, g);
}

}  // namespace sr

using namespace sr;

extern "C" int sr_config_get(const sr_tracks *t, const sr_grid *g, int comp, int precision,
                             sr_config *out) {
  clear_error();
  if (!t || !g || !out) return fail(SR_ERR_INVALID, "NULL argument");
  if (precision != SR_PREC_MIXED)
    return fail(SR_ERR_UNSUPPORTED, "only the mixed-precision kernels have a work shape");
  to_public(mixed_config(t, g, comp), 0.0, out);
  return SR_OK;
}

extern "C" int sr_config_set(const sr_tracks *t, const sr_grid *g, int comp, int precision,
                             const sr_config *c) {
  clear_error();
  if (!t || !g || !c) return fail(SR_ERR_INVALID, "NULL argument");
  if (precision != SR_PREC_MIXED)
    return fail(SR_ERR_UNSUPPORTED, "only the mixed-precision kernels have a work shape");
  const bool far = g->mode == SR_MODE_FAR;
  const int K = c->points_per_lane, L = c->lanes_per_direction, st = c->steps_per_stage;
  if (far ? (K != 8 && K != 16 && K != 24 && K != 32) : (K != 8 && K != 16))
    return fail(SR_ERR_INVALID, "points per lane %d (far: 8, 16, 24, 32; near: 8, 16)", K);
  if (L != 8 && L != 16 && L != 32)
    return fail(SR_ERR_INVALID, "lanes per direction %d (8, 16 or 32)", L);
  if (far && (st < 32 || st > 512 || (st & 31) != 0))
    return fail(SR_ERR_INVALID, "steps per stage %d (multiples of 32 in [32, 512])", st);
  if (far && far_mixed_smem_bytes(32 / L, st) > 232448)
    return fail(SR_ERR_INVALID,
                "work shape (%d lanes per direction, %d steps per stage) needs %zu bytes of "
                "shared memory per CTA (at most 232448)",
                L, st, far_mixed_smem_bytes(32 / L, st));
  if (c->track_subsets < 0 || c->track_subsets > 64)
    return fail(SR_ERR_INVALID, "track subsets %d (0: default, at most 64)", c->track_subsets);
  const uint32_t n_dirs = g->n_theta * g->n_phi;
  const FarMixedConfig cfg =
      far ? far_mixed_make(g->n_omega, n_dirs, t->n_tracks, device_sm_count(), K, L, st,
                           c->track_subsets)
          : near_mixed_make(g->n_omega, n_dirs, t->n_tracks, device_sm_count(), K, L,
                            c->track_subsets);
  std::lock_guard<std::mutex> lk(g_tmu);
  g_cache[key_of(t, g, comp)] = cfg;
  return SR_OK;
}

extern "C" int sr_config_clear(void) {
  std::lock_guard<std::mutex> lk(g_tmu);
  g_cache.clear();
  return SR_OK;
}

extern "C" int sr_autotune(const sr_tracks *t, const sr_grid *g, int comp, int precision,
                           double budget_ms, void *stream, sr_config *best_out,
                           sr_config *default_out) {
  clear_error();
  void *probe[6] = {(void *)1, (void *)1, (void *)1, (void *)1, (void *)1, (void *)1};
  int rc = validate_spectrum_args(t, g, comp, precision, probe);
  if (rc) return rc;
  if (precision != SR_PREC_MIXED)
    return fail(SR_ERR_UNSUPPORTED, "only the mixed-precision kernels are tuned");
  const uint64_t P = (uint64_t)g->n_omega * g->n_theta * g->n_phi;
  const FarMixedConfig dflt = default_config(t, g);
  to_public(dflt, 0.0, default_out);
  to_public(dflt, 0.0, best_out);
  if (P == 0 || t->n_tracks == 0 || t->n_snaps == 0 || t->total_steps == 0) return SR_OK;
  if (budget_ms <= 0) budget_ms = 3000.0;
  const auto t_start = std::chrono::steady_clock::now();
  auto elapsed_ms = [&]() {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_start)
        .count();
  };
  cudaStream_t s = (cudaStream_t)stream;
  const int n_out = n_outputs(comp);
  const int n_sm = device_sm_count();
  const uint32_t n_dirs = g->n_theta * g->n_phi;
  const bool far = g->mode == SR_MODE_FAR;

  // Sample: the leading tracks, about budget / 100 ms of work at 2e12 pt-steps/s.
  // The offsets are read on the call's stream: work queued there before the
  // call (e.g. the host-to-device copy of a streamed chunk, which the stream
  // waits for) completes first.  A plain cudaMemcpy runs on the legacy
  // stream, which does not wait for non-blocking streams, and could read the
  // buffer before the copy landed.
  std::vector<int64_t> off(t->n_tracks + 1);
  cudaError_t e = cudaMemcpyAsync(off.data(), t->offsets, off.size() * sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, (cudaStream_t)stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize((cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(e, "offsets read");
  const double target = std::max(1e9, budget_ms / 100.0 * 2e9);
  uint32_t n_s = 1;
  while (n_s < t->n_tracks && (double)off[n_s] * (double)P < target) ++n_s;
  sr_tracks ts = *t;
  ts.n_tracks = n_s;
  ts.total_steps = off[n_s];
  const bool full = (n_s == t->n_tracks);

  // candidates
  std::vector<FarMixedConfig> kl;
  if (far) {
    for (int K : {32, 24, 16, 8})
      for (int L : {32, 16, 8}) {
        const uint64_t tile = (uint64_t)K * L;
        const uint64_t tiles = (g->n_omega + tile - 1) / tile;
        if ((double)(tiles * tile) > 1.34 * g->n_omega + 8.0 * L) continue;  // idle lanes
        kl.push_back(far_mixed_make(g->n_omega, n_dirs, n_s, n_sm, K, L, dflt.stage, 0));
      }
  } else {
    for (int K : {16, 8})
      for (int L : {32, 16, 8}) {
        const uint64_t tile = (uint64_t)K * L;
        const uint64_t tiles = (g->n_omega + tile - 1) / tile;
        if ((double)(tiles * tile) > 1.34 * g->n_omega + 8.0 * L) continue;
        kl.push_back(near_mixed_make(g->n_omega, n_dirs, n_s, n_sm, K, L, 0));
      }
  }
  const FarMixedConfig dflt_s =
      far ? far_mixed_make(g->n_omega, n_dirs, n_s, n_sm, dflt.K, dflt.L, dflt.stage, 0)
          : near_mixed_make(g->n_omega, n_dirs, n_s, n_sm, dflt.K, dflt.L, 0);
  kl.insert(kl.begin(), dflt_s);  // the default is always timed, first

  // scratch: outputs and the largest workspace any candidate can need
  size_t ws_need = 0;
  auto grow = [&](const FarMixedConfig &c) { ws_need = std::max(ws_need, workspace_of(&ts, g, n_out, c)); };
  for (const auto &c : kl) grow(c);
  {
    FarMixedConfig c64 = dflt_s;
    c64.n_sub = std::min<int>(64, (int)n_s);
    grow(c64);
    c64.stage = 256;
    grow(c64);
  }
  std::vector<void *> outs(6, nullptr);
  void *ws = nullptr;
  const size_t out_bytes = (size_t)(t->n_snaps) * P * 8;
  for (int i = 0; i < n_out && e == cudaSuccess; ++i) e = cudaMalloc(&outs[i], out_bytes);
  if (e == cudaSuccess) e = cudaMalloc(&ws, ws_need);
  auto release = [&]() {
    for (void *o : outs)
      if (o) cudaFree(o);
    if (ws) cudaFree(ws);
  };
  if (e != cudaSuccess) {
    release();
    return cuda_fail(e, "autotune scratch allocation");
  }
  for (int i = 0; i < n_out; ++i) cudaMemsetAsync(outs[i], 0, out_bytes, s);

  const int reps = 2;
  FarMixedConfig best = dflt_s;
  double best_ms = 1e300, dflt_ms = -1.0;
  auto consider = [&](const FarMixedConfig &c) -> int {
    const double ms = time_config(&ts, g, comp, c, outs.data(), ws, ws_need, s, reps);
    if (ms < 0) return SR_ERR_CUDA;
    if (ms < best_ms) {
      best_ms = ms;
      best = c;
    }
    return SR_OK;
  };
  // (K, L)
  for (size_t i = 0; i < kl.size(); ++i) {
    if (i > 0 && elapsed_ms() > budget_ms) break;
    rc = consider(kl[i]);
    if (rc) break;
    if (i == 0) dflt_ms = best_ms;
  }
  // steps per stage
  if (rc == SR_OK && far)
    for (int st : {64, 256}) {
      if (elapsed_ms() > budget_ms) break;
      FarMixedConfig c = far_mixed_make(g->n_omega, n_dirs, n_s, n_sm, best.K, best.L, st, 0);
      rc = consider(c);
      if (rc) break;
    }
  // track subsets
  int sub_scale_num = 1, sub_scale_den = 1;
  if (rc == SR_OK) {
    const int h = best.n_sub;
    for (int v : {h / 2, h * 2}) {
      if (v < 1 || v > 64 || v > (int)n_s || v == h || elapsed_ms() > budget_ms) continue;
      FarMixedConfig c =
          far ? far_mixed_make(g->n_omega, n_dirs, n_s, n_sm, best.K, best.L, best.stage, v)
              : near_mixed_make(g->n_omega, n_dirs, n_s, n_sm, best.K, best.L, v);
      const int before = best.n_sub;
      rc = consider(c);
      if (rc) break;
      if (best.n_sub != before) {
        sub_scale_num = best.n_sub;
        sub_scale_den = h;
      }
    }
  }
  cudaStreamSynchronize(s);
  release();
  if (rc) {
    char msg[256];
    snprintf(msg, sizeof(msg), "%s", sr_last_error());
    return fail(rc, "autotune run failed: %s", msg);
  }

  // the choice for the whole problem
  FarMixedConfig chosen;
  if (full) {
    chosen = best;
  } else {
    const FarMixedConfig h = far ? far_mixed_make(g->n_omega, n_dirs, t->n_tracks, n_sm, best.K,
                                                  best.L, best.stage, 0)
                                 : near_mixed_make(g->n_omega, n_dirs, t->n_tracks, n_sm, best.K,
                                                   best.L, 0);
    const int nsub = std::max(1, std::min(64, h.n_sub * sub_scale_num / sub_scale_den));
    chosen = far ? far_mixed_make(g->n_omega, n_dirs, t->n_tracks, n_sm, best.K, best.L,
                                  best.stage, nsub)
                 : near_mixed_make(g->n_omega, n_dirs, t->n_tracks, n_sm, best.K, best.L, nsub);
  }
  {
    std::lock_guard<std::mutex> lk(g_tmu);
    g_cache[key_of(t, g, comp)] = chosen;
  }
  to_public(chosen, best_ms, best_out);
  if (default_out) default_out->ms = dflt_ms;
  return SR_OK;
}

// ---------------------------------------------------------------------------
// CUDA graphs: one spectrum call (status reset, step records, the persistent
// kernel, the subset reduction) captured once and replayed.
// ---------------------------------------------------------------------------
struct sr_graph {
  cudaGraph_t graph;
  cudaGraphExec_t exec;
};

extern "C" int sr_graph_create(const sr_tracks *t, const sr_grid *g, int comp, int precision,
                               void *const *out, void *workspace, size_t workspace_bytes,
                               sr_graph **graph_out) {
  clear_error();
  if (!graph_out) return fail(SR_ERR_INVALID, "graph_out is NULL");
  *graph_out = nullptr;
  cudaStream_t cs;
  cudaError_t e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking);
  if (e != cudaSuccess) return cuda_fail(e, "capture stream");
  e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) {
    cudaStreamDestroy(cs);
    return cuda_fail(e, "begin capture");
  }
  const int rc = sr_spectrum(t, g, comp, precision, out, workspace, workspace_bytes, cs);
  cudaGraph_t graph = nullptr;
  e = cudaStreamEndCapture(cs, &graph);
  cudaStreamDestroy(cs);
  if (rc != SR_OK) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda_fail(e, "end capture");
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, graph, 0);
  if (e != cudaSuccess) {
    cudaGraphDestroy(graph);
    return cuda_fail(e, "graph instantiate");
  }
  sr_graph *h = new sr_graph{graph, exec};
  *graph_out = h;
  return SR_OK;
}

extern "C" int sr_graph_launch(sr_graph *h, void *stream) {
  clear_error();
  if (!h) return fail(SR_ERR_INVALID, "graph is NULL");
  return cuda_fail(cudaGraphLaunch(h->exec, (cudaStream_t)stream), "graph launch");
}

extern "C" int sr_graph_nodes(const sr_graph *h, int *n_kernels, int *n_nodes) {
  clear_error();
  if (!h) return fail(SR_ERR_INVALID, "graph is NULL");
  size_t n = 0;
  cudaError_t e = cudaGraphGetNodes(h->graph, nullptr, &n);
  if (e != cudaSuccess) return cuda_fail(e, "graph nodes");
  std::vector<cudaGraphNode_t> nodes(n);
  e = cudaGraphGetNodes(h->graph, nodes.data(), &n);
  if (e != cudaSuccess) return cuda_fail(e, "graph nodes");
  int k = 0;
  for (size_t i = 0; i < n; ++i) {
    cudaGraphNodeType ty;
    if (cudaGraphNodeGetType(nodes[i], &ty) == cudaSuccess && ty == cudaGraphNodeTypeKernel) ++k;
  }
  if (n_kernels) *n_kernels = k;
  if (n_nodes) *n_nodes = (int)n;
  return SR_OK;
}

extern "C" void sr_graph_destroy(sr_graph *h) {
  if (!h) return;
  cudaGraphExecDestroy(h->exec);
  cudaGraphDestroy(h->graph);
  delete h;
}
