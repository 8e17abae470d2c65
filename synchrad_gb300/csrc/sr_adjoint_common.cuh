// Pieces shared by the far- and near-field adjoint kernels.
#pragma once

#include "sr_common.cuh"
#include "sr_internal.h"
#include "sr_mixed_common.cuh"

namespace sr {
namespace {

struct AdjGlobals {
  float dw_h, dw_l;        // omega spacing (rad per unit time) as a double-float
  float w0f, dwf;          // first omega and spacing in FP32
  float wabs_min, wabs_max;
  int uniform;             // omega axis uniform to 1e-12
  int pad_;
};

// Omega table, axis uniformity and |omega| range (one block).
__global__ void adj_globals_kernel(FarMixedParams p, float4 *wtab, AdjGlobals *glob) {
  const uint32_t nO = p.n_omega;
  const double w0 = p.omega[0];
  const double dw = (nO > 1) ? (p.omega[nO - 1] - w0) / (double)(nO - 1) : 0.0;
  bool uni = true;
  float amin = 3.0e38f, amax = 0.f;
  for (uint32_t m = threadIdx.x; m < nO; m += blockDim.x) {
    const double wm = p.omega[m];
    if (fabs(wm - (w0 + (double)m * dw)) > 1e-12 * fabs(wm) + 1e-300) uni = false;
    const df r = df_from_double(wm * 0.15915494309189533577);
    const float aw = (float)fabs(wm);
    wtab[m] = make_float4(r.hi, r.lo, (float)wm, aw);
    amin = fminf(amin, aw);
    amax = fmaxf(amax, aw);
  }
  __shared__ float smin[256], smax[256];
  smin[threadIdx.x] = amin;
  smax[threadIdx.x] = amax;
  const int all_uni = __syncthreads_and(uni ? 1 : 0);
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int)threadIdx.x < o) {
      smin[threadIdx.x] = fminf(smin[threadIdx.x], smin[threadIdx.x + o]);
      smax[threadIdx.x] = fmaxf(smax[threadIdx.x], smax[threadIdx.x + o]);
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    AdjGlobals g;
    const df d = df_from_double(dw);
    g.dw_h = d.hi;
    g.dw_l = d.lo;
    g.w0f = (float)w0;
    g.dwf = (float)dw;
    g.wabs_min = smin[0];
    g.wabs_max = smax[0];
    g.uniform = all_uni;
    g.pad_ = 0;
    *glob = g;
  }
}

// Snapshot segments of a track.  The forward writes snapshot k after step
// f_k (the reference's state machine, SnapState); the snapshots that fire form
// a run k_first .. k_last with increasing f_k, a step s enters every fired
// snapshot with f_k >= s, and steps after the last fired one enter none.  So
// the body steps fall into segments, segment i holding the steps after
// f_{k_first + i - 1} up to f_{k_first + i}, each entering snapshots
// k_first + i .. k_last.  Work items never cross a segment; a segment of n
// steps makes ceil(n / per_item) items.
struct SnapSegment {
  uint32_t r0, r1;  // steps [r0, r1) of the item
  uint32_t k0, k1;  // snapshots k0 .. k1 (inclusive) receive them
};

__device__ __forceinline__ uint32_t last_fired(const FarMixedParams &p, uint32_t t) {
  SnapState st;
  const uint32_t *snaps = p.snap_its + (size_t)t * p.snap_stride;
  st.init(p.it_start[t], p.it_end[t], snaps, p.n_snaps);
  uint32_t last = 0xffffffffu;
  while (st.fire_it != SnapState::NEVER) {
    last = st.k;
    st.advance(p.it_start[t], p.it_end[t], snaps, p.n_snaps);
  }
  return last;
}

// Items of track t (count == nullptr) or the j-th of them (into *seg).
__device__ __forceinline__ uint32_t track_segments(const FarMixedParams &p, uint32_t t,
                                                   uint32_t per_item, uint32_t j,
                                                   SnapSegment *seg) {
  const uint32_t n_body = track_body(p, t);
  if (n_body == 0) return 0;
  const uint32_t k_last = last_fired(p, t);
  if (k_last == 0xffffffffu) return 0;  // no snapshot fires: nothing to differentiate
  SnapState st;
  const uint32_t *snaps = p.snap_its + (size_t)t * p.snap_stride;
  st.init(p.it_start[t], p.it_end[t], snaps, p.n_snaps);
  uint32_t lo = 0, items = 0;
  while (st.fire_it != SnapState::NEVER && lo < n_body) {
    const int64_t last_body = (int64_t)n_body - 1;
    const uint32_t hi = (uint32_t)(st.fire_it < last_body ? st.fire_it : last_body);  // inclusive
    if (hi >= lo) {
      const uint32_t n = (hi - lo + per_item) / per_item;
      if (seg != nullptr && j < items + n) {
        seg->r0 = lo + (j - items) * per_item;
        seg->r1 = min(hi + 1, seg->r0 + per_item);
        seg->k0 = st.k;
        seg->k1 = k_last;
        return items + n;
      }
      items += n;
      lo = hi + 1;
    }
    st.advance(p.it_start[t], p.it_end[t], snaps, p.n_snaps);
  }
  return items;
}

// Work items per track (snapshot segments cut into runs of steps_per_item),
// as an exclusive prefix (one block of 1024 threads, each scanning a
// contiguous run of tracks).
__global__ void adj_items_kernel(FarMixedParams p, int64_t *item_off, uint32_t steps_per_item) {
  const uint32_t n = p.n_tracks;
  const uint32_t per = (n + blockDim.x - 1) / blockDim.x;
  const uint32_t t0 = min(n, threadIdx.x * per), t1 = min(n, t0 + per);
  int64_t local = 0;
  for (uint32_t t = t0; t < t1; ++t) local += track_segments(p, t, steps_per_item, 0, nullptr);
  __shared__ int64_t sums[1024];
  sums[threadIdx.x] = local;
  __syncthreads();
  for (uint32_t off = 1; off < blockDim.x; off <<= 1) {
    const int64_t v = threadIdx.x >= off ? sums[threadIdx.x - off] : 0;
    __syncthreads();
    sums[threadIdx.x] += v;
    __syncthreads();
  }
  int64_t run = threadIdx.x ? sums[threadIdx.x - 1] : 0;
  for (uint32_t t = t0; t < t1; ++t) {
    item_off[t] = run;
    run += track_segments(p, t, steps_per_item, 0, nullptr);
  }
  if (threadIdx.x == blockDim.x - 1) item_off[n] = sums[blockDim.x - 1];
}

// Weight gradients are summed in two fixed-order stages: block (t, b) sums
// chunk b of track t's points into wpart[t][b] by a fixed tree, then one
// thread per track adds its chunks in order (sr_far_adjoint.cu,
// sr_near_adjoint.cu).
constexpr int kWeightThreads = 256;

inline uint32_t adj_weight_chunks(uint64_t P, uint32_t n_tracks, int n_sm) {
  uint64_t c = (4ull * (uint64_t)n_sm + n_tracks - 1) / (n_tracks ? n_tracks : 1);
  const uint64_t cmax = (P + kWeightThreads - 1) / kWeightThreads;
  if (c > cmax) c = cmax;
  if (c > 256) c = 256;
  return (uint32_t)(c < 1 ? 1 : c);
}

}  // namespace
}  // namespace sr
