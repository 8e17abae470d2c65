/* The C ABI of synchrad_gb300 used from plain C (no Python, no PyTorch):
 * device buffers from the CUDA runtime, one sr_spectrum call per precision.
 *
 * usage: sr_c_example <input.bin> <output.bin>
 * input (little-endian): uint32 n_steps, uint32 nO, uint32 nT, uint32 nP,
 *   double dt, double weight, then x, y, z, ux, uy, uz [n_steps] doubles,
 *   omega2pi [nO], sin_theta, cos_theta [nT], sin_phi, cos_phi [nP] doubles.
 * output: the 'total' spectrum [nP][nT][nO] doubles, mixed precision, then
 *   the same with the plain FP64 kernel.  Exit status 0 on success. */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>

#include <cuda_runtime_api.h>

#include "synchrad_gb300.h"

static void *to_dev(const void *h, size_t bytes) {
  void *d = NULL;
  if (cudaMalloc(&d, bytes) != cudaSuccess) return NULL;
  if (h && cudaMemcpy(d, h, bytes, cudaMemcpyHostToDevice) != cudaSuccess) return NULL;
  return d;
}

static int fail(const char *what) {
  fprintf(stderr, "%s: %s\n", what, sr_last_error());
  return 1;
}

int main(int argc, char **argv) {
  if (argc != 3) return 2;
  FILE *f = fopen(argv[1], "rb");
  if (!f) return 2;
  uint32_t hdr[4];
  double dt, w;
  if (fread(hdr, 4, 4, f) != 4 || fread(&dt, 8, 1, f) != 1 || fread(&w, 8, 1, f) != 1) return 2;
  const uint32_t n = hdr[0], nO = hdr[1], nT = hdr[2], nP = hdr[3];
  const size_t P = (size_t)nO * nT * nP;
  double *host = (double *)malloc(sizeof(double) * (6 * (size_t)n + nO + 2 * nT + 2 * nP));
  const size_t nvals = 6 * (size_t)n + nO + 2 * nT + 2 * nP;
  if (!host || fread(host, 8, nvals, f) != nvals) return 2;
  fclose(f);

  /* one track: CSR offsets {0, n}, it_start 0, it_end n, one snapshot at n */
  const int64_t offsets[2] = {0, (int64_t)n};
  const uint32_t it_start = 0, it_end = n, snap = n;
  sr_tracks t = {0};
  t.n_tracks = 1;
  t.dtype = SR_DTYPE_F64;
  t.total_steps = n;
  t.offsets = (const int64_t *)to_dev(offsets, sizeof offsets);
  const void **coords[6] = {&t.x, &t.y, &t.z, &t.ux, &t.uy, &t.uz};
  for (int k = 0; k < 6; ++k) *coords[k] = to_dev(host + (size_t)k * n, 8 * (size_t)n);
  t.weight = (const double *)to_dev(&w, 8);
  t.it_start = (const uint32_t *)to_dev(&it_start, 4);
  t.it_end = (const uint32_t *)to_dev(&it_end, 4);
  t.snap_its = (const uint32_t *)to_dev(&snap, 4);
  t.snap_stride = 1;
  t.n_snaps = 1;
  t.dt = dt;

  const double *ax = host + 6 * (size_t)n;
  sr_grid g = {0};
  g.mode = SR_MODE_FAR;
  g.dtype = SR_DTYPE_F64;
  g.n_omega = nO;
  g.n_theta = nT;
  g.n_phi = nP;
  g.omega = to_dev(ax, 8 * (size_t)nO);
  g.axis1 = to_dev(ax + nO, 8 * (size_t)nT);
  g.axis2 = to_dev(ax + nO + nT, 8 * (size_t)nT);
  g.sin_phi = to_dev(ax + nO + 2 * nT, 8 * (size_t)nP);
  g.cos_phi = to_dev(ax + nO + 2 * nT + nP, 8 * (size_t)nP);

  double *result = (double *)malloc(16 * P);
  const int precisions[2] = {SR_PREC_MIXED, SR_PREC_DOUBLE};
  for (int i = 0; i < 2; ++i) {
    void *out = to_dev(NULL, 8 * P);
    if (!out || cudaMemset(out, 0, 8 * P) != cudaSuccess) return fail("output");
    void *outs[6] = {out, NULL, NULL, NULL, NULL, NULL};
    const int64_t need = sr_workspace_bytes(&t, &g, SR_COMP_TOTAL, precisions[i]);
    if (need < 0) return fail("sr_workspace_bytes");
    void *ws = need > 0 ? to_dev(NULL, (size_t)need) : NULL;
    if (sr_spectrum(&t, &g, SR_COMP_TOTAL, precisions[i], outs, ws, (size_t)need, NULL) != SR_OK)
      return fail("sr_spectrum");
    if (ws && sr_workspace_status(ws, NULL) != SR_OK) return fail("sr_workspace_status");
    if (cudaMemcpy(result + i * P, out, 8 * P, cudaMemcpyDeviceToHost) != cudaSuccess)
      return fail("copy back");
    cudaFree(out);
    if (ws) cudaFree(ws);
  }
  FILE *o = fopen(argv[2], "wb");
  if (!o || fwrite(result, 8, 2 * P, o) != 2 * P) return 2;
  fclose(o);
  printf("sr_c_example: %zu points, version %d\n", P, sr_version());
  return 0;
}
