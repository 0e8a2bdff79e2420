/* A second C caller of the public headers only: the 1D/2D multi-splines
 * (CPU entries and the 1D batched GPU entry), the third-derivative entry,
 * double-float evaluation of an FP64 table, and the fused determinant step.
 * Each part checks the library against itself through a second route
 * (GPU entry vs CPU entry, vghgh vs vgh, determinant ratio vs a dot product
 * of CPU-entry values).  Exit status 0 on success; the failing part's
 * number otherwise. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <cuda_runtime_api.h>

#include "multi_bspline.h"
#include "multi_bspline_create_cuda.h"
#include "multi_bspline_eval_cuda.h"
#include "einspline_gb300.h"

static unsigned long long state = 0x9E3779B97F4A7C15ull;
static double uniform01(void) { /* xorshift64* */
  state ^= state >> 12; state ^= state << 25; state ^= state >> 27;
  return (double)((state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
}

static double rel(double a, double b, double scale) { return fabs(a - b) / (scale > 0 ? scale : 1.0); }

/* 1: 1D d spline, CPU vgl against the batched GPU vgl (cell-unit derivatives) */
static int part_1d(void) {
  const int M = 24, N = 20, P = 64;
  Ugrid g = {0.0, 1.0, M, 0.0, 0.0};
  BCtype_d bc = {PERIODIC, PERIODIC, 0.0, 0.0};
  multi_UBspline_1d_d *sp = create_multi_UBspline_1d_d(g, bc, N);
  if (!sp) return 1;
  double data[24];
  for (int n = 0; n < N; n++) {
    for (int i = 0; i < M; i++) data[i] = 2.0 * uniform01() - 1.0;
    set_multi_UBspline_1d_d(sp, n, data);
  }
  multi_UBspline_1d_d_cuda *cs = create_multi_UBspline_1d_d_cuda(sp);
  if (!cs || cs->dim != M || cs->num_splines != N) return 1;
  double *blk_d, *pos_d, **v_d, **g_d, **l_d, *v[64], *gr[64], *lp[64], pos[64];
  cudaMalloc((void **)&blk_d, sizeof(double) * 3 * N * P);
  cudaMalloc((void **)&pos_d, sizeof(double) * P);
  cudaMalloc((void **)&v_d, sizeof(double *) * P);
  cudaMalloc((void **)&g_d, sizeof(double *) * P);
  cudaMalloc((void **)&l_d, sizeof(double *) * P);
  for (int p = 0; p < P; p++) {
    v[p] = blk_d + p * N; gr[p] = blk_d + (P + p) * N; lp[p] = blk_d + (2 * P + p) * N;
    pos[p] = uniform01();
  }
  cudaMemcpy(v_d, v, sizeof(v), cudaMemcpyHostToDevice);
  cudaMemcpy(g_d, gr, sizeof(gr), cudaMemcpyHostToDevice);
  cudaMemcpy(l_d, lp, sizeof(lp), cudaMemcpyHostToDevice);
  cudaMemcpy(pos_d, pos, sizeof(pos), cudaMemcpyHostToDevice);
  eval_multi_multi_UBspline_1d_d_vgl_cuda(cs, pos_d, v_d, g_d, l_d, P);
  if (einspline_gb300_last_error()) return 1;
  double *out = (double *)malloc(sizeof(double) * 3 * N * P);
  cudaMemcpy(out, blk_d, sizeof(double) * 3 * N * P, cudaMemcpyDeviceToHost);
  double cv[20], cg[20], cl[20], err = 0.0;
  const double delta = 1.0 / M;
  for (int p = 0; p < P; p++) {
    eval_multi_UBspline_1d_d_vgl(sp, pos[p], cv, cg, cl);
    for (int n = 0; n < N; n++) {
      err = fmax(err, rel(cv[n], out[p * N + n], 1.0));
      err = fmax(err, rel(cg[n] * delta, out[(P + p) * N + n], 1.0));
      err = fmax(err, rel(cl[n] * delta * delta, out[(2 * P + p) * N + n], 1.0));
    }
  }
  printf("1d: max diff %.3g\n", err);
  free(out);
  cudaFree(blk_d); cudaFree(pos_d); cudaFree(v_d); cudaFree(g_d); cudaFree(l_d);
  destroy_multi_UBspline_1d_d_cuda(cs);
  destroy_Bspline(sp);
  return err < 1e-12 ? 0 : 1;
}

/* 2: 2D z spline: vgh Hessian symmetric, vgl laplacian its trace, vg = vgh's */
static int part_2d(void) {
  const int Mx = 12, My = 10, N = 6;
  Ugrid gx = {0.0, 2.0, Mx, 0.0, 0.0}, gy = {-1.0, 1.0, My, 0.0, 0.0};
  BCtype_z bx = {PERIODIC, PERIODIC, 0.0, 0.0, 0.0, 0.0};
  BCtype_z by = {DERIV1, NATURAL, 0.5, -0.25, 0.0, 0.0};
  multi_UBspline_2d_z *sp = create_multi_UBspline_2d_z(gx, gy, bx, by, N);
  if (!sp) return 2;
  complex_double data[12 * 10];
  for (int n = 0; n < N; n++) {
    for (int i = 0; i < Mx * My; i++) data[i] = (2.0 * uniform01() - 1.0) + (2.0 * uniform01() - 1.0) * I;
    set_multi_UBspline_2d_z(sp, n, data);
  }
  complex_double v1[6], g1[12], l1[6], v2[6], g2[12], h2[24];
  double err = 0.0;
  for (int k = 0; k < 10; k++) {
    const double x = 2.0 * uniform01(), y = 2.0 * uniform01() - 1.0;
    eval_multi_UBspline_2d_z_vgl(sp, x, y, v1, g1, l1);
    eval_multi_UBspline_2d_z_vgh(sp, x, y, v2, g2, h2);
    if (einspline_gb300_last_error()) return 2;
    for (int n = 0; n < N; n++) {
      double s = cabs(h2[4 * n]) + cabs(h2[4 * n + 3]) + 1.0;
      err = fmax(err, cabs(v1[n] - v2[n]));
      err = fmax(err, cabs(g1[2 * n] - g2[2 * n]) + cabs(g1[2 * n + 1] - g2[2 * n + 1]));
      err = fmax(err, cabs(h2[4 * n + 1] - h2[4 * n + 2]));
      err = fmax(err, cabs(l1[n] - (h2[4 * n] + h2[4 * n + 3])) / s);
    }
  }
  printf("2d: max diff %.3g\n", err);
  destroy_Bspline(sp);
  return err < 1e-12 ? 0 : 2;
}

/* 3: 3D d spline: vghgh's first three outputs equal vgh's; double-float
 * evaluation of the same table within 1e-12 of IEEE FP64 */
static int part_3d(void) {
  const int M = 10, N = 8;
  Ugrid g = {0.0, 1.0, M, 0.0, 0.0};
  BCtype_d bc = {PERIODIC, PERIODIC, 0.0, 0.0};
  multi_UBspline_3d_d *sp = create_multi_UBspline_3d_d(g, g, g, bc, bc, bc, N);
  if (!sp) return 3;
  double *data = (double *)malloc(sizeof(double) * M * M * M);
  for (int n = 0; n < N; n++) {
    for (int i = 0; i < M * M * M; i++) data[i] = 2.0 * uniform01() - 1.0;
    set_multi_UBspline_3d_d(sp, n, data);
  }
  free(data);
  double v[8], gr[24], h[72], v3[8], g3[24], h3[72], gh[216], vd[8], gd[24], hd[72];
  double err = 0.0, errdf = 0.0;
  for (int k = 0; k < 8; k++) {
    const double x = uniform01(), y = uniform01(), z = uniform01();
    eval_multi_UBspline_3d_d_vgh(sp, x, y, z, v, gr, h);
    eval_multi_UBspline_3d_d_vghgh(sp, x, y, z, v3, g3, h3, gh);
    if (memcmp(v, v3, sizeof(v)) || memcmp(gr, g3, sizeof(gr)) || memcmp(h, h3, sizeof(h))) return 3;
    for (int n = 0; n < N; n++) err = fmax(err, fabs(gh[27 * n + 5] - gh[27 * n + 7]));  /* xyz = xzy */
    if (einspline_gb300_set_fp64_mode(sp->gb300, 1)) return 3;
    eval_multi_UBspline_3d_d_vgh(sp, x, y, z, vd, gd, hd);
    if (einspline_gb300_set_fp64_mode(sp->gb300, 0)) return 3;
    double sv = 0, sh = 0;
    for (int n = 0; n < N; n++) sv = fmax(sv, fabs(v[n]));
    for (int i = 0; i < 9 * N; i++) sh = fmax(sh, fabs(h[i]));
    for (int n = 0; n < N; n++) errdf = fmax(errdf, rel(vd[n], v[n], sv));
    for (int i = 0; i < 9 * N; i++) errdf = fmax(errdf, rel(hd[i], h[i], sh));
  }
  printf("3d: vghgh symmetry %.3g, double-float vs FP64 %.3g\n", err, errdf);
  destroy_Bspline(sp);
  return (err == 0.0 && errdf < 1e-12) ? 0 : 3;
}

/* 4: the fused determinant ratio against a dot product of CPU-entry values */
static int part_det(void) {
  const int M = 12, N = 8, W = 5, K = 3;
  Ugrid g = {0.0, 1.0, M, 0.0, 0.0};
  BCtype_s bc = {PERIODIC, PERIODIC, 0.0f, 0.0f};
  multi_UBspline_3d_s *sp = create_multi_UBspline_3d_s(g, g, g, bc, bc, bc, N);
  if (!sp) return 4;
  float *data = (float *)malloc(sizeof(float) * M * M * M);
  for (int n = 0; n < N; n++) {
    for (int i = 0; i < M * M * M; i++) data[i] = (float)(2.0 * uniform01() - 1.0);
    set_multi_UBspline_3d_s(sp, n, data);
  }
  free(data);
  /* any inverse-like matrix will do for the contraction: Ainv[j][e] random */
  float ainv[5][8][8], pos[3 * 5], ratio[5];
  for (int w = 0; w < W; w++)
    for (int j = 0; j < N; j++)
      for (int e = 0; e < N; e++) ainv[w][j][e] = (float)(2.0 * uniform01() - 1.0);
  for (int i = 0; i < 3 * W; i++) pos[i] = (float)uniform01();
  float *ainv_d, *pos_d, *ratio_d, **list_d, *list[5];
  cudaMalloc((void **)&ainv_d, sizeof(ainv));
  cudaMalloc((void **)&pos_d, sizeof(pos));
  cudaMalloc((void **)&ratio_d, sizeof(ratio));
  cudaMalloc((void **)&list_d, sizeof(list));
  for (int w = 0; w < W; w++) list[w] = ainv_d + w * N * N;
  cudaMemcpy(ainv_d, ainv, sizeof(ainv), cudaMemcpyHostToDevice);
  cudaMemcpy(pos_d, pos, sizeof(pos), cudaMemcpyHostToDevice);
  cudaMemcpy(list_d, list, sizeof(list), cudaMemcpyHostToDevice);
  einspline_gb300_det_opts o = {N, K, N, 0, 0, 1};
  if (einspline_gb300_det_ratio(sp->gb300, &o, W, pos_d, (const float *const *)list_d, ratio_d, NULL, NULL, NULL,
                                NULL))
    return 4;
  cudaMemcpy(ratio, ratio_d, sizeof(ratio), cudaMemcpyDeviceToHost);
  double err = 0.0;
  float v[8];
  for (int w = 0; w < W; w++) {
    eval_multi_UBspline_3d_s(sp, pos[3 * w], pos[3 * w + 1], pos[3 * w + 2], v);
    double r = 0.0, s = 0.0;
    for (int j = 0; j < N; j++) {
      r += (double)v[j] * ainv[w][j][K];
      s += fabs((double)v[j] * ainv[w][j][K]);
    }
    err = fmax(err, rel(ratio[w], r, s));
  }
  printf("det: max rel diff %.3g\n", err);
  cudaFree(ainv_d); cudaFree(pos_d); cudaFree(ratio_d); cudaFree(list_d);
  destroy_Bspline(sp);
  return err < 2e-5 ? 0 : 4;
}

int main(void) {
  einspline_gb300_set_abort_on_error(0);
  int r;
  if ((r = part_1d())) return r;
  if ((r = part_2d())) return r;
  if ((r = part_3d())) return r;
  if ((r = part_det())) return r;
  return 0;
}
