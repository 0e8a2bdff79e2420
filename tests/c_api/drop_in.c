/* A C caller written against the einspline API only (the pattern of the
 * reference's src/test_multi_cuda.cu), compiled with gcc against include/ and
 * linked with libeinspline_gb300.so.  It builds a periodic multi-spline with
 * create/set, evaluates it through the CPU entry and through the batched CUDA
 * entry with device pointer arrays, and checks that the two agree.
 * Exit status 0 on success. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <cuda_runtime_api.h>

#include "multi_bspline.h"
#include "multi_bspline_create_cuda.h"
#include "multi_bspline_eval_cuda.h"
#include "einspline_gb300.h"

static unsigned long long state = 88172645463325252ull;
static double uniform01(void) { /* xorshift64* */
  state ^= state >> 12; state ^= state << 25; state ^= state >> 27;
  return (double)((state * 2685821657736338717ull) >> 11) * (1.0 / 9007199254740992.0);
}

int main(void) {
  const int M = 16, N = 40, W = 300;
  Ugrid g = {0.0, 1.0, M, 0.0, 0.0};
  BCtype_s bc = {PERIODIC, PERIODIC, 0.0f, 0.0f};
  multi_UBspline_3d_s *sp = create_multi_UBspline_3d_s(g, g, g, bc, bc, bc, N);
  if (!sp) return 2;
  float *data = (float *)malloc(sizeof(float) * M * M * M);
  for (int n = 0; n < N; n++) {
    for (int i = 0; i < M * M * M; i++) data[i] = (float)(2.0 * uniform01() - 1.0);
    set_multi_UBspline_3d_s(sp, n, data);
  }
  free(data);
  multi_UBspline_3d_s_cuda *cs = create_multi_UBspline_3d_s_cuda(sp);
  if (!cs || cs->num_splines != N || cs->dim.x != (unsigned)M) return 3;

  /* device buffers as the reference test lays them out */
  float *block_d, *pos_d, **vals_d, **grads_d, **hess_d;
  float *vals[W], *grads[W], *hess[W];
  cudaMalloc((void **)&block_d, sizeof(float) * 10 * N * W);
  cudaMalloc((void **)&pos_d, sizeof(float) * 3 * W);
  cudaMalloc((void **)&vals_d, sizeof(float *) * W);
  cudaMalloc((void **)&grads_d, sizeof(float *) * W);
  cudaMalloc((void **)&hess_d, sizeof(float *) * W);
  for (int w = 0; w < W; w++) {
    vals[w] = block_d + w * N;
    grads[w] = block_d + N * W + 3 * w * N;
    hess[w] = block_d + 4 * N * W + 6 * w * N;
  }
  cudaMemcpy(vals_d, vals, sizeof(float *) * W, cudaMemcpyHostToDevice);
  cudaMemcpy(grads_d, grads, sizeof(float *) * W, cudaMemcpyHostToDevice);
  cudaMemcpy(hess_d, hess, sizeof(float *) * W, cudaMemcpyHostToDevice);
  float pos[3 * W];
  for (int i = 0; i < 3 * W; i++) pos[i] = (float)uniform01();
  cudaMemcpy(pos_d, pos, sizeof(pos), cudaMemcpyHostToDevice);

  eval_multi_multi_UBspline_3d_s_vgh_cuda(cs, pos_d, vals_d, grads_d, hess_d, W);
  if (einspline_gb300_last_error()) return 4;
  float *out = (float *)malloc(sizeof(float) * 10 * N * W);
  cudaMemcpy(out, block_d, sizeof(float) * 10 * N * W, cudaMemcpyDeviceToHost);

  /* the CPU entry at the same points (the start is 0, so both rules agree) */
  float v[N], gr[3 * N], h[9 * N];
  double maxv = 0, maxdv = 0, maxg = 0, maxdg = 0, maxh = 0, maxdh = 0;
  const int h6[6] = {0, 1, 2, 4, 5, 8};
  for (int w = 0; w < W; w++) {
    eval_multi_UBspline_3d_s_vgh(sp, pos[3 * w], pos[3 * w + 1], pos[3 * w + 2], v, gr, h);
    for (int n = 0; n < N; n++) {
      maxv = fmax(maxv, fabs(v[n]));
      maxdv = fmax(maxdv, fabs(v[n] - out[w * N + n]));
      for (int c = 0; c < 3; c++) {
        maxg = fmax(maxg, fabs(gr[3 * n + c]));
        maxdg = fmax(maxdg, fabs(gr[3 * n + c] - out[N * W + 3 * (w * N + n) + c]));
      }
      for (int q = 0; q < 6; q++) {
        maxh = fmax(maxh, fabs(h[9 * n + h6[q]]));
        maxdh = fmax(maxdh, fabs(h[9 * n + h6[q]] - out[4 * N * W + 6 * (w * N + n) + q]));
      }
    }
  }
  printf("max rel diff: value %.3g gradient %.3g hessian %.3g\n", maxdv / maxv, maxdg / maxg, maxdh / maxh);
  const int ok = maxdv / maxv < 2e-5 && maxdg / maxg < 2e-5 && maxdh / maxh < 2e-5;
  free(out);
  cudaFree(block_d); cudaFree(pos_d); cudaFree(vals_d); cudaFree(grads_d); cudaFree(hess_d);
  destroy_multi_UBspline_3d_s_cuda(cs);
  destroy_Bspline(sp);
  return ok ? 0 : 1;
}
