// Fused QMC determinant step: orbital evaluation + Slater-determinant ratio,
// and the Sherman-Morrison update of the inverse after an accepted move.
//
// The reference's QMC prototype (src/cuda_walker.cu) moves electron k of
// every walker, evaluates the N orbitals at the new positions into a row
// buffer (calc_new_row, :69-88, eval_multi_multi_UBspline_3d_s_cuda), dots
// that row with column k of each walker's inverse Slater matrix (calc_ratios,
// :171-201) and, for accepted walkers, updates the inverse in two kernels
// (update_inverse_cuda1/2, src/determinant_update.h:9-111, launched at
// src/cuda_walker.cu:92-136).
//
// k_det_ratio fuses the first two: one block per walker gathers the stencil
// of all N orbitals with the evaluation kernels' separable reduction and
// contracts value, gradient and Laplacian with the inverse column in
// registers, so the per-orbital outputs never reach HBM (only the value row,
// on request, for the update).  Block sums use a fixed shuffle tree: results
// are deterministic.
//
// The update is two passes over each accepted walker's inverse:
//   pass 1: x = delta^T Ainv (delta = u - A[k,:]) and colk = Ainv[:,k];
//   pass 2: Ainv += (-1 / (1 + x[k])) colk x^T, A[k,:] = u.
// Unlike the reference's kernel 1, where every block of a walker writes the
// new row into A while other blocks still read the old one, A is only read in
// pass 1 and written in pass 2.
#include <string.h>

#include "eval_core.h"

namespace eg {

struct DetArgs {
  EvalArgs e;                  // geometry, storage scale, positions, rule
  const float *const *ainv;    // per walker
  float *const *amat;          // update: per walker A (row k replaced)
  const float *const *urow;    // update: per walker new row u
  float *const *row_out;       // ratio: optional value row per walker
  float *ratio, *grad, *lapl;  // ratio outputs (grad, lapl optional)
  float *work;                 // update scratch: [walker][2][n] (x, colk)
  int n, k, ld, trans;
};

constexpr int kDetThreads = 128;

// Inverse entry (orbital j, electron c).
__device__ __forceinline__ float ainv_at(const float *m, int j, int c, int ld, int trans) {
  return trans ? m[(int64_t)c * ld + j] : m[(int64_t)j * ld + c];
}

template <int ST, bool GL>
__global__ void __launch_bounds__(kDetThreads, 3) k_det_ratio(const DetArgs d) {
  constexpr int VW = CT<ST>::VW;
  static_assert(sizeof(typename CT<ST>::A) == 4, "determinant step: real float tables only");
  __shared__ float sw[36];
  __shared__ int sidx[3];
  __shared__ float red[kDetThreads / 32][5];
  const EvalArgs &a = d.e;
  const int w = blockIdx.x;
  if (threadIdx.x < 3) {
    const int ax = threadIdx.x;
    const double xd = a.pos_f64 ? reinterpret_cast<const double *>(a.pos)[3 * (int64_t)w + ax]
                                : (double)reinterpret_cast<const float *>(a.pos)[3 * (int64_t)w + ax];
    int idx;
    float t;
    cell(a, ax, xd, idx, t);
    bspline_weights<float>(t, sw + 12 * ax, a.dinvf[ax]);
    sidx[ax] = idx;
  }
  __syncthreads();
  const float *ainv = d.ainv[w];
  float *row = d.row_out ? d.row_out[w] : nullptr;
  const int64_t xsb = a.xs * CT<ST>::BYTES, ysb = a.ys * CT<ST>::BYTES, zsb = a.zs * CT<ST>::BYTES;
  const char *base = reinterpret_cast<const char *>(a.coefs) + sidx[0] * xsb + sidx[1] * ysb + sidx[2] * zsb;
  float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
  for (int col0 = threadIdx.x * VW; col0 < d.n; col0 += kDetThreads * VW) {
    float o[10][VW];
    contract<ST, GL>(base + (int64_t)col0 * CT<ST>::BYTES, xsb, ysb, zsb, sw, o);
    if (a.scale) {
#pragma unroll
      for (int e = 0; e < VW; e++) {
        const float sc = a.scale[col0 + e];
#pragma unroll
        for (int q = 0; q < (GL ? 10 : 1); q++) o[q][e] *= sc;
      }
    }
#pragma unroll
    for (int e = 0; e < VW; e++) {
      const int j = col0 + e;
      if (j >= d.n) break;
      const float c = ainv_at(ainv, j, d.k, d.ld, d.trans);
      acc[0] = fmaf(o[0][e], c, acc[0]);
      if (GL) {
        acc[1] = fmaf(o[1][e], c, acc[1]);
        acc[2] = fmaf(o[2][e], c, acc[2]);
        acc[3] = fmaf(o[3][e], c, acc[3]);
        acc[4] = fmaf((o[4][e] + o[7][e]) + o[9][e], c, acc[4]);
      }
      if (row) row[j] = o[0][e];
    }
  }
#pragma unroll
  for (int q = 0; q < 5; q++)
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], off);
  const int warp = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int q = 0; q < 5; q++) red[warp][q] = acc[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    float s[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      s[q] = red[0][q];
#pragma unroll
      for (int r = 1; r < kDetThreads / 32; r++) s[q] += red[r][q];
    }
    d.ratio[w] = s[0];
    if (GL) {
      const float inv = 1.0f / s[0];
      if (d.grad) {
        d.grad[3 * (int64_t)w] = s[1] * inv;
        d.grad[3 * (int64_t)w + 1] = s[2] * inv;
        d.grad[3 * (int64_t)w + 2] = s[3] * inv;
      }
      if (d.lapl) d.lapl[w] = s[4] * inv;
    }
  }
}

// Pass 1, reference layout (Ainv[j][c] row-major): thread per column c,
// rows streamed in order with delta staged in shared memory; the thread that
// owns column k also copies that column out.
__global__ void __launch_bounds__(256) k_det_update1_rows(const DetArgs d) {
  __shared__ float sdelta[256];
  const int w = blockIdx.y;
  const int c = blockIdx.x * 256 + threadIdx.x;
  const float *ainv = d.ainv[w];
  const float *u = d.urow[w];
  const float *ak = d.amat[w] + (int64_t)d.k * d.ld;
  float *x = d.work + (int64_t)w * 2 * d.n, *colk = x + d.n;
  float acc = 0.f;
  for (int j0 = 0; j0 < d.n; j0 += 256) {
    const int jn = min(256, d.n - j0);
    __syncthreads();
    if (threadIdx.x < jn) sdelta[threadIdx.x] = u[j0 + threadIdx.x] - ak[j0 + threadIdx.x];
    __syncthreads();
    if (c < d.n) {
      for (int i = 0; i < jn; i++) {
        const float v = ainv[(int64_t)(j0 + i) * d.ld + c];
        if (c == d.k) colk[j0 + i] = v;
        acc = fmaf(v, sdelta[i], acc);
      }
    }
  }
  if (c < d.n) x[c] = acc;
}

// Pass 1, transposed layout (AinvT[c][j]): warp per row c, a dot product
// with delta; the warp on row k also copies that row (column k of Ainv).
__global__ void __launch_bounds__(256) k_det_update1_trans(const DetArgs d) {
  const int w = blockIdx.y;
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= d.n) return;
  const float *ainvr = d.ainv[w] + (int64_t)c * d.ld;
  const float *u = d.urow[w];
  const float *ak = d.amat[w] + (int64_t)d.k * d.ld;
  float *x = d.work + (int64_t)w * 2 * d.n, *colk = x + d.n;
  float acc = 0.f;
  for (int j = lane; j < d.n; j += 32) {
    const float v = ainvr[j];
    if (c == d.k) colk[j] = v;
    acc = fmaf(v, u[j] - ak[j], acc);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) x[c] = acc;
}

// Pass 2: rank-1 correction of every entry and the new row of A.
// Row r of the stored matrix: orbital j = r (reference layout) or electron
// c = r (transposed).
__global__ void __launch_bounds__(256) k_det_update2(const DetArgs d) {
  const int w = blockIdx.y;
  const int r = blockIdx.x;
  const float *x = d.work + (int64_t)w * 2 * d.n, *colk = x + d.n;
  const float p = -1.0f / (1.0f + x[d.k]);
  float *m = const_cast<float *>(d.ainv[w]) + (int64_t)r * d.ld;
  if (!d.trans) {
    const float f = p * colk[r];
    for (int c = threadIdx.x; c < d.n; c += blockDim.x) m[c] = fmaf(x[c], f, m[c]);
  } else {
    const float xr = x[r];
    for (int j = threadIdx.x; j < d.n; j += blockDim.x) m[j] = fmaf(xr, p * colk[j], m[j]);
  }
  if (r == d.k) {
    float *ak = d.amat[w] + (int64_t)d.k * d.ld;
    const float *u = d.urow[w];
    for (int j = threadIdx.x; j < d.n; j += blockDim.x) ak[j] = u[j];
  }
}

}  // namespace eg

using namespace eg;

namespace {

int check_det_opts(const einspline_gb300_det_opts *o, const char *fn) {
  if (!o) return fail(EINSPLINE_GB300_EINVAL, "%s: NULL options", fn);
  if (o->nelec <= 0) return fail(EINSPLINE_GB300_EINVAL, "%s: nelec must be positive", fn);
  if (o->k < 0 || o->k >= o->nelec) return fail(EINSPLINE_GB300_EINVAL, "%s: k out of [0, nelec)", fn);
  if (o->ld < o->nelec) return fail(EINSPLINE_GB300_EINVAL, "%s: ld < nelec", fn);
  if (o->ainv_trans != 0 && o->ainv_trans != 1) return fail(EINSPLINE_GB300_EINVAL, "%s: ainv_trans must be 0 or 1", fn);
  if (o->rule != 0 && o->rule != 1) return fail(EINSPLINE_GB300_EINVAL, "%s: rule must be 0 or 1", fn);
  return 0;
}

template <int ST>
void launch_ratio(const DetArgs &d, bool gl, int nw, cudaStream_t s) {
  if (gl) k_det_ratio<ST, true><<<nw, kDetThreads, 0, s>>>(d);
  else k_det_ratio<ST, false><<<nw, kDetThreads, 0, s>>>(d);
}

}  // namespace

extern "C" {

int einspline_gb300_det_ratio(einspline_gb300_table *t, const einspline_gb300_det_opts *o, int nwalkers,
                              const void *pos_d, const float *const *ainv_d, float *ratio_d, float *grad_d,
                              float *lapl_d, float *const *row_d, void *stream) {
  static const char *fn = "einspline_gb300_det_ratio";
  clear();
  if (!table_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "%s: bad table handle", fn);
  if (int r = check_det_opts(o, fn)) return r;
  if (t->ncomp != 1 || t->storage == ST_F64)
    return fail(EINSPLINE_GB300_EINVAL, "%s: real float tables only (s kind, any float/16-bit storage)", fn);
  if (o->nelec > t->num_splines) return fail(EINSPLINE_GB300_EINVAL, "%s: nelec exceeds the table's splines", fn);
  if (nwalkers < 0) return fail(EINSPLINE_GB300_EINVAL, "%s: nwalkers < 0", fn);
  if (nwalkers == 0) return 0;
  if (!pos_d || !ainv_d || !ratio_d) return fail(EINSPLINE_GB300_EINVAL, "%s: NULL buffer", fn);
  if (int r = table_flush(t)) return r;
  DetArgs d;
  memset(&d, 0, sizeof(d));
  fill_eval_geometry(t, d.e);
  d.e.pos = pos_d;
  d.e.pos_f64 = o->pos_f64 ? 1 : 0;
  d.e.rule = o->rule;
  d.e.npts = nwalkers;
  d.ainv = ainv_d;
  d.row_out = row_d;
  d.ratio = ratio_d;
  d.grad = grad_d;
  d.lapl = lapl_d;
  d.n = o->nelec;
  d.k = o->k;
  d.ld = o->ld;
  d.trans = o->ainv_trans;
  const bool gl = grad_d || lapl_d;
  cudaStream_t s = stream ? (cudaStream_t)stream : cudaStreamLegacy;
  switch (t->storage) {
    case ST_F32: launch_ratio<ST_F32>(d, gl, nwalkers, s); break;
    case ST_F16: launch_ratio<ST_F16>(d, gl, nwalkers, s); break;
    case ST_BF16: launch_ratio<ST_BF16>(d, gl, nwalkers, s); break;
    default: launch_ratio<ST_I16>(d, gl, nwalkers, s); break;
  }
  EG_CUDA(cudaGetLastError());
  count_launch();
  return 0;
}

int einspline_gb300_det_update(const einspline_gb300_det_opts *o, int naccept, float *const *a_d,
                               float *const *ainv_d, const float *const *row_d, float *work_d, void *stream) {
  static const char *fn = "einspline_gb300_det_update";
  clear();
  if (int r = check_det_opts(o, fn)) return r;
  if (naccept < 0) return fail(EINSPLINE_GB300_EINVAL, "%s: naccept < 0", fn);
  if (naccept == 0) return 0;
  if (naccept > 65535) return fail(EINSPLINE_GB300_ESIZE, "%s: at most 65535 walkers per call", fn);
  if (!a_d || !ainv_d || !row_d || !work_d) return fail(EINSPLINE_GB300_EINVAL, "%s: NULL buffer", fn);
  DetArgs d;
  memset(&d, 0, sizeof(d));
  d.ainv = ainv_d;
  d.amat = a_d;
  d.urow = row_d;
  d.work = work_d;
  d.n = o->nelec;
  d.k = o->k;
  d.ld = o->ld;
  d.trans = o->ainv_trans;
  cudaStream_t s = stream ? (cudaStream_t)stream : cudaStreamLegacy;
  if (!d.trans) k_det_update1_rows<<<dim3((d.n + 255) / 256, naccept), 256, 0, s>>>(d);
  else k_det_update1_trans<<<dim3((d.n + 7) / 8, naccept), 256, 0, s>>>(d);
  EG_CUDA(cudaGetLastError());
  k_det_update2<<<dim3(d.n, naccept), 256, 0, s>>>(d);
  EG_CUDA(cudaGetLastError());
  count_launch(2);
  return 0;
}

}  // extern "C"
