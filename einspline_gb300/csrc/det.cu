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
// k_det_ratio fuses the first two: a block of 4 warps gathers the stencil
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
// Copy-pipeline depth: two stages keep a block at ~70 KB of shared memory so
// three blocks (12 warps) share an SM; the register cap of the kernel
// (launch bounds) matches.
constexpr int kDetStages = 2;
constexpr int kDetBlocksPerSM = 3;

// Inverse entry (orbital j, electron c).
__device__ __forceinline__ float ainv_at(const float *m, int j, int c, int ld, int trans) {
  return trans ? m[(int64_t)c * ld + j] : m[(int64_t)j * ld + c];
}

// Shared memory of k_det_ratio: the evaluation prologue's weights, cells and
// sources for pb walkers, the copy pipeline, and per-warp partial sums.
__host__ __device__ __forceinline__ size_t det_pipe_off(int pb) { return align_up(smem_total(pb, 4), 16); }
__host__ __device__ __forceinline__ size_t det_red_off(int pb, int rb) {
  return det_pipe_off(pb) + pipe_bytes(kDetThreads, rb, kDetStages);
}
__host__ __device__ __forceinline__ size_t det_ptr_off(int pb, int rb) {
  return align_up(det_red_off(pb, rb) + (size_t)pb * (kDetThreads / 32) * 5 * sizeof(float), 16);
}
__host__ __device__ __forceinline__ size_t det_av_off(int pb, int rb) {
  return align_up(det_ptr_off(pb, rb) + (size_t)pb * sizeof(void *), 16);
}
__host__ __device__ __forceinline__ size_t det_smem(int pb, int rb) {
  return det_av_off(pb, rb) + (size_t)kDetThreads * 8 * sizeof(float);
}

// A block takes pb walkers and all N orbitals, in column groups of
// kDetThreads * VW.  A pipeline stage is one x-plane (16 stencil rows) of one
// column group of one walker; as in k_eval_pipe each thread copies its own
// columns of the rows of stage s+2 into shared memory while it reduces stage
// s, and reads back only what it copied.  At the end of a walker's planes the
// thread dots its columns' value, gradient and Laplacian with the inverse
// column (loaded when the walker's first plane starts, so its latency hides
// behind the reduction); at the end of the walker each warp folds its lanes
// with a fixed shuffle tree into shared memory, and after the loop one thread
// per walker adds the warps in order.  WIDE (16-bit tables): 8 columns and
// one 16-byte copy per thread and row.
template <int ST, bool GL, bool WIDE>
__global__ void __launch_bounds__(kDetThreads, kDetBlocksPerSM) k_det_ratio(const DetArgs d) {
  using Raw = typename CT<ST>::Raw;
  static_assert(sizeof(typename CT<ST>::A) == 4, "determinant step: real float tables only");
  constexpr int VW = WIDE ? 2 * CT<ST>::VW : CT<ST>::VW;
  constexpr int RB = WIDE ? 2 * (int)sizeof(Raw) : (int)sizeof(Raw);
  constexpr int NW = kDetThreads / 32;
  extern __shared__ __align__(16) unsigned char smem[];
  const EvalArgs &a = d.e;
  const int64_t p0 = (int64_t)blockIdx.x * a.pb;
  const int pn = eval_prologue<float>(a, smem, p0, a.pb, threadIdx.x, kDetThreads);
  const float **sptr = reinterpret_cast<const float **>(smem + det_ptr_off(a.pb, RB));
  for (int q = threadIdx.x; q < pn; q += kDetThreads) sptr[q] = d.ainv[p0 + q];
  __syncthreads();
  const float *sw = reinterpret_cast<const float *>(smem);
  const int *sidx = reinterpret_cast<const int *>(smem + smem_w_bytes(a.pb, 4));
  const int64_t *ssrc = reinterpret_cast<const int64_t *>(smem + smem_w_bytes(a.pb, 4) + align_up((size_t)a.pb * 12, 8));
  unsigned char *pipe = smem + det_pipe_off(a.pb);
  float *red = reinterpret_cast<float *>(smem + det_red_off(a.pb, RB));
  // the thread's inverse-column entries of the walker in flight: copied with
  // the walker's first plane, read when that plane is reduced (the next
  // first plane is four stages later, after the pipeline's depth)
  float *avbuf = reinterpret_cast<float *>(smem + det_av_off(a.pb, RB)) + threadIdx.x * VW;

  constexpr int GC = kDetThreads * VW;  // columns per group
  const int G = (d.n + GC - 1) / GC;
  const int64_t xsb = a.xs * CT<ST>::BYTES, ysb = a.ys * CT<ST>::BYTES, zsb = a.zs * CT<ST>::BYTES;
  const char *cbase = reinterpret_cast<const char *>(a.coefs) + (int64_t)threadIdx.x * VW * CT<ST>::BYTES;
  const unsigned my = (unsigned)__cvta_generic_to_shared(pipe + (size_t)threadIdx.x * RB);
  constexpr unsigned row_step = (unsigned)(kDetThreads * RB), slot_step = 16u * row_step;
  const int S = pn * G * 4;
  auto issue = [&](int st) {
    const int i = st & 3, rest = st >> 2, g = rest % G, pp = rest / G;
    if ((g * kDetThreads + (int)threadIdx.x) * VW >= d.n) return;
    const char *plane = cbase + (int64_t)g * GC * CT<ST>::BYTES + (sidx[3 * pp] + i) * xsb +
                        sidx[3 * pp + 1] * ysb + sidx[3 * pp + 2] * zsb;
    const unsigned dst = my + (unsigned)(st % kDetStages) * slot_step;
#pragma unroll
    for (int r = 0; r < 16; r++) cp_async<RB>(dst + r * row_step, plane + (r >> 2) * ysb + (r & 3) * zsb);
    if (i == 0) {
      const int col0 = (g * kDetThreads + (int)threadIdx.x) * VW;
      const float *src = d.trans ? sptr[pp] + (int64_t)d.k * d.ld + col0 : sptr[pp] + (int64_t)col0 * d.ld + d.k;
      const unsigned av = (unsigned)__cvta_generic_to_shared(avbuf);
      if (d.trans && col0 + VW <= d.n && al16(src)) {
#pragma unroll
        for (int e = 0; e < VW; e += 4) cp_async<16>(av + 4 * e, reinterpret_cast<const char *>(src + e));
      } else {
        const int64_t step = d.trans ? 1 : d.ld;
#pragma unroll
        for (int e = 0; e < VW; e++)
          if (col0 + e < d.n) cp_async<4>(av + 4 * e, reinterpret_cast<const char *>(src + e * step));
      }
    }
  };
#pragma unroll
  for (int st = 0; st < kDetStages - 1; st++) {
    if (st < S) issue(st);
    cp_async_commit();
  }
  float o[10][VW];  // assigned by each point's plane 0
  float wz[3][4];
  float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  float av[VW];
  for (int st = 0; st < S; st++) {
    if (st + kDetStages - 1 < S) issue(st + kDetStages - 1);
    cp_async_commit();
    cp_async_wait<kDetStages - 1>();
    const int i = st & 3, rest = st >> 2, g = rest % G, pp = rest / G;
    const int col0 = (g * kDetThreads + (int)threadIdx.x) * VW;
    const bool live = col0 < d.n;
    const float *w = sw + pp * 36;
    if (i == 0) {
      z_weights<float>(w, wz);
      if (live) {
#pragma unroll
        for (int e = 0; e < VW; e++) av[e] = col0 + e < d.n ? avbuf[e] : 0.f;
      }
    }
    if (live) {
      const unsigned char *slot = pipe + (size_t)(st % kDetStages) * slot_step + (size_t)threadIdx.x * RB;
      reduce_plane<float, VW, GL>(
          i, w, wz,
          [&](int j, int k, float(&c)[VW]) {
            const Raw *rp = reinterpret_cast<const Raw *>(slot + (j * 4 + k) * row_step);
            if (WIDE) {
              float lo[CT<ST>::VW], hi[CT<ST>::VW];
              CT<ST>::decode(rp[0], lo);
              CT<ST>::decode(rp[1], hi);
#pragma unroll
              for (int e = 0; e < CT<ST>::VW; e++) { c[e] = lo[e]; c[CT<ST>::VW + e] = hi[e]; }
            } else {
              CT<ST>::decode(rp[0], *reinterpret_cast<float(*)[CT<ST>::VW]>(&c[0]));
            }
          },
          o);
    }
    if (i == 3) {
      if (live) {
        if (a.scale) {
#pragma unroll
          for (int e = 0; e < VW; e++) {
            const float sc = a.scale[col0 + e];
#pragma unroll
            for (int q = 0; q < (GL ? 10 : 1); q++) o[q][e] *= sc;
          }
        }
        float *row = d.row_out ? d.row_out[ssrc[pp]] : nullptr;
#pragma unroll
        for (int e = 0; e < VW; e++) {
          acc[0] = fmaf(o[0][e], av[e], acc[0]);
          if (GL) {
            acc[1] = fmaf(o[1][e], av[e], acc[1]);
            acc[2] = fmaf(o[2][e], av[e], acc[2]);
            acc[3] = fmaf(o[3][e], av[e], acc[3]);
            acc[4] = fmaf((o[4][e] + o[7][e]) + o[9][e], av[e], acc[4]);
          }
          if (row && col0 + e < d.n) row[col0 + e] = o[0][e];
        }
      }
      if (g == G - 1) {
#pragma unroll
        for (int q = 0; q < 5; q++) {
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], off);
          if ((threadIdx.x & 31) == 0) red[(pp * NW + (threadIdx.x >> 5)) * 5 + q] = acc[q];
          acc[q] = 0.f;
        }
      }
    }
  }
  __syncthreads();
  if ((int)threadIdx.x < pn) {
    const int pp = threadIdx.x;
    float s[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      s[q] = red[pp * NW * 5 + q];
#pragma unroll
      for (int r = 1; r < NW; r++) s[q] += red[(pp * NW + r) * 5 + q];
    }
    const int64_t wk = ssrc[pp];
    d.ratio[wk] = s[0];
    if (GL) {
      const float inv = 1.0f / s[0];
      if (d.grad) {
        d.grad[3 * wk] = s[1] * inv;
        d.grad[3 * wk + 1] = s[2] * inv;
        d.grad[3 * wk + 2] = s[3] * inv;
      }
      if (d.lapl) d.lapl[wk] = s[4] * inv;
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
// with delta (16-byte loads when the rows allow); the warp on row k also
// copies that row (column k of Ainv).
__global__ void __launch_bounds__(256) k_det_update1_trans(const DetArgs d) {
  const int w = blockIdx.y;
  const int c = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (c >= d.n) return;
  const float *ainvr = d.ainv[w] + (int64_t)c * d.ld;
  const float *u = d.urow[w];
  const float *ak = d.amat[w] + (int64_t)d.k * d.ld;
  float *x = d.work + (int64_t)w * 2 * d.n, *colk = x + d.n;
  const bool copy = c == d.k;
  float acc = 0.f;
  int j0 = 0;
  if (al16(ainvr) && al16(u) && al16(ak) && (!copy || al16(colk))) {
    const int n4 = d.n >> 2;
    for (int q = lane; q < n4; q += 32) {
      const float4 v = reinterpret_cast<const float4 *>(ainvr)[q];
      const float4 uu = reinterpret_cast<const float4 *>(u)[q];
      const float4 aa = reinterpret_cast<const float4 *>(ak)[q];
      if (copy) reinterpret_cast<float4 *>(colk)[q] = v;
      acc = fmaf(v.x, uu.x - aa.x, acc);
      acc = fmaf(v.y, uu.y - aa.y, acc);
      acc = fmaf(v.z, uu.z - aa.z, acc);
      acc = fmaf(v.w, uu.w - aa.w, acc);
    }
    j0 = n4 << 2;
  }
  for (int j = j0 + lane; j < d.n; j += 32) {
    const float v = ainvr[j];
    if (copy) colk[j] = v;
    acc = fmaf(v, u[j] - ak[j], acc);
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, off);
  if (lane == 0) x[c] = acc;
}

// Pass 2: rank-1 correction of every entry and the new row of A; warp per
// stored row, 16-byte accesses when the row allows.  Entry (orbital j,
// electron c) becomes Ainv + x[c] * (p * colk[j]) in both layouts (the
// reference's kernel 2 expression, src/determinant_update.h:104-106).
__global__ void __launch_bounds__(256) k_det_update2(const DetArgs d) {
  const int w = blockIdx.y;
  const int r = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (r >= d.n) return;
  const float *x = d.work + (int64_t)w * 2 * d.n, *colk = x + d.n;
  const float p = -1.0f / (1.0f + x[d.k]);
  float *m = const_cast<float *>(d.ainv[w]) + (int64_t)r * d.ld;
  // reference layout: row r is orbital j = r, columns are electrons c;
  // transposed: row r is electron c = r, columns are orbitals j
  const float *vec = d.trans ? colk : x;
  const float rs = d.trans ? x[r] : p * colk[r];
  int i0 = 0;
  if (al16(m) && al16(vec)) {
    const int n4 = d.n >> 2;
    for (int q = lane; q < n4; q += 32) {
      float4 mv = reinterpret_cast<float4 *>(m)[q];
      const float4 v = reinterpret_cast<const float4 *>(vec)[q];
      if (d.trans) {
        mv.x = fmaf(rs, p * v.x, mv.x); mv.y = fmaf(rs, p * v.y, mv.y);
        mv.z = fmaf(rs, p * v.z, mv.z); mv.w = fmaf(rs, p * v.w, mv.w);
      } else {
        mv.x = fmaf(v.x, rs, mv.x); mv.y = fmaf(v.y, rs, mv.y);
        mv.z = fmaf(v.z, rs, mv.z); mv.w = fmaf(v.w, rs, mv.w);
      }
      reinterpret_cast<float4 *>(m)[q] = mv;
    }
    i0 = n4 << 2;
  }
  for (int i = i0 + lane; i < d.n; i += 32) m[i] = d.trans ? fmaf(rs, p * vec[i], m[i]) : fmaf(vec[i], rs, m[i]);
  if (r == d.k) {
    float *ak = d.amat[w] + (int64_t)d.k * d.ld;
    const float *u = d.urow[w];
    for (int j = lane; j < d.n; j += 32) ak[j] = u[j];
  }
}

}  // namespace eg

using namespace eg;

namespace {

int num_sms() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 152;
  }
  return n;
}

int check_det_opts(const einspline_gb300_det_opts *o, const char *fn) {
  if (!o) return fail(EINSPLINE_GB300_EINVAL, "%s: NULL options", fn);
  if (o->nelec <= 0) return fail(EINSPLINE_GB300_EINVAL, "%s: nelec must be positive", fn);
  if (o->k < 0 || o->k >= o->nelec) return fail(EINSPLINE_GB300_EINVAL, "%s: k out of [0, nelec)", fn);
  if (o->ld < o->nelec) return fail(EINSPLINE_GB300_EINVAL, "%s: ld < nelec", fn);
  if (o->ainv_trans != 0 && o->ainv_trans != 1) return fail(EINSPLINE_GB300_EINVAL, "%s: ainv_trans must be 0 or 1", fn);
  if (o->rule != 0 && o->rule != 1) return fail(EINSPLINE_GB300_EINVAL, "%s: rule must be 0 or 1", fn);
  return 0;
}

template <int ST, bool GL>
cudaError_t launch_ratio_k(const DetArgs &d, unsigned grid, cudaStream_t s) {
  constexpr bool WIDE = ST != ST_F32;
  constexpr int RB = WIDE ? 16 : (int)sizeof(typename CT<ST>::Raw);
  const size_t sm = det_smem(d.e.pb, RB);
  const void *f = (const void *)k_det_ratio<ST, GL, WIDE>;
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_det_ratio<ST, GL, WIDE><<<grid, kDetThreads, sm, s>>>(d);
  return cudaGetLastError();
}

template <int ST>
cudaError_t launch_ratio(const DetArgs &d, bool gl, unsigned grid, cudaStream_t s) {
  return gl ? launch_ratio_k<ST, true>(d, grid, s) : launch_ratio_k<ST, false>(d, grid, s);
}

}  // namespace

extern "C" {

int einspline_gb300_det_ratio(einspline_gb300_table *t, const einspline_gb300_det_opts *o, int nwalkers,
                              const void *pos_d, const float *const *ainv_d, float *ratio_d, float *grad_d,
                              float *lapl_d, float *const *row_d, void *stream) {
  static const char *fn = "einspline_gb300_det_ratio";
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "%s: bad table handle", fn);
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
  // kDetBlocksPerSM blocks fit on an SM.  The walkers are spread evenly
  // over at most one wave of such blocks, so each block runs one long
  // pipeline over its walkers (no per-block fill and drain for every walker,
  // no partial last wave); beyond 32 walkers per block the grid grows
  // instead.
  const int slots = kDetBlocksPerSM * num_sms();
  int pb = (nwalkers + slots - 1) / slots;
  pb = pb < 1 ? 1 : (pb > 32 ? 32 : pb);
  d.e.pb = pb;
  const unsigned grid = (unsigned)((nwalkers + pb - 1) / pb);
  cudaError_t e;
  switch (t->storage) {
    case ST_F32: e = launch_ratio<ST_F32>(d, gl, grid, s); break;
    case ST_F16: e = launch_ratio<ST_F16>(d, gl, grid, s); break;
    case ST_BF16: e = launch_ratio<ST_BF16>(d, gl, grid, s); break;
    default: e = launch_ratio<ST_I16>(d, gl, grid, s); break;
  }
  EG_CUDA(e);
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
  k_det_update2<<<dim3((d.n + 7) / 8, naccept), 256, 0, s>>>(d);
  EG_CUDA(cudaGetLastError());
  count_launch(2);
  return 0;
}

}  // extern "C"
