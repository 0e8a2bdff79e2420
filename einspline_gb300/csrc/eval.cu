// Evaluation kernels: value and value+gradient+Hessian of every spline of a
// uniform 3D multi-spline at many points (src/multi_bspline_cuda_s_impl.h:179
// and :343 for the batched GPU entries, src/multi_bspline_eval_std_s_impl.h:480
// and :740 for the CPU entries; d, c, z alike).
//
// Work split: a block owns pb points and a tile of tx*VW consecutive real
// columns (splines, or re/im halves of complex splines).  Each thread owns VW
// consecutive columns and reads every stencil row with one 16-byte (FP32,
// FP64) or 8-byte (FP16/BF16) load, so a warp reads 512/256 contiguous bytes
// per row.  Cell and basis weights of the block's points are computed once
// in a prologue and kept in shared memory.  The 64-row stencil is reduced
// separably -- z first (3 sums per row pair), then y (6), then x (10) -- 328
// multiply-adds per column and point instead of 640; the order does not
// depend on the tile shape, so a point's results are bit-identical whichever
// block or batch evaluates it.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <limits.h>
#include <string.h>

#include <map>
#include <mutex>
#include <tuple>

#include "eval_core.h"

namespace eg {

int elems_per_thread(const Table *t) { return t->storage == ST_F64 ? 2 : 4; }
static int acc_bytes(const Table *t) { return t->storage == ST_F64 ? 8 : 4; }

template <int N>
__device__ __forceinline__ void st_vec(float *p, const float (&v)[N]) {
#pragma unroll
  for (int c = 0; c < N / 4; c++)
    __stcs(reinterpret_cast<float4 *>(p) + c, make_float4(v[4 * c], v[4 * c + 1], v[4 * c + 2], v[4 * c + 3]));
}
template <int N>
__device__ __forceinline__ void st_vec(double *p, const double (&v)[N]) {
#pragma unroll
  for (int c = 0; c < N / 2; c++) __stcs(reinterpret_cast<double2 *>(p) + c, make_double2(v[2 * c], v[2 * c + 1]));
}
// Index of Hessian entry m (row-major 3x3) among (xx, xy, xz, yy, yz, zz).
__device__ __forceinline__ int h9to6(int m) {
  return (m == 0) ? 0 : (m == 1 || m == 3) ? 1 : (m == 2 || m == 6) ? 2 : (m == 4) ? 3 : (m == 5 || m == 7) ? 4 : 5;
}

template <typename A, int VW, bool VGH, bool SCALE = true>
__device__ __forceinline__ void epilogue(const EvalArgs &a, int64_t src, int col0, A (&o)[10][VW]) {
  if (SCALE && a.scale) {
    float sc[VW];
    if constexpr (VW % 4 != 0) {
#pragma unroll
      for (int e = 0; e < VW; e++) sc[e] = a.scale[col0 + e];
    }
#pragma unroll
    for (int c = 0; c < VW / 4; c++) {
      const float4 s4 = *reinterpret_cast<const float4 *>(a.scale + col0 + 4 * c);
      sc[4 * c] = s4.x; sc[4 * c + 1] = s4.y; sc[4 * c + 2] = s4.z; sc[4 * c + 3] = s4.w;
    }
    if constexpr (std::is_same<A, float>::value && VW % 2 == 0) {
      // column pairs in one packed multiply each (the same IEEE products)
#pragma unroll
      for (int q = 0; q < (VGH ? 10 : 1); q++)
#pragma unroll
        for (int e = 0; e < VW; e += 2)
          upk2(mul2(pk2(o[q][e], o[q][e + 1]), pk2(sc[e], sc[e + 1])), o[q][e], o[q][e + 1]);
    } else {
#pragma unroll
      for (int q = 0; q < (VGH ? 10 : 1); q++)
#pragma unroll
        for (int e = 0; e < VW; e++) o[q][e] *= (A)sc[e];
    }
  }
  if (a.sign) {
    const A sg = reinterpret_cast<const A *>(a.sign)[src];
#pragma unroll
    for (int q = 0; q < (VGH ? 10 : 1); q++)
#pragma unroll
      for (int e = 0; e < VW; e++) o[q][e] *= sg;
  }
  A *vp = a.vals_pp ? (A *)a.vals_pp[src] : (A *)a.vals + src * a.vstride;
  // vector stores need whole 16-byte groups of columns in this thread
  const bool full = (sizeof(A) == 8 ? VW % 2 == 0 : VW % 4 == 0) && col0 + VW <= a.ncol;
  {
    A v[VW];
#pragma unroll
    for (int e = 0; e < VW; e++) v[e] = o[0][e];
    if (full && al16(vp + col0)) st_vec<VW>(vp + col0, v);
    else
#pragma unroll
      for (int e = 0; e < VW; e++)
        if (col0 + e < a.ncol) vp[col0 + e] = v[e];
  }
  if (!VGH) return;
  if (a.out == 1) {
    // Lattice transform (src/multi_bspline_cuda_s_impl.h:706-733): rows
    // G.grad (3) and Tr(G^T G H), each lrow reals apart.
    const A *L = reinterpret_cast<const A *>(a.linv);
    A G[9];
#pragma unroll
    for (int m = 0; m < 9; m++) G[m] = L[m];
    A GG[3][3];
#pragma unroll
    for (int r = 0; r < 3; r++)
#pragma unroll
      for (int c = 0; c < 3; c++) GG[r][c] = G[r] * G[c] + G[3 + r] * G[3 + c] + G[6 + r] * G[6 + c];
    A *gl = (A *)a.grads_pp[src];
    A row[4][VW];
#pragma unroll
    for (int e = 0; e < VW; e++) {
      const A gx = o[1][e], gy = o[2][e], gz = o[3][e];
      const A hxx = o[4][e], hxy = o[5][e], hxz = o[6][e], hyy = o[7][e], hyz = o[8][e], hzz = o[9][e];
#pragma unroll
      for (int r = 0; r < 3; r++) row[r][e] = G[3 * r] * gx + G[3 * r + 1] * gy + G[3 * r + 2] * gz;
      row[3][e] = GG[0][0] * hxx + GG[1][0] * hxy + GG[2][0] * hxz + GG[0][1] * hxy + GG[1][1] * hyy +
                  GG[2][1] * hyz + GG[0][2] * hxz + GG[1][2] * hyz + GG[2][2] * hzz;
    }
#pragma unroll
    for (int r = 0; r < 4; r++) {
      A *rp = gl + r * a.lrow + col0;
      if (full && al16(rp)) st_vec<VW>(rp, row[r]);
      else
#pragma unroll
        for (int e = 0; e < VW; e++)
          if (col0 + e < a.ncol) rp[e] = row[r][e];
    }
    return;
  }
  A *gp = a.grads_pp ? (A *)a.grads_pp[src] : (A *)a.grads + src * a.gstride;
  A *hp = a.hess_pp ? (A *)a.hess_pp[src] : (A *)a.hess + src * a.hstride;
  const bool cpx_cpu = a.is_complex && a.layout == 1;
  {
    A g[3 * VW];
#pragma unroll
    for (int e = 0; e < VW; e++)
#pragma unroll
      for (int c = 0; c < 3; c++) {
        const int idx = cpx_cpu ? 6 * (e >> 1) + 2 * c + (e & 1) : 3 * e + c;
        g[idx] = o[1 + c][e];
      }
    A *gb = gp + 3 * (int64_t)col0;
    if (full && al16(gb)) st_vec<3 * VW>(gb, g);
    else
#pragma unroll
      for (int e = 0; e < VW; e++)
        if (col0 + e < a.ncol)
#pragma unroll
          for (int c = 0; c < 3; c++) {
            const int idx = cpx_cpu ? 6 * (e >> 1) + 2 * c + (e & 1) : 3 * e + c;
            gb[idx] = g[idx];
          }
  }
  if (a.out == 3) return;
  if (a.out == 2) {
    // CPU vgl (src/multi_bspline_eval_std_s_impl.h:724-731): lapl = (xx + yy) + zz.
    A l[VW];
#pragma unroll
    for (int e = 0; e < VW; e++) l[e] = (o[4][e] + o[7][e]) + o[9][e];
    A *lb = hp + col0;
    if (full && al16(lb)) st_vec<VW>(lb, l);
    else
#pragma unroll
      for (int e = 0; e < VW; e++)
        if (col0 + e < a.ncol) lb[e] = l[e];
    return;
  }
  if (a.layout == 0) {
    A h[6 * VW];
#pragma unroll
    for (int e = 0; e < VW; e++)
#pragma unroll
      for (int q = 0; q < 6; q++) h[6 * e + q] = o[4 + q][e];
    A *hb = hp + 6 * (int64_t)col0;
    if (full && al16(hb)) st_vec<6 * VW>(hb, h);
    else
#pragma unroll
      for (int e = 0; e < VW; e++)
        if (col0 + e < a.ncol)
#pragma unroll
          for (int q = 0; q < 6; q++) hb[6 * e + q] = h[6 * e + q];
  } else {
    A h[9 * VW];
#pragma unroll
    for (int e = 0; e < VW; e++)
#pragma unroll
      for (int m = 0; m < 9; m++) {
        const int idx = a.is_complex ? 18 * (e >> 1) + 2 * m + (e & 1) : 9 * e + m;
        h[idx] = o[4 + h9to6(m)][e];
      }
    A *hb = hp + 9 * (int64_t)col0;
    if (full && al16(hb)) st_vec<9 * VW>(hb, h);
    else
#pragma unroll
      for (int e = 0; e < VW; e++)
        if (col0 + e < a.ncol)
#pragma unroll
          for (int m = 0; m < 9; m++) {
            const int idx = a.is_complex ? 18 * (e >> 1) + 2 * m + (e & 1) : 9 * e + m;
            hb[idx] = h[idx];
          }
  }
}

template <int ST, bool VGH>
__global__ void __launch_bounds__(256) k_eval(const EvalArgs a) {
  using A = typename CT<ST>::A;
  constexpr int VW = CT<ST>::VW;
  extern __shared__ __align__(16) unsigned char smem[];
  A *sw = reinterpret_cast<A *>(smem);
  int *sidx = reinterpret_cast<int *>(smem + smem_w_bytes(a.pb, sizeof(A)));
  int64_t *ssrc = reinterpret_cast<int64_t *>(smem + smem_w_bytes(a.pb, sizeof(A)) + align_up((size_t)a.pb * 12, 8));

  const int tile = blockIdx.x % a.ntiles;
  const int64_t grp = blockIdx.x / a.ntiles;
  const int64_t p0 = group_first(a, grp);
  const int pn = (int)min((int64_t)group_cap(a, grp), a.npts - p0);
  const int nthr = blockDim.x * blockDim.y;
  const int tid = threadIdx.y * blockDim.x + threadIdx.x;
  for (int q = tid; q < pn * 3; q += nthr) {
    const int pp = q / 3, ax = q - 3 * pp;
    const int64_t src = a.perm ? (int64_t)a.perm[p0 + pp] : p0 + pp;
    double xd;
    if (!a.pos) xd = a.inl[ax];
    else if (a.pos_f64) xd = reinterpret_cast<const double *>(a.pos)[3 * src + ax];
    else xd = (double)reinterpret_cast<const float *>(a.pos)[3 * src + ax];
    int idx;
    if constexpr (ST == ST_DF) {
      // FP64 cell and weights, carried into the reduction as hi + lo
      double t, w[12];
      cell(a, ax, xd, idx, t);
      bspline_weights<double>(t, w, a.dinv[ax]);
#pragma unroll
      for (int m = 0; m < 12; m++) sw[pp * 36 + ax * 12 + m] = to_dfl(w[m]);
    } else {
      A t;
      cell(a, ax, xd, idx, t);
      bspline_weights<A>(t, sw + pp * 36 + ax * 12, sizeof(A) == 4 ? (A)a.dinvf[ax] : (A)a.dinv[ax]);
    }
    sidx[pp * 3 + ax] = idx;
    if (ax == 0) ssrc[pp] = src;
  }
  __syncthreads();

  if (a.mode == 1) {
    // Ask L2 for every stencil row segment of this block's points at once:
    // the bulk prefetches hold no registers, so the DRAM requests of all pb
    // points are in flight together and the loads below mostly hit L2.
    const int64_t c0 = (int64_t)tile * blockDim.x * VW;
    const int64_t cn = min((int64_t)a.ncol_pad, c0 + (int64_t)blockDim.x * VW) - c0;
    const unsigned bytes = (unsigned)(cn * CT<ST>::BYTES);
    const char *tb = reinterpret_cast<const char *>(a.coefs) + c0 * CT<ST>::BYTES;
    for (int q = tid; q < pn * 64; q += nthr) {
      const int pp = q >> 6, r = q & 63;
      const int64_t off = (int64_t)(sidx[3 * pp] + (r >> 4)) * a.xs + (int64_t)(sidx[3 * pp + 1] + ((r >> 2) & 3)) * a.ys +
                          (int64_t)(sidx[3 * pp + 2] + (r & 3)) * a.zs;
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(tb + off * CT<ST>::BYTES), "r"(bytes)
                   : "memory");
    }
  }

  const int col0 = (tile * blockDim.x + threadIdx.x) * VW;
  if (col0 >= a.ncol) return;
  const char *cbase = reinterpret_cast<const char *>(a.coefs) + (int64_t)col0 * CT<ST>::BYTES;
  const int64_t xsb = a.xs * CT<ST>::BYTES, ysb = a.ys * CT<ST>::BYTES, zsb = a.zs * CT<ST>::BYTES;
  for (int pp = threadIdx.y; pp < pn; pp += blockDim.y) {
    const char *base = cbase + sidx[3 * pp] * xsb + sidx[3 * pp + 1] * ysb + sidx[3 * pp + 2] * zsb;
    A o[10][VW];
    contract<ST, VGH>(base, xsb, ysb, zsb, sw + pp * 36, o);
    if constexpr (ST == ST_DF) {
      double od[10][VW];
#pragma unroll
      for (int q = 0; q < (VGH ? 10 : 1); q++)
#pragma unroll
        for (int e = 0; e < VW; e++) od[q][e] = to_double(o[q][e]);
      epilogue<double, VW, VGH>(a, ssrc[pp], col0, od);
    } else {
      epilogue<A, VW, VGH>(a, ssrc[pp], col0, o);
    }
  }
}

// Pipelined variant: a stage is one x-plane (16 stencil rows) of one point.
// Each thread copies its own columns of the rows of stage s+2 into shared
// memory with asynchronous copies while it reduces stage s, so the bytes in
// flight are held in shared memory, not registers.  A thread only reads back
// what it copied itself: the copy-group waits order it, no block barrier is
// needed.  WIDE (16-bit tables): 8 columns and one 16-byte copy per thread
// and row instead of 4 columns and 8 bytes.  Same arithmetic, same order as
// k_eval.
template <int ST, bool VGH, bool WIDE>
__device__ __forceinline__ void eval_pipe_body(const EvalArgs &a) {
  using A = typename CT<ST>::A;
  using Raw = typename CT<ST>::Raw;
  constexpr int VW = WIDE ? 2 * CT<ST>::VW : CT<ST>::VW;
  constexpr int RB = WIDE ? 2 * (int)sizeof(Raw) : (int)sizeof(Raw);
  constexpr int NS = pipe_stages(ST, WIDE);
  extern __shared__ __align__(16) unsigned char smem[];
  const int tile = blockIdx.x % a.ntiles;
  const int64_t grp = blockIdx.x / a.ntiles;
  const int64_t p0 = group_first(a, grp);
  // The wide variant always runs one warp per block, which makes every
  // shared-memory row offset below a compile-time constant.
  const int nthr = WIDE ? 32 : blockDim.x;
  const int pn = eval_prologue<A>(a, smem, p0, group_cap(a, grp), threadIdx.x, nthr);
  __syncthreads();
  const A *sw = reinterpret_cast<const A *>(smem);
  const int *sidx = reinterpret_cast<const int *>(smem + smem_w_bytes(a.pb, sizeof(A)));
  const int64_t *ssrc =
      reinterpret_cast<const int64_t *>(smem + smem_w_bytes(a.pb, sizeof(A)) + align_up((size_t)a.pb * 12, 8));
  unsigned char *pipe = smem + align_up(smem_total(a.pb, sizeof(A)), 16);

  const int col0 = (tile * blockDim.x + threadIdx.x) * VW;
  if (col0 >= a.ncol) return;
  const char *cbase = reinterpret_cast<const char *>(a.coefs) + (int64_t)col0 * CT<ST>::BYTES;
  const int64_t xsb = a.xs * CT<ST>::BYTES, ysb = a.ys * CT<ST>::BYTES, zsb = a.zs * CT<ST>::BYTES;
  const unsigned my = (unsigned)__cvta_generic_to_shared(pipe + (size_t)threadIdx.x * RB);
  const unsigned row_step = (unsigned)(nthr * RB), slot_step = 16u * row_step;
  const int S = pn * 4;
  auto issue = [&](int st) {
    const int pp = st >> 2, i = st & 3;
    const char *plane = cbase + (sidx[3 * pp] + i) * xsb + sidx[3 * pp + 1] * ysb + sidx[3 * pp + 2] * zsb;
    const unsigned dst = my + (unsigned)(st % NS) * slot_step;
#pragma unroll
    for (int r = 0; r < 16; r++) cp_async<RB>(dst + r * row_step, plane + (r >> 2) * ysb + (r & 3) * zsb);
  };
#pragma unroll
  for (int st = 0; st < NS - 1; st++) {
    if (st < S) issue(st);
    cp_async_commit();
  }
  A o[10][VW];  // assigned by each point's plane 0
  A wz[3][4];
  for (int st = 0; st < S; st++) {
    if (st + NS - 1 < S) issue(st + NS - 1);
    cp_async_commit();
    cp_async_wait<NS - 1>();
    const int pp = st >> 2, i = st & 3;
    const A *w = sw + pp * 36;
    if (i == 0) z_weights<A>(w, wz);
    const unsigned char *slot = pipe + (size_t)(st % NS) * slot_step + (size_t)threadIdx.x * RB;
    reduce_plane<A, VW, VGH>(
        i, w, wz,
        [&](int j, int k, A(&c)[VW]) {
          const Raw *rp = reinterpret_cast<const Raw *>(slot + (j * 4 + k) * row_step);
          if (WIDE) {
            A lo[CT<ST>::VW], hi[CT<ST>::VW];
            CT<ST>::decode(rp[0], lo);
            CT<ST>::decode(rp[1], hi);
#pragma unroll
            for (int e = 0; e < CT<ST>::VW; e++) { c[e] = lo[e]; c[CT<ST>::VW + e] = hi[e]; }
          } else {
            CT<ST>::decode(rp[0], *reinterpret_cast<A(*)[CT<ST>::VW]>(&c[0]));
          }
        },
        o);
    if (i == 3) {
      if constexpr (ST == ST_DF) {
        double od[10][VW];
#pragma unroll
        for (int q = 0; q < (VGH ? 10 : 1); q++)
#pragma unroll
          for (int e = 0; e < VW; e++) od[q][e] = to_double(o[q][e]);
        epilogue<double, VW, VGH>(a, ssrc[pp], col0, od);
      } else {
        epilogue<A, VW, VGH>(a, ssrc[pp], col0, o);
      }
    }
  }
}

template <int ST, bool VGH, bool WIDE>
__global__ void __launch_bounds__(256) k_eval_pipe(const EvalArgs a) {
  eval_pipe_body<ST, VGH, WIDE>(a);
}

// The double-float variant is held to 128 registers (ptxas fits it without
// spills): registers then allow four warps a sub-partition, so shared memory
// (two 16 KB stages a warp) sets the residency, 12 warps per SM for 4-warp
// tiles and 14 for 2-warp tiles.  Measured on 48^3 x 512 at 32k points, tile
// 128x1x16: 2.05 ms against 2.10 ms with a 168-register cap (the same 12
// warps, scheduled differently).
template <bool VGH>
__global__ void __maxnreg__(128) k_eval_pipe_df(const EvalArgs a) {
  eval_pipe_body<ST_DF, VGH, false>(a);
}

// Tensor-map pipeline: a stage is again one x-plane of one point, but the
// block's whole 16-row slice of it arrives by one tiled TMA copy per box
// (a box is <= 256 stored reals wide x 4 z x 4 y x 1 x; a tile wider than
// that takes several boxes side by side), issued by thread 0 and completing on
// the stage's full mbarrier.  A box lands row by row, (j*4 + k) * box_bytes
// apart, which is the row layout the reduction reads.  Each warp releases a
// stage on its empty mbarrier once its lanes have read it; thread 0 waits
// for every warp's release before it refills the buffer.  Every thread reads
// 16 bytes a row: 8 columns of a 16-bit table, 4 FP32 or 2 double-float.
// Same arithmetic, same order as k_eval.  A wait that runs out sets
// a.wait_err, leaves the loop on every warp, and thread 0 then waits (again
// bounded) for the copies it issued before the block exits.
template <int ST, bool VGH>
__global__ void __launch_bounds__(256) k_eval_tma(const __grid_constant__ EvalArgs a) {
  using A = typename CT<ST>::A;
  using Raw = typename CT<ST>::Raw;
  constexpr bool WIDE = is16(ST);
  constexpr int VW = WIDE ? 2 * CT<ST>::VW : CT<ST>::VW;
  constexpr int NS = TmaStages<ST>::value;
  extern __shared__ __align__(16) unsigned char smem[];
  const int tile = blockIdx.x % a.ntiles;
  const int64_t grp = blockIdx.x / a.ntiles;
  const int64_t p0 = group_first(a, grp);
  const int nthr = blockDim.x;
  if (threadIdx.x == 0) tma_prefetch_map(&a.tmap);
  const int pn = eval_prologue<A>(a, smem, p0, group_cap(a, grp), threadIdx.x, nthr);
  const unsigned base_s = (unsigned)__cvta_generic_to_shared(smem);
  const unsigned pipe_s = (base_s + (unsigned)smem_total(a.pb, sizeof(A)) + 127u) & ~127u;
  const unsigned stage_bytes = 256u * (unsigned)nthr;
  const unsigned full_s = pipe_s + NS * stage_bytes, empty_s = full_s + 8 * NS;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int s = 0; s < NS; s++) {
      mbar_init(full_s + 8 * s, 1);
      mbar_init(empty_s + 8 * s, (unsigned)(nthr >> 5));
    }
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  const A *sw = reinterpret_cast<const A *>(smem);
  const int *sidx = reinterpret_cast<const int *>(smem + smem_w_bytes(a.pb, sizeof(A)));
  const int64_t *ssrc =
      reinterpret_cast<const int64_t *>(smem + smem_w_bytes(a.pb, sizeof(A)) + align_up((size_t)a.pb * 12, 8));
  const unsigned char *pipe = smem + (pipe_s - base_s);

  const int bb = a.box_bytes;
  const int nbox = (nthr * 16) / bb;
  const int c_first = tile * nthr * VW;  // first stored real of the block's tile
  const int box_cols = bb / CT<ST>::BYTES;
  const int col0 = c_first + threadIdx.x * VW;
  const bool active = col0 < a.ncol;
  const unsigned my = (unsigned)((threadIdx.x * 16 / bb) * 16 * bb + (threadIdx.x * 16) % bb);
  const int S = pn * 4;

  // Thread 0 only: refill the buffer of stage q once every warp has released
  // its previous stage (q - NS).
  const unsigned long long lim = a.wait_ns ? a.wait_ns : kWaitNs;
  auto produce = [&](int q) -> bool {
    const int slot = q % NS;
    if (q >= NS && !mbar_wait(empty_s + 8 * slot, (unsigned)((q / NS - 1) & 1), lim)) return false;
    // test hook: no arrival and no copy for this stage, so its full barrier
    // never completes and the consumers' bounded wait runs out
    if (a.test_skip == q + 1 && blockIdx.x == 0) return true;
    const int pp = q >> 2, i = q & 3;
    const unsigned full = full_s + 8 * slot;
    mbar_arrive_expect_tx(full, stage_bytes);
    for (int b = 0; b < nbox; b++)
      tma_load_4d(pipe_s + slot * stage_bytes + b * 16 * bb, &a.tmap, full, c_first + b * box_cols,
                  sidx[3 * pp + 2], sidx[3 * pp + 1], sidx[3 * pp] + i);
    return true;
  };
  int issued = 0;
  if (threadIdx.x == 0)
    for (; issued < NS - 1 && issued < S; issued++) produce(issued);

  A o[10][VW];  // assigned by each point's plane 0
  A wz[3][4];
  int st = 0;
  for (; st < S; st++) {
    bool good = true;
    if (threadIdx.x == 0 && issued < S) {
      good = produce(issued);
      if (good) issued++;
    }
    good = mbar_wait(full_s + 8 * (st % NS), (unsigned)((st / NS) & 1), lim) && good;
    if (!__all_sync(0xffffffffu, good)) break;
    const int pp = st >> 2, i = st & 3;
    const A *w = sw + pp * 36;
    if (i == 0) z_weights<A>(w, wz);
    const unsigned char *slot = pipe + (size_t)(st % NS) * stage_bytes + my;
    reduce_plane<A, VW, VGH>(
        i, w, wz,
        [&](int j, int k, A(&c)[VW]) {
          const Raw *rp = reinterpret_cast<const Raw *>(slot + (j * 4 + k) * bb);
          if (WIDE) {
            A lo[CT<ST>::VW], hi[CT<ST>::VW];
            CT<ST>::decode(rp[0], lo);
            CT<ST>::decode(rp[1], hi);
#pragma unroll
            for (int e = 0; e < CT<ST>::VW; e++) { c[e] = lo[e]; c[CT<ST>::VW + e] = hi[e]; }
          } else {
            CT<ST>::decode(rp[0], *reinterpret_cast<A(*)[CT<ST>::VW]>(&c[0]));
          }
        },
        o);
    __syncwarp();
    if ((threadIdx.x & 31) == 0) mbar_arrive(empty_s + 8 * (st % NS));
    if (i == 3) {
      if (active) {
        if constexpr (ST == ST_DF) {
          double od[10][VW];
#pragma unroll
          for (int q = 0; q < (VGH ? 10 : 1); q++)
#pragma unroll
            for (int e = 0; e < VW; e++) od[q][e] = to_double(o[q][e]);
          epilogue<double, VW, VGH>(a, ssrc[pp], col0, od);
        } else {
          epilogue<A, VW, VGH>(a, ssrc[pp], col0, o);
        }
      }
    }
  }
  if (st < S) {
    // A wait ran out: report it, and let no copy land after the block exits.
    if ((threadIdx.x & 31) == 0 && a.wait_err) {
      *(volatile int *)a.wait_err = 1;
      __threadfence_system();
    }
    if (threadIdx.x == 0)
      for (int q = st; q < issued; q++) mbar_wait(full_s + 8 * (q % NS), (unsigned)((q / NS) & 1), lim);
  }
}

// Tensor-core evaluation (load mode 5, F16 and BF16 tables).  For one point
// the ten outputs of a column are a product of the point's 10 x 64 stencil
// weights with the column's 64 stencil coefficients, so for each 128-column
// tile of its kTcCols columns a block computes, point after point of its
// group,
//   D[128 columns x 32] = A[128 columns x 64 rows] * B[64 rows x 32]
// with four tcgen05.mma (M 128, N 32, K 16: one per x-plane) into f32
// accumulators in tensor memory.  A is the stencil exactly as stored: TMA
// boxes of 64 columns x 4 z x 4 y x 4 x in the 128-byte swizzle, which is
// the MN-major operand layout.  B holds each output's weight w_x w_y w_z
// (FP32, without the delta_inv factors) split into parts of the table's
// type, each part in its own column: f16 high and low parts (22 bits), or
// bf16 high, middle and low parts (the weight exactly).  The products are
// exact and each column sums them in FP32; the epilogue adds an output's
// columns and scales the sum by its delta_inv factors, the spline's factor
// and the point's sign.  Results agree with the FMA kernels to FP32
// rounding (not bit for bit).  Four MMAs per tile, not one per x-plane and
// part: the MMA issue rate, not the math, bounded the cell-sorted case.
// Warp roles, synchronised only through mbarriers: warp 0 (one lane) keeps
// up to kTcStages stencil copies in flight, one stage per tile of a point;
// warp 1 (one lane) issues a tile's MMAs once its stencil, the point's
// weight matrix and a free accumulator are there, commits each tile to the
// barrier that frees its stage and each point to the one that fills the
// accumulator; warps 2-5 (each the TMEM lanes of its quarter: one column of
// every tile a thread) read a point's accumulator, build the weight matrix
// of the point two ahead in the buffer whose last reader was that point's
// MMAs, then store the point's outputs, so that the stores are not on the
// path from one point's MMAs to the next's.  Weight matrices and
// accumulators are double-buffered.
// Every wait is bounded and also ends once another role gave up (a shared
// flag): a block that gave up sets a.wait_err, waits (again bounded) for its
// copies and MMAs in flight, and frees its tensor memory.
template <int ST, bool VGH>
__global__ void __launch_bounds__(kTcThreads) k_eval_tc(const __grid_constant__ EvalArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NS = kTcStages, NP = TcCfg<ST>::parts, T = kTcTiles;
  constexpr unsigned kB = 4096u;  // bytes of a weight matrix: four 32 x 16 tiles
  constexpr unsigned kStage = 16384u, kAcc = T * kTcN;  // bytes of a stage (one tile), TMEM columns per accumulator
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int tile = blockIdx.x % a.ntiles;
  const int64_t grp = blockIdx.x / a.ntiles;
  const int64_t p0 = group_first(a, grp);
  float *sw = reinterpret_cast<float *>(smem);
  int *sidx = reinterpret_cast<int *>(smem + smem_w_bytes(a.pb, 4));
  int64_t *ssrc = reinterpret_cast<int64_t *>(smem + smem_w_bytes(a.pb, 4) + align_up((size_t)a.pb * 12, 8));
  const int pn = (int)min((int64_t)group_cap(a, grp), a.npts - p0);
  // cells and the unscaled basis weights (delta_inv applied to the outputs)
  for (int q = tid; q < pn * 3; q += kTcThreads) {
    const int pp = q / 3, ax = q - 3 * pp;
    const int64_t src = a.perm ? (int64_t)a.perm[p0 + pp] : p0 + pp;
    double xd;
    if (!a.pos) xd = a.inl[ax];
    else if (a.pos_f64) xd = reinterpret_cast<const double *>(a.pos)[3 * src + ax];
    else xd = (double)reinterpret_cast<const float *>(a.pos)[3 * src + ax];
    int idx;
    float t;
    cell(a, ax, xd, idx, t);
    bspline_weights<float>(t, sw + pp * 36 + ax * 12, 1.0f);
    sidx[pp * 3 + ax] = idx;
    if (ax == 0) ssrc[pp] = src;
  }
  const unsigned base_s = (unsigned)__cvta_generic_to_shared(smem);
  const unsigned a_s = (base_s + (unsigned)smem_total(a.pb, 4) + 1023u) & ~1023u;
  const unsigned b_s = a_s + NS * kStage;
  // mbarriers: full/empty per stage; weight matrix full, accumulator
  // full/empty per buffer; then the TMEM address, the abort flag and the
  // count of stencil stages the MMA warp consumed
  const unsigned full_s = b_s + 2 * kB, empty_s = full_s + 8 * NS, bfull_s = empty_s + 8 * NS;
  const unsigned tfull_s = bfull_s + 16, tempty_s = tfull_s + 16, slot_s = tempty_s + 16;
  unsigned char *bgen = smem + (b_s - base_s);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + (slot_s + 4 - base_s));
  volatile int *consumed = reinterpret_cast<volatile int *>(smem + (slot_s + 8 - base_s));
  // weight columns 10..15 (and all but 0 for value only) stay zero
  for (int e = tid; e < 2 * (int)kB / 16; e += kTcThreads) reinterpret_cast<uint4 *>(bgen)[e] = make_uint4(0, 0, 0, 0);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_s), "n"(2 * kAcc)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  if (tid == 32) {
#pragma unroll
    for (int s = 0; s < NS; s++) {
      mbar_init(full_s + 8 * s, 1);
      mbar_init(empty_s + 8 * s, 1);
    }
#pragma unroll
    for (int b = 0; b < 2; b++) {
      mbar_init(bfull_s + 8 * b, 128);
      mbar_init(tfull_s + 8 * b, 1);
      mbar_init(tempty_s + 8 * b, 128);
    }
    *abort_flag = 0;
    *consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  fence_proxy_async();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const unsigned tmem = *reinterpret_cast<volatile unsigned *>(smem + (slot_s - base_s));
  const int c_first = tile * kTcCols;
  const unsigned long long lim = a.wait_ns ? a.wait_ns : kWaitNs;
  // a bounded wait that also gives up once another role has
  auto wait = [&](unsigned bar, unsigned parity) -> bool {
    if (*abort_flag) return false;
    if (mbar_wait(bar, parity, lim)) return true;
    *abort_flag = 1;
    return false;
  };
  int issued = 0, skipped = -1, last_commit = -1;
  if (warp == 0) {
    if (lane == 0) {
      // stencil copies, one stage per tile of a point (unit u = p * T + t)
      tma_prefetch_map(&a.tmap);
      for (int u = 0; u < pn * T; u++) {
        const int s = u % NS, p = u / T, t = u % T;
        if (u >= NS && !wait(empty_s + 8 * s, (unsigned)((u / NS - 1) & 1))) break;
        issued = u + 1;
        // test hook: no copy for this point, so its wait runs out
        if (a.test_skip == p + 1 && blockIdx.x == 0) { skipped = p; continue; }
        mbar_arrive_expect_tx(full_s + 8 * s, kStage);
#pragma unroll
        for (int mg = 0; mg < 2; mg++)
          tma_load_4d(a_s + s * kStage + mg * 8192u, &a.tmap, full_s + 8 * s, c_first + 128 * t + 64 * mg,
                      sidx[3 * p + 2], sidx[3 * p + 1], sidx[3 * p]);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      // MMAs: per tile, the four x-planes against each part of the weights
      constexpr uint32_t idesc = umma_idesc_16(128, kTcN, TcCfg<ST>::fmt);
      bool go = true;
      for (int p = 0; p < pn && go; p++) {
        const int bb = p & 1;
        if (!wait(bfull_s + 8 * bb, (unsigned)((p >> 1) & 1))) break;
        if (p >= 2 && !wait(tempty_s + 8 * bb, (unsigned)(((p >> 1) - 1) & 1))) break;
#pragma unroll
        for (int t = 0; t < T; t++) {
          const int u = p * T + t, s = u % NS;
          if (!wait(full_s + 8 * s, (unsigned)((u / NS) & 1))) { go = false; break; }
          *consumed = u + 1;
          tc_fence_after();
#pragma unroll
          for (int i = 0; i < 4; i++)
            umma_f16(tmem + bb * kAcc + t * kTcN, umma_desc(a_s + s * kStage + i * 2048u, 8192u, 1024u, 2),
                     umma_desc(b_s + bb * kB + i * 1024u, 128u, 256u, 0), idesc, i > 0);
          umma_commit(empty_s + 8 * s);
          last_commit = p;
        }
        if (!go) break;
        umma_commit(tfull_s + 8 * bb);
      }
    }
  } else {
    // weight matrices and outputs: thread et owns column colr of every tile
    const int et = tid - 64;
    const int colr = (warp & 3) * 32 + lane;
    // this thread's share of a weight matrix: stencil row k, outputs 0-4
    // (even threads) or 5-9 (odd threads)
    const int k = et >> 1;
    const int ki = k >> 4, kj = (k >> 2) & 3, km = k & 3, kk = k & 15;
    const unsigned boff = ki * 1024 + (kk >> 3) * 128 + (kk & 7) * 2;
    // derivative orders in x, y, z of each output (v, gx, gy, gz, hxx, hxy, hxz, hyy, hyz, hzz)
    static constexpr int OA[10] = {0, 1, 0, 0, 2, 1, 1, 0, 0, 0};
    static constexpr int OB[10] = {0, 0, 1, 0, 0, 1, 0, 2, 1, 0};
    static constexpr int OC[10] = {0, 0, 0, 1, 0, 0, 1, 0, 1, 2};
    // the common batched form: flat outputs in the GPU layout, no sign
    const bool plain = VGH && a.out == 0 && a.layout == 0 && !a.vals_pp && !a.grads_pp && !a.hess_pp && !a.sign;
    // per column: the spline's factor times each output's delta_inv factors
    float f[T][10];
    {
      const float dx = a.dinvf[0], dy = a.dinvf[1], dz = a.dinvf[2];
      const float d[10] = {1.f, dx, dy, dz, dx * dx, dx * dy, dx * dz, dy * dy, dy * dz, dz * dz};
#pragma unroll
      for (int t = 0; t < T; t++) {
        const int col = c_first + t * 128 + colr;
        const float sc = (a.scale && col < a.ncol) ? a.scale[col] : 1.f;
#pragma unroll
        for (int q = 0; q < 10; q++) f[t][q] = sc * d[q];
      }
    }
    // Weight matrix of point p into buffer p & 1, then arrive on its barrier.
    auto build_b = [&](int p) {
      const float *w = sw + p * 36;
      unsigned char *bm = bgen + (p & 1) * kB + boff;
      // the nine basis weights of this stencil row (value, d1, d2 per axis)
      float wx[3], wy[3], wz[3];
#pragma unroll
      for (int d = 0; d < 3; d++) {
        wx[d] = w[4 * d + ki];
        wy[d] = w[12 + 4 * d + kj];
        wz[d] = w[24 + 4 * d + km];
      }
      // weight of output q at this row, split into the parts' tiles: f16 high
      // and low parts; bf16 high, middle and low parts (each remainder is
      // exact in FP32, and the three parts sum to the weight exactly)
      auto put = [&](auto qc) {
        constexpr int q = decltype(qc)::value;
        const float wq = wx[OA[q]] * wy[OB[q]] * wz[OC[q]];
        auto at = [&](int n) { return bm + (n >> 3) * 256 + (n & 7) * 16; };
        if constexpr (ST == ST_BF16) {
          const __nv_bfloat16 hi = __float2bfloat16_rn(wq);
          const float r1 = wq - __bfloat162float(hi);
          const __nv_bfloat16 mid = __float2bfloat16_rn(r1);
          const __nv_bfloat16 lo = __float2bfloat16_rn(r1 - __bfloat162float(mid));
          *reinterpret_cast<__nv_bfloat16 *>(at(3 * q)) = hi;
          *reinterpret_cast<__nv_bfloat16 *>(at(3 * q + 1)) = mid;
          *reinterpret_cast<__nv_bfloat16 *>(at(3 * q + 2)) = lo;
        } else {
          const __half hi = __float2half_rn(wq);
          const __half lo = __float2half_rn(wq - __half2float(hi));
          *reinterpret_cast<__half *>(at(2 * q)) = hi;
          *reinterpret_cast<__half *>(at(2 * q + 1)) = lo;
        }
      };
      if (!(et & 1)) {
        put(std::integral_constant<int, 0>());
        if constexpr (VGH) {
          put(std::integral_constant<int, 1>());
          put(std::integral_constant<int, 2>());
          put(std::integral_constant<int, 3>());
          put(std::integral_constant<int, 4>());
        }
      } else if constexpr (VGH) {
        put(std::integral_constant<int, 5>());
        put(std::integral_constant<int, 6>());
        put(std::integral_constant<int, 7>());
        put(std::integral_constant<int, 8>());
        put(std::integral_constant<int, 9>());
      }
      fence_proxy_async();
      mbar_arrive(bfull_s + 8 * (p & 1));
    };
    build_b(0);
    if (pn > 1) build_b(1);
    for (int p = 0; p < pn; p++) {
      const int bb = p & 1;
      if (!wait(tfull_s + 8 * bb, (unsigned)((p >> 1) & 1))) break;
      // the MMAs of point p, the last to read weight buffer bb, are
      // complete: point p + 2's weights go there now, so that its MMAs wait
      // on neither this point's stores nor their issue
      if (p + 2 < pn) build_b(p + 2);
      tc_fence_after();
      uint32_t rr[T][32];
#pragma unroll
      for (int t = 0; t < T; t++) tmem_ld32(tmem + ((unsigned)((warp & 3) * 32) << 16) + bb * kAcc + t * kTcN, rr[t]);
      tc_fence_before();
      mbar_arrive(tempty_s + 8 * bb);
      // each output: the sum of its weight parts' columns
      uint32_t r[T * 16];
#pragma unroll
      for (int t = 0; t < T; t++)
#pragma unroll
        for (int q = 0; q < 10; q++) {
          float v = __uint_as_float(rr[t][NP * q]);
#pragma unroll
          for (int h = 1; h < NP; h++) v += __uint_as_float(rr[t][NP * q + h]);
          r[t * 16 + q] = __float_as_uint(v);
        }
      const int64_t src = ssrc[p];
      if (plain) {
        // flat GPU layout: value, 3 gradient and 6 Hessian reals per column
        float *vp = reinterpret_cast<float *>(a.vals) + src * a.vstride;
        float *gp = reinterpret_cast<float *>(a.grads) + src * a.gstride;
        float *hp = reinterpret_cast<float *>(a.hess) + src * a.hstride;
#pragma unroll
        for (int t = 0; t < T; t++) {
          const int col = c_first + t * 128 + colr;
          if (col >= a.ncol) continue;
          float o[10];
#pragma unroll
          for (int q = 0; q < 10; q++) o[q] = __uint_as_float(r[t * 16 + q]) * f[t][q];
          vp[col] = o[0];
#pragma unroll
          for (int c = 0; c < 3; c++) gp[3 * col + c] = o[1 + c];
#pragma unroll
          for (int c = 0; c < 6; c++) hp[6 * col + c] = o[4 + c];
        }
        continue;
      }
#pragma unroll
      for (int t = 0; t < T; t++) {
        const int col = c_first + t * 128 + colr;
        if (col >= a.ncol) continue;
        float o[10][1];
#pragma unroll
        for (int q = 0; q < (VGH ? 10 : 1); q++) o[q][0] = __uint_as_float(r[t * 16 + q]) * f[t][q];
        epilogue<float, 1, VGH, false>(a, src, col, o);
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  if (*abort_flag) {
    // a wait ran out: report it, and let no copy or MMA outlive the block
    if (tid == 0) {
      if (a.wait_err) {
        *(volatile int *)a.wait_err = 1;
        __threadfence_system();
      }
      for (int u = *consumed; u < issued; u++)
        if (u / T != skipped) mbar_wait(full_s + 8 * (u % NS), (unsigned)((u / NS) & 1), lim);
    }
    // the last MMAs committed complete before their tensor memory is freed
    if (tid == 32 && last_commit >= 0) {
      const int u = *consumed - 1;
      mbar_wait(empty_s + 8 * (u % NS), (unsigned)((u / NS) & 1), lim);
    }
  }
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(2 * kAcc) : "memory");
}

// Index of third-derivative entry m (3x3x3 row-major, m = 9a + 3b + c) among
// the ten distinct ones (xxx, xxy, xxz, xyy, xyz, xzz, yyy, yyz, yzz, zzz).
__device__ __forceinline__ int g27to10(int m) {
  int a = m / 9, b = (m / 3) % 3, c = m % 3, t;
  if (a > b) { t = a; a = b; b = t; }
  if (b > c) { t = b; b = c; c = t; }
  if (a > b) { t = a; a = b; b = t; }
  // sorted (a <= b <= c): rank among the 10 multisets in lexicographic order
  return (a == 0) ? ((b == 0) ? c : (b == 1) ? 2 + c : 5) : (a == 1) ? ((b == 1) ? 5 + c : 8) : 9;
}

// Value, gradient, Hessian and third derivatives at one point
// (eval_multi_UBspline_3d_*_vghgh, src/multi_bspline_eval_std_s_impl.h:866-1038),
// CPU-entry cell rule and CPU layout.  The first ten outputs use exactly the
// operations of the vgh reduction, so they equal the vgh entry's bit for bit;
// the third derivatives add the constant rows {-1, 3, -3, 1} * delta_inv^3.
template <int ST>
__global__ void __launch_bounds__(128) k_eval_vghgh(const EvalArgs a) {
  using A = typename CT<ST>::A;
  constexpr int VW = CT<ST>::VW;
  const int col0 = (blockIdx.x * blockDim.x + threadIdx.x) * VW;
  if (col0 >= a.ncol) return;
  A w[36], w3[3][4];
  int idx[3];
#pragma unroll
  for (int ax = 0; ax < 3; ax++) {
    A t;
    cell(a, ax, a.inl[ax], idx[ax], t);
    const A d = sizeof(A) == 4 ? (A)a.dinvf[ax] : (A)a.dinv[ax];
    bspline_weights<A>(t, w + 12 * ax, d);
    const A d3 = (d * d) * d;
    w3[ax][0] = -d3; w3[ax][1] = A(3) * d3; w3[ax][2] = A(-3) * d3; w3[ax][3] = d3;
  }
  A wz[3][4];
  z_weights<A>(w, wz);
  const int64_t xsb = a.xs * CT<ST>::BYTES, ysb = a.ys * CT<ST>::BYTES, zsb = a.zs * CT<ST>::BYTES;
  const char *base = reinterpret_cast<const char *>(a.coefs) + (int64_t)col0 * CT<ST>::BYTES + idx[0] * xsb +
                     idx[1] * ysb + idx[2] * zsb;
  A o[20][VW];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    // y[0..5] as in reduce_plane; y[6..9] = b3c0, b2c1, b1c2, b0c3.  As
    // there, every sum starts with a product.
    A y[10][VW];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      A c[4][VW];
#pragma unroll
      for (int k = 0; k < 4; k++) load_row<ST>(base + i * xsb + j * ysb + k * zsb, c[k]);
      const A by = w[12 + j], dby = w[16 + j], d2by = w[20 + j], d3by = w3[1][j];
#pragma unroll
      for (int e = 0; e < VW; e++) {
        A z0 = c[0][e] * wz[0][0];
        z0 = fmaT(c[1][e], wz[0][1], z0);
        z0 = fmaT(c[2][e], wz[0][2], z0);
        z0 = fmaT(c[3][e], wz[0][3], z0);
        A z1 = c[0][e] * wz[1][0];
        z1 = fmaT(c[1][e], wz[1][1], z1);
        z1 = fmaT(c[2][e], wz[1][2], z1);
        z1 = fmaT(c[3][e], wz[1][3], z1);
        A z2 = c[0][e] * wz[2][0];
        z2 = fmaT(c[1][e], wz[2][1], z2);
        z2 = fmaT(c[2][e], wz[2][2], z2);
        z2 = fmaT(c[3][e], wz[2][3], z2);
        A z3 = c[0][e] * w3[2][0];
        z3 = fmaT(c[1][e], w3[2][1], z3);
        z3 = fmaT(c[2][e], w3[2][2], z3);
        z3 = fmaT(c[3][e], w3[2][3], z3);
        const A yw[10] = {by, dby, d2by, by, dby, by, d3by, d2by, dby, by};
        const A zz[10] = {z0, z0, z0, z1, z1, z2, z0, z1, z2, z3};
#pragma unroll
        for (int q = 0; q < 10; q++) y[q][e] = j == 0 ? yw[q] * zz[q] : fmaT(yw[q], zz[q], y[q][e]);
      }
    }
    const A ax = w[i], dax = w[4 + i], d2ax = w[8 + i], d3ax = w3[0][i];
    // o[q] += x weight * y[r]: value, gradient, Hessian (as in reduce_plane),
    // then xxx, xxy, xxz, xyy, xyz, xzz, yyy, yyz, yzz, zzz
    const A xw[20] = {ax, dax, ax, ax, d2ax, dax, dax, ax, ax, ax, d3ax, d2ax, d2ax, dax, dax, dax, ax, ax, ax, ax};
    constexpr int R[20] = {0, 0, 1, 3, 0, 1, 3, 2, 4, 5, 0, 1, 3, 2, 4, 5, 6, 7, 8, 9};
#pragma unroll
    for (int e = 0; e < VW; e++)
#pragma unroll
      for (int q = 0; q < 20; q++) o[q][e] = i == 0 ? xw[q] * y[R[q]][e] : fmaT(xw[q], y[R[q]][e], o[q][e]);
  }
  if (a.scale) {
#pragma unroll
    for (int e = 0; e < VW; e++) {
      const A sc = (A)a.scale[col0 + e];
#pragma unroll
      for (int q = 0; q < 20; q++) o[q][e] *= sc;
    }
  }
  A *vp = (A *)a.vals, *gp = (A *)a.grads, *hp = (A *)a.hess, *tp = (A *)a.ghess;
#pragma unroll
  for (int e = 0; e < VW; e++) {
    const int col = col0 + e;
    if (col >= a.ncol) break;
    // complex columns interleave re/im of one spline: element m of spline
    // col/2 sits at 2m + (col & 1) within that spline's block
    const int n = a.is_complex ? col >> 1 : col, p = a.is_complex ? col & 1 : 0, nc = a.is_complex ? 2 : 1;
    vp[col] = o[0][e];
#pragma unroll
    for (int c = 0; c < 3; c++) gp[nc * (3 * n + c) + p] = o[1 + c][e];
#pragma unroll
    for (int m = 0; m < 9; m++) hp[nc * (9 * n + m) + p] = o[4 + h9to6(m)][e];
#pragma unroll
    for (int m = 0; m < 27; m++) tp[nc * (27 * n + m) + p] = o[10 + g27to10(m)][e];
  }
}

int launch_vghgh(Table *t, const EvalArgs &a, cudaStream_t s) {
  const int VW = elems_per_thread(t);
  const int nthr = (a.ncol + VW - 1) / VW;
  const int tx = nthr < 128 ? (nthr + 31) / 32 * 32 : 128;
  const unsigned grid = (unsigned)((nthr + tx - 1) / tx);
  switch (t->storage) {
    case ST_F32: k_eval_vghgh<ST_F32><<<grid, tx, 0, s>>>(a); break;
    case ST_F16: k_eval_vghgh<ST_F16><<<grid, tx, 0, s>>>(a); break;
    case ST_BF16: k_eval_vghgh<ST_BF16><<<grid, tx, 0, s>>>(a); break;
    case ST_I16: k_eval_vghgh<ST_I16><<<grid, tx, 0, s>>>(a); break;
    default: k_eval_vghgh<ST_F64><<<grid, tx, 0, s>>>(a); break;
  }
  EG_CUDA(cudaGetLastError());
  count_launch();
  return 0;
}

void fill_eval_geometry(const Table *t, EvalArgs &a) {
  a.coefs = t->coefs;
  a.scale = t->scale;
  a.xs = t->xs; a.ys = t->ys; a.zs = t->zs;
  a.ncol = t->ncol;
  a.ncol_pad = t->ncol_pad;
  for (int i = 0; i < 3; i++) {
    a.lim[i] = t->Nc[i] - 4;
    a.start[i] = t->start[i];
    a.dinv[i] = t->dinv[i];
    a.dinvf[i] = (float)t->dinv[i];
  }
  a.is_complex = t->ncomp == 2;
}

// Load modes: 0 direct, 1 L2 prefetch + direct, 2 shared-memory pipeline,
// 3 shared-memory pipeline with 8 columns per thread (16-bit tables),
// 4 shared-memory pipeline fed by tensor-map (TMA) copies.
// (IEEE FP64 has only the direct-load kernel; the double-float path has the
// direct, the 4-column pipelined and the TMA kernels.)
template <int ST, bool VGH>
static const void *kernel_for(int mode) {
  if constexpr (ST != ST_F64) {
    if (mode == 4) return (const void *)k_eval_tma<ST, VGH>;
    if constexpr (ST == ST_DF) {
      if (mode == 2 || mode == 3) return (const void *)k_eval_pipe_df<VGH>;
    } else {
      if constexpr (ST == ST_F16 || ST == ST_BF16)
        if (mode == 5) return (const void *)k_eval_tc<ST, VGH>;
      if (mode == 2) return (const void *)k_eval_pipe<ST, VGH, false>;
      if (mode == 3) return (const void *)k_eval_pipe<ST, VGH, (ST == ST_F16 || ST == ST_BF16 || ST == ST_I16)>;
    }
  }
  return (const void *)k_eval<ST, VGH>;
}

template <int ST, bool VGH>
static cudaError_t launch_k(const EvalArgs &a, unsigned grid, dim3 block, size_t smem, cudaStream_t s) {
  const void *f = kernel_for<ST, VGH>(a.mode);
  void *args[] = {const_cast<EvalArgs *>(&a)};
  return cudaLaunchKernel(f, dim3(grid), block, args, smem, s);
}

// The kernel type of a table's launches: its storage, or the double-float
// shadow of an FP64 table in fp64_mode 1.
static int kernel_storage(const Table *t) {
  return (t->storage == ST_F64 && t->fp64_mode == 1 && t->df_coefs) ? (int)ST_DF : t->storage;
}

// The driver's tensor-map encoder, looked up once through the runtime (no
// link-time dependence on the driver library).
using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
static EncodeTiled encoder() {
  static EncodeTiled fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    return reinterpret_cast<EncodeTiled>(p);
  }();
  return fn;
}

// Tensor map of a table's coefficients (base: the stored table or its
// double-float shadow, es bytes per stored real) as [x][y][z][column], one
// box = box_cols columns x 4 z x 4 y x box_x x (box_x 4 with the 128-byte
// swizzle: the whole stencil in the tensor cores' operand layout).  Columns
// past ncol_pad read as zero.  The base is a cudaMalloc address and every
// stride a multiple of the 128-byte row, so the encoder's 16-byte rules hold.
static int encode_table_map(const Table *t, const void *base, int es, int box_cols, CUtensorMap *map,
                            int box_x = 1, CUtensorMapSwizzle swz = CU_TENSOR_MAP_SWIZZLE_NONE) {
  EncodeTiled fn = encoder();
  if (!fn) return fail(EINSPLINE_GB300_ECUDA, "cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[4] = {(cuuint64_t)t->ncol_pad, (cuuint64_t)t->Nc[2], (cuuint64_t)t->Nc[1],
                              (cuuint64_t)t->Nc[0]};
  const cuuint64_t strides[3] = {(cuuint64_t)(t->zs * es), (cuuint64_t)(t->ys * es), (cuuint64_t)(t->xs * es)};
  const cuuint32_t box[4] = {(cuuint32_t)box_cols, 4, 4, (cuuint32_t)box_x};
  const cuuint32_t estr[4] = {1, 1, 1, 1};
  const CUtensorMapDataType dt =
      es == 2 ? CU_TENSOR_MAP_DATA_TYPE_UINT16 : es == 4 ? CU_TENSOR_MAP_DATA_TYPE_UINT32 : CU_TENSOR_MAP_DATA_TYPE_UINT64;
  const CUresult r = fn(map, dt, 4, const_cast<void *>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        swz, CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(EINSPLINE_GB300_ECUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return 0;
}

// The tensor-core kernels' map: boxes of 64 columns x 4 z x 4 y x 4 x in
// the 128-byte swizzle (the MMA's MN-major operand layout).
int tc_table_map(const Table *t, EvalArgs &a) {
  return encode_table_map(t, a.coefs, 2, 64, &a.tmap, 4, CU_TENSOR_MAP_SWIZZLE_128B);
}

// Largest dynamic shared memory a block may opt into on the current device.
static size_t max_smem_optin() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) {
    cudaGetLastError();
    return 227 * 1024;
  }
  return (size_t)v;
}

// Kernel, block and dynamic shared memory of a launch; the pipelined kernels
// run one point lane (ty = 1) and need their stage buffers raised above the
// 48 KB default once per kernel.
static int shape_launch(Table *t, EvalArgs &a, bool vgh, int tx, int ty, int pb, const void **func, dim3 *block,
                        size_t *smem, int mode = -1) {
  if (tx < 32 || tx % 32 || ty < 1 || tx * ty > 256 || pb < 1 || pb > 64)
    return fail(EINSPLINE_GB300_EINVAL, "bad launch shape tx=%d ty=%d pb=%d", tx, ty, pb);
  a.pb = pb;
  a.mode = mode >= 0 ? mode : pick_mode(t, vgh, a.perm != nullptr);
  const int ks = kernel_storage(t);
  if (a.mode >= 2 && ks == ST_F64) a.mode = 0;        // IEEE FP64 is FMA-bound: no pipeline variant
  // tensor cores: F16 and BF16 tables; one column a thread, so not the
  // complex CPU layout, whose outputs interleave a spline's two columns
  if (a.mode == 5 && ((t->storage != ST_F16 && t->storage != ST_BF16) || (a.is_complex && a.layout == 1)))
    a.mode = is16(t->storage) ? 3 : 2;
  if (a.mode == 3 && !is16(t->storage)) a.mode = 2;   // the wide variant is for 16-bit tables
  const int VW = elems_per_thread(t) * ((a.mode == 3 || (a.mode == 4 && is16(t->storage))) ? 2 : 1);
  a.ntiles = (a.ncol + tx * VW - 1) / (tx * VW);
  *smem = smem_total(pb, acc_bytes(t));
  if (a.mode == 3) {
    tx = 32;  // the wide pipeline runs one warp per block
    a.ntiles = (a.ncol + tx * VW - 1) / (tx * VW);
  }
  if (ks == ST_DF) a.coefs = t->df_coefs;
  if (a.mode == 5) {
    tx = kTcThreads;
    ty = 1;
    a.ntiles = (a.ncol + kTcCols - 1) / kTcCols;
    a.wait_err = t->wait_err_d;
    if (int r = tc_table_map(t, a)) return r;
    *smem = tc_smem(pb);
  } else if (a.mode == 4) {
    ty = 1;
    // narrower tiles where the stage buffers would not fit in shared memory
    const int stages = ks == ST_DF ? TmaStages<ST_DF>::value : kTmaStages;
    while (tx > 32 && tma_smem(pb, acc_bytes(t), tx, stages) > max_smem_optin()) tx /= 2;
    a.ntiles = (a.ncol + tx * VW - 1) / (tx * VW);
    const int es = is16(t->storage) ? 2 : (ks == ST_F32 ? 4 : 8);
    a.box_bytes = tx * 16 < 256 * es ? tx * 16 : 256 * es;
    a.wait_err = t->wait_err_d;
    if (int r = encode_table_map(t, a.coefs, es, a.box_bytes / es, &a.tmap)) return r;
    *smem = tma_smem(pb, acc_bytes(t), tx, stages);
  } else if (a.mode >= 2) {
    ty = 1;
    const int rb = (ks == ST_F32 || ks == ST_DF || a.mode == 3) ? 16 : 8;
    *smem = align_up(*smem, 16) + pipe_bytes(tx, rb, pipe_stages(ks, a.mode == 3 && is16(ks)));
  }
  *block = dim3(tx, ty);
  switch (ks) {
    case ST_DF: *func = vgh ? kernel_for<ST_DF, true>(a.mode) : kernel_for<ST_DF, false>(a.mode); break;
    case ST_F32: *func = vgh ? kernel_for<ST_F32, true>(a.mode) : kernel_for<ST_F32, false>(a.mode); break;
    case ST_F16: *func = vgh ? kernel_for<ST_F16, true>(a.mode) : kernel_for<ST_F16, false>(a.mode); break;
    case ST_BF16: *func = vgh ? kernel_for<ST_BF16, true>(a.mode) : kernel_for<ST_BF16, false>(a.mode); break;
    case ST_I16: *func = vgh ? kernel_for<ST_I16, true>(a.mode) : kernel_for<ST_I16, false>(a.mode); break;
    default: *func = vgh ? kernel_for<ST_F64, true>(a.mode) : kernel_for<ST_F64, false>(a.mode); break;
  }
  if (*smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(*func, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)*smem);
    if (e != cudaSuccess) return cuda_check(e, "cudaFuncSetAttribute(max dynamic shared memory)");
  }
  return 0;
}

// Blocks of a kernel that one SM holds at once, looked up once per
// (kernel, block size, shared memory) on the current device.
static int resident_blocks(const void *func, int threads, size_t smem) {
  struct Key {
    const void *f;
    int threads, dev;
    size_t smem;
    bool operator<(const Key &o) const {
      return std::tie(f, threads, dev, smem) < std::tie(o.f, o.threads, o.dev, o.smem);
    }
  };
  static std::mutex mu;
  static std::map<Key, int> cache;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) { cudaGetLastError(); return 0; }
  const Key k{func, threads, dev, smem};
  std::lock_guard<std::mutex> g(mu);
  auto it = cache.find(k);
  if (it != cache.end()) return it->second;
  int per_sm = 0, sms = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, func, threads, smem) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return cache[k] = per_sm * sms;
}

// Point groups of a launch.  A launch of more than two waves gives the
// points of its last wave of full groups to groups of pb/4 points: every
// block computes its points the same way whatever its group holds, so the
// results do not change, and the launch ends with short blocks instead of
// SMs idling while the last full ones finish.
static int64_t plan_groups(EvalArgs &a, const void *func, dim3 block, size_t smem) {
  a.pb_tail = 0;
  a.g_tail = 0;
  const int64_t groups = (a.npts + a.pb - 1) / a.pb;
  if (a.pb < 4) return groups;
  const int64_t wave = (int64_t)resident_blocks(func, (int)(block.x * block.y), smem) / a.ntiles;
  if (wave <= 0 || groups <= 2 * wave) return groups;
  a.pb_tail = a.pb / 4;
  a.g_tail = groups - wave;
  const int64_t rest = a.npts - a.g_tail * a.pb;
  return a.g_tail + (rest + a.pb_tail - 1) / a.pb_tail;
}

int launch_eval(Table *t, EvalArgs &a, bool vgh, cudaStream_t s, int tx, int ty, int pb, int mode) {
  if (a.npts <= 0) return 0;
  const void *func;
  dim3 block;
  size_t smem;
  if (int r = shape_launch(t, a, vgh, tx, ty, pb, &func, &block, &smem, mode)) return r;
  if ((a.mode == 4 || a.mode == 5) && t->test_skip.load(std::memory_order_relaxed)) {
    a.test_skip = t->test_skip.exchange(0);
    a.wait_ns = t->test_wait_ns;
  }
  const int64_t blocks = plan_groups(a, func, block, smem) * a.ntiles;
  if (blocks > INT_MAX) return fail(EINSPLINE_GB300_ESIZE, "too many points in one call (%lld)", (long long)a.npts);
  cudaError_t e;
  switch (kernel_storage(t)) {
    case ST_DF: e = vgh ? launch_k<ST_DF, true>(a, (unsigned)blocks, block, smem, s)
                        : launch_k<ST_DF, false>(a, (unsigned)blocks, block, smem, s); break;
    case ST_F32: e = vgh ? launch_k<ST_F32, true>(a, (unsigned)blocks, block, smem, s)
                         : launch_k<ST_F32, false>(a, (unsigned)blocks, block, smem, s); break;
    case ST_F16: e = vgh ? launch_k<ST_F16, true>(a, (unsigned)blocks, block, smem, s)
                         : launch_k<ST_F16, false>(a, (unsigned)blocks, block, smem, s); break;
    case ST_BF16: e = vgh ? launch_k<ST_BF16, true>(a, (unsigned)blocks, block, smem, s)
                          : launch_k<ST_BF16, false>(a, (unsigned)blocks, block, smem, s); break;
    case ST_I16: e = vgh ? launch_k<ST_I16, true>(a, (unsigned)blocks, block, smem, s)
                         : launch_k<ST_I16, false>(a, (unsigned)blocks, block, smem, s); break;
    default: e = vgh ? launch_k<ST_F64, true>(a, (unsigned)blocks, block, smem, s)
                     : launch_k<ST_F64, false>(a, (unsigned)blocks, block, smem, s); break;
  }
  count_launch();
  if (e != cudaSuccess) return cuda_check(e, "evaluation kernel launch");
  return 0;
}

int load_eval_kernel(Table *t, bool vgh, bool sorted) {
  EvalArgs a;
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(t, a);
  static const int one = 0;
  if (sorted) a.perm = &one;  // only its presence matters: it selects the sorted launch shape
  int tx, ty, pb;
  pick_tile(t, vgh, 1, tx, ty, pb, sorted);
  const void *func;
  dim3 block;
  size_t smem;
  if (int r = shape_launch(t, a, vgh, tx, ty, pb, &func, &block, &smem)) return r;
  cudaFuncAttributes fa;
  EG_CUDA(cudaFuncGetAttributes(&fa, func));
  return 0;
}

int prepare_eval(Table *t, EvalArgs &a, bool vgh, int tx, int ty, int pb, const void **func, dim3 *grid,
                 dim3 *block, size_t *smem) {
  if (int r = shape_launch(t, a, vgh, tx, ty, pb, func, block, smem)) return r;
  const int64_t blocks = plan_groups(a, *func, *block, *smem) * a.ntiles;
  if (blocks > INT_MAX) return fail(EINSPLINE_GB300_ESIZE, "too many points in one call (%lld)", (long long)a.npts);
  *grid = dim3((unsigned)(blocks > 0 ? blocks : 1));
  return 0;
}

// Untuned defaults for vgh are the autotuner's choices on GB300 at 64^3 x
// 1024 and 128^3 x 2048 (and 48^3 x 512 double-float): the shared-memory
// copy pipeline, 8-column wide for 16-bit tables; value-only evaluation uses
// the wide pipeline for 16-bit tables and direct loads otherwise; IEEE FP64
// (FMA-bound) always uses direct loads.
int pick_mode(Table *t, bool vgh, bool sorted) {
  if (t->tile_mode >= 0) return t->tile_mode;
  const int v = vgh ? 1 : 0;
  if (sorted && t->tuned_s_tx[v]) return t->tuned_s_mode[v];
  if (t->tuned_tx[v]) return t->tuned_mode[v];
  // F16 and BF16 vgh: the tensor-core reduction (64^3 x 1024, 64 walkers:
  // F16 45.7 G evals/s random and 66.3 G cell-sorted against 43.0 G and
  // 44.6 G for the wide copy pipeline; BF16 45.5 G and 64.4 G against 42.9 G
  // and 46.1 G); value only stays on the wide pipeline (58.4 G random and
  // 90.9 G sorted against 57.8 G and 74.0 G for F16)
  if (vgh && (t->storage == ST_F16 || t->storage == ST_BF16)) return 5;
  if (vgh && kernel_storage(t) != ST_F64) return is16(t->storage) ? 3 : 2;
  // value only: the wide pipeline for 16-bit tables (0.294 against 0.413 ms
  // with direct loads at 64^3 x 1024, 17k points); FP32 is as fast direct
  if (is16(t->storage)) return 3;
  return 0;
}

void pick_tile(Table *t, bool vgh, int64_t npts, int &tx, int &ty, int &pb, bool sorted) {
  if (t->tile_tx) { tx = t->tile_tx; ty = t->tile_ty; pb = t->tile_pb; return; }
  const int v = vgh ? 1 : 0;
  if (sorted && t->tuned_s_tx[v]) { tx = t->tuned_s_tx[v]; ty = t->tuned_s_ty[v]; pb = t->tuned_s_pb[v]; return; }
  if (t->tuned_tx[v]) { tx = t->tuned_tx[v]; ty = t->tuned_ty[v]; pb = t->tuned_pb[v]; return; }
  if ((t->storage == ST_F16 || t->storage == ST_BF16) && ((vgh && t->tile_mode < 0) || t->tile_mode == 5)) {
    // tensor cores: 10 points a block keep three blocks on an SM (74.7 KB of
    // shared memory each); the block's threads are fixed by the kernel
    tx = 128;
    ty = 1;
    pb = 10;
    return;
  }
  const int VW = elems_per_thread(t);
  const int need = (t->ncol + VW - 1) / VW;
  tx = (need + 31) / 32 * 32;
  if ((vgh || is16(t->storage)) && kernel_storage(t) != ST_F64 && t->tile_mode < 0) {
    // pipelined defaults (pick_mode): one lane of points, 8 points a block
    const int cap = is16(t->storage) ? 32 : (kernel_storage(t) == ST_DF ? 128 : 64);
    tx = tx > cap ? cap : tx;
    ty = 1;
    pb = 8;
    return;
  }
  if (tx > 256) tx = 256;
  ty = 256 / tx;
  if (ty > 8) ty = 8;
  pb = 2 * ty;
  (void)npts;
}

int wait_status(Table *t, const char *fn) {
  if (t->wait_err_h && *(volatile int *)t->wait_err_h) {
    *(volatile int *)t->wait_err_h = 0;
    return fail(EINSPLINE_GB300_ETIMEOUT, "%s: a TMA-staged evaluation gave up a bounded wait; its results are incomplete",
                fn);
  }
  return 0;
}

// Output scratch of the single-point entries: 40 output reals per column
// (value, 3 gradient, 9 Hessian, 27 third-derivative) in pinned host memory
// mapped into the device's address space.  The kernels write their outputs
// there directly, so a call needs no device-to-host copy: after the stream
// synchronises the host reads them in place.
int point_scratch(Table *t, const char *fn) {
  if (t->pt_host) return 0;
  const size_t sz = 40 * (size_t)t->ncol * acc_bytes(t);
  void *h = nullptr, *d = nullptr;
  if (cudaHostAlloc(&h, sz, cudaHostAllocMapped) != cudaSuccess || cudaHostGetDevicePointer(&d, h, 0) != cudaSuccess) {
    cudaGetLastError();
    if (h) cudaFreeHost(h);
    return fail(EINSPLINE_GB300_ENOMEM, "%s: scratch allocation failed", fn);
  }
  t->pt_host = h;
  t->pt_dev = d;
  return 0;
}

// Launch shape of a single-point evaluation: one warp per block and as many
// blocks as the columns need, so a wide table's point is spread over many
// SMs; the stencil rows of the point are first asked of L2 with bulk
// prefetches (load mode 1), all 64 at once, unless the table forces a mode.
int launch_point(Table *t, EvalArgs &a, bool vgh) {
  const int mode = t->tile_mode >= 0 ? t->tile_mode : 1;
  return launch_eval(t, a, vgh, t->stream, 32, 1, 1, mode);
}

}  // namespace eg

using namespace eg;

namespace {

template <typename S>
Table *host_table(S *s, const char *fn) {
  if (!s || !table3_ok(s->gb300)) {
    fail(EINSPLINE_GB300_EINVAL, "%s: not a spline made by this library", fn);
    return nullptr;
  }
  return s->gb300;
}


// Single point, host outputs in the CPU layout.  out: 0 vgh, 2 vgl, 3 vg.
template <typename S, typename V>
void eval_point(S *s, double x, double y, double z, V *vals, V *grads, V *hess, bool vgh, const char *fn,
                int out = 0) {
  clear();
  Table *t = host_table(s, fn);
  if (!t) return;
  if (table_flush(t)) return;
  std::lock_guard<std::mutex> g(t->mu);
  const size_t rb = acc_bytes(t);
  const size_t n = (size_t)t->ncol;
  if (point_scratch(t, fn)) return;
  EvalArgs a;
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(t, a);
  a.pos = nullptr;
  a.inl[0] = x; a.inl[1] = y; a.inl[2] = z;
  a.rule = 0;
  a.layout = 1;
  a.out = out;
  a.npts = 1;
  a.vals = t->pt_dev;
  a.grads = (char *)t->pt_dev + n * rb;
  a.hess = (char *)t->pt_dev + 4 * n * rb;
  if (launch_point(t, a, vgh)) return;
  if (cudaError_t e = cudaStreamSynchronize(t->stream)) {
    cuda_check(e, fn);
    return;
  }
  if (wait_status(t, fn)) return;
  memcpy(vals, t->pt_host, n * rb);
  if (vgh) {
    memcpy(grads, (char *)t->pt_host + n * rb, 3 * n * rb);
    if (out == 0) memcpy(hess, (char *)t->pt_host + 4 * n * rb, 9 * n * rb);
    if (out == 2) memcpy(hess, (char *)t->pt_host + 4 * n * rb, n * rb);
  }
}

// Single point value/gradient/Hessian/third derivatives, CPU layout.
template <typename S, typename V>
void eval_point_vghgh(S *s, double x, double y, double z, V *vals, V *grads, V *hess, V *gradhess, const char *fn) {
  clear();
  Table *t = host_table(s, fn);
  if (!t) return;
  if (!vals || !grads || !hess || !gradhess) { fail(EINSPLINE_GB300_EINVAL, "%s: NULL output", fn); return; }
  if (table_flush(t)) return;
  std::lock_guard<std::mutex> g(t->mu);
  const size_t rb = acc_bytes(t);
  const size_t n = (size_t)t->ncol;
  if (point_scratch(t, fn)) return;
  EvalArgs a;
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(t, a);
  a.inl[0] = x; a.inl[1] = y; a.inl[2] = z;
  a.rule = 0;
  a.layout = 1;
  a.npts = 1;
  a.vals = t->pt_dev;
  a.grads = (char *)t->pt_dev + n * rb;
  a.hess = (char *)t->pt_dev + 4 * n * rb;
  a.ghess = (char *)t->pt_dev + 13 * n * rb;
  if (launch_vghgh(t, a, t->stream)) return;
  if (cudaError_t e = cudaStreamSynchronize(t->stream)) {
    cuda_check(e, fn);
    return;
  }
  memcpy(vals, t->pt_host, n * rb);
  memcpy(grads, (char *)t->pt_host + n * rb, 3 * n * rb);
  memcpy(hess, (char *)t->pt_host + 4 * n * rb, 9 * n * rb);
  memcpy(gradhess, (char *)t->pt_host + 13 * n * rb, 27 * n * rb);
}

// Batched, reference GPU-entry semantics and layout, pointer-array outputs.
// out 1 (vgl): grads_d holds the grad_lapl pointers, linv/lrow the transform.
template <typename CS>
void eval_cuda(CS *c, const void *pos_d, bool pos_f64, void *const *vals_d, void *const *grads_d,
               void *const *hess_d, int num, bool vgh, const char *fn, int out = 0, const void *sign = nullptr,
               const void *linv = nullptr, int64_t lrow = 0) {
  clear();
  if (!c || !table3_ok(c->gb300)) { fail(EINSPLINE_GB300_EINVAL, "%s: not a handle made by this library", fn); return; }
  if (num <= 0) return;
  Table *t = c->gb300;
  EvalArgs a;
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(t, a);
  a.pos = pos_d;
  a.pos_f64 = pos_f64;
  a.rule = 1;
  a.layout = 0;
  a.npts = num;
  a.vals_pp = vals_d; a.grads_pp = grads_d; a.hess_pp = hess_d;
  a.out = out;
  a.sign = sign;
  a.linv = linv;
  a.lrow = lrow;
  if (out == 1 && (!linv || !grads_d)) { fail(EINSPLINE_GB300_EINVAL, "%s: Linv and grad_lapl are required", fn); return; }
  int tx, ty, pb;
  pick_tile(t, vgh, num, tx, ty, pb);
  if (launch_eval(t, a, vgh, cudaStreamLegacy, tx, ty, pb)) return;
  cudaError_t e = cudaStreamSynchronize(cudaStreamLegacy);
  if (e != cudaSuccess) cuda_check(e, fn);
}

}  // namespace

extern "C" {

void eval_multi_UBspline_3d_s(multi_UBspline_3d_s *s, double x, double y, double z, float *vals) {
  eval_point<multi_UBspline_3d_s, float>(s, x, y, z, vals, nullptr, nullptr, false, "eval_multi_UBspline_3d_s");
}
void eval_multi_UBspline_3d_s_vgh(multi_UBspline_3d_s *s, double x, double y, double z, float *vals, float *grads,
                                  float *hess) {
  eval_point<multi_UBspline_3d_s, float>(s, x, y, z, vals, grads, hess, true, "eval_multi_UBspline_3d_s_vgh");
}
void eval_multi_UBspline_3d_d(multi_UBspline_3d_d *s, double x, double y, double z, double *vals) {
  eval_point<multi_UBspline_3d_d, double>(s, x, y, z, vals, nullptr, nullptr, false, "eval_multi_UBspline_3d_d");
}
void eval_multi_UBspline_3d_d_vgh(multi_UBspline_3d_d *s, double x, double y, double z, double *vals, double *grads,
                                  double *hess) {
  eval_point<multi_UBspline_3d_d, double>(s, x, y, z, vals, grads, hess, true, "eval_multi_UBspline_3d_d_vgh");
}
void eval_multi_UBspline_3d_c(multi_UBspline_3d_c *s, double x, double y, double z, complex_float *vals) {
  eval_point<multi_UBspline_3d_c, complex_float>(s, x, y, z, vals, nullptr, nullptr, false,
                                                 "eval_multi_UBspline_3d_c");
}
void eval_multi_UBspline_3d_c_vgh(multi_UBspline_3d_c *s, double x, double y, double z, complex_float *vals,
                                  complex_float *grads, complex_float *hess) {
  eval_point<multi_UBspline_3d_c, complex_float>(s, x, y, z, vals, grads, hess, true,
                                                 "eval_multi_UBspline_3d_c_vgh");
}
void eval_multi_UBspline_3d_z(multi_UBspline_3d_z *s, double x, double y, double z, complex_double *vals) {
  eval_point<multi_UBspline_3d_z, complex_double>(s, x, y, z, vals, nullptr, nullptr, false,
                                                  "eval_multi_UBspline_3d_z");
}
void eval_multi_UBspline_3d_z_vgh(multi_UBspline_3d_z *s, double x, double y, double z, complex_double *vals,
                                  complex_double *grads, complex_double *hess) {
  eval_point<multi_UBspline_3d_z, complex_double>(s, x, y, z, vals, grads, hess, true,
                                                  "eval_multi_UBspline_3d_z_vgh");
}

// Third derivatives: src/multi_bspline_eval_std_s_impl.h:866,
// src/multi_bspline_eval_std_d_impl.h:868, src/multi_bspline_eval_std_c_impl.h:864,
// src/multi_bspline_eval_std_z_impl.h:868.
void eval_multi_UBspline_3d_s_vghgh(multi_UBspline_3d_s *s, double x, double y, double z, float *vals, float *grads,
                                    float *hess, float *gradhess) {
  eval_point_vghgh(s, x, y, z, vals, grads, hess, gradhess, "eval_multi_UBspline_3d_s_vghgh");
}
void eval_multi_UBspline_3d_d_vghgh(multi_UBspline_3d_d *s, double x, double y, double z, double *vals,
                                    double *grads, double *hess, double *gradhess) {
  eval_point_vghgh(s, x, y, z, vals, grads, hess, gradhess, "eval_multi_UBspline_3d_d_vghgh");
}
void eval_multi_UBspline_3d_c_vghgh(multi_UBspline_3d_c *s, double x, double y, double z, complex_float *vals,
                                    complex_float *grads, complex_float *hess, complex_float *gradhess) {
  eval_point_vghgh(s, x, y, z, vals, grads, hess, gradhess, "eval_multi_UBspline_3d_c_vghgh");
}
void eval_multi_UBspline_3d_z_vghgh(multi_UBspline_3d_z *s, double x, double y, double z, complex_double *vals,
                                    complex_double *grads, complex_double *hess, complex_double *gradhess) {
  eval_point_vghgh(s, x, y, z, vals, grads, hess, gradhess, "eval_multi_UBspline_3d_z_vghgh");
}

void eval_multi_UBspline_3d_s_vg(multi_UBspline_3d_s *s, double x, double y, double z, float *vals, float *grads) {
  eval_point<multi_UBspline_3d_s, float>(s, x, y, z, vals, grads, nullptr, true, "eval_multi_UBspline_3d_s_vg", 3);
}
void eval_multi_UBspline_3d_s_vgl(multi_UBspline_3d_s *s, double x, double y, double z, float *vals, float *grads,
                                  float *lapl) {
  eval_point<multi_UBspline_3d_s, float>(s, x, y, z, vals, grads, lapl, true, "eval_multi_UBspline_3d_s_vgl", 2);
}
void eval_multi_UBspline_3d_d_vg(multi_UBspline_3d_d *s, double x, double y, double z, double *vals, double *grads) {
  eval_point<multi_UBspline_3d_d, double>(s, x, y, z, vals, grads, nullptr, true, "eval_multi_UBspline_3d_d_vg", 3);
}
void eval_multi_UBspline_3d_d_vgl(multi_UBspline_3d_d *s, double x, double y, double z, double *vals, double *grads,
                                  double *lapl) {
  eval_point<multi_UBspline_3d_d, double>(s, x, y, z, vals, grads, lapl, true, "eval_multi_UBspline_3d_d_vgl", 2);
}
void eval_multi_UBspline_3d_c_vg(multi_UBspline_3d_c *s, double x, double y, double z, complex_float *vals,
                                 complex_float *grads) {
  eval_point<multi_UBspline_3d_c, complex_float>(s, x, y, z, vals, grads, nullptr, true,
                                                 "eval_multi_UBspline_3d_c_vg", 3);
}
void eval_multi_UBspline_3d_c_vgl(multi_UBspline_3d_c *s, double x, double y, double z, complex_float *vals,
                                  complex_float *grads, complex_float *lapl) {
  eval_point<multi_UBspline_3d_c, complex_float>(s, x, y, z, vals, grads, lapl, true,
                                                 "eval_multi_UBspline_3d_c_vgl", 2);
}
void eval_multi_UBspline_3d_z_vg(multi_UBspline_3d_z *s, double x, double y, double z, complex_double *vals,
                                 complex_double *grads) {
  eval_point<multi_UBspline_3d_z, complex_double>(s, x, y, z, vals, grads, nullptr, true,
                                                  "eval_multi_UBspline_3d_z_vg", 3);
}
void eval_multi_UBspline_3d_z_vgl(multi_UBspline_3d_z *s, double x, double y, double z, complex_double *vals,
                                  complex_double *grads, complex_double *lapl) {
  eval_point<multi_UBspline_3d_z, complex_double>(s, x, y, z, vals, grads, lapl, true,
                                                  "eval_multi_UBspline_3d_z_vgl", 2);
}

void eval_multi_multi_UBspline_3d_s_sign_cuda(multi_UBspline_3d_s_cuda *c, float *pos_d, float *sign_d,
                                              float *vals_d[], int num) {
  if (!sign_d) { clear(); fail(EINSPLINE_GB300_EINVAL, "eval_multi_multi_UBspline_3d_s_sign_cuda: sign_d is NULL"); return; }
  eval_cuda(c, pos_d, false, (void *const *)vals_d, nullptr, nullptr, num, false,
            "eval_multi_multi_UBspline_3d_s_sign_cuda", 0, sign_d);
}
void eval_multi_multi_UBspline_3d_s_vgl_cuda(multi_UBspline_3d_s_cuda *c, float *pos_d, float *Linv_d,
                                             float *vals_d[], float *grad_lapl_d[], int num, int row_stride) {
  eval_cuda(c, pos_d, false, (void *const *)vals_d, (void *const *)grad_lapl_d, nullptr, num, true,
            "eval_multi_multi_UBspline_3d_s_vgl_cuda", 1, nullptr, Linv_d, row_stride);
}
void eval_multi_multi_UBspline_3d_s_vgl_sign_cuda(multi_UBspline_3d_s_cuda *c, float *pos_d, float *sign_d,
                                                  float *Linv_d, float *vals_d[], float *grad_lapl_d[], int num,
                                                  int row_stride) {
  if (!sign_d) { clear(); fail(EINSPLINE_GB300_EINVAL, "eval_multi_multi_UBspline_3d_s_vgl_sign_cuda: sign_d is NULL"); return; }
  eval_cuda(c, pos_d, false, (void *const *)vals_d, (void *const *)grad_lapl_d, nullptr, num, true,
            "eval_multi_multi_UBspline_3d_s_vgl_sign_cuda", 1, sign_d, Linv_d, row_stride);
}
void eval_multi_multi_UBspline_3d_d_vgl_cuda(multi_UBspline_3d_d_cuda *c, double *pos_d, double *Linv_d,
                                             double *vals_d[], double *grad_lapl_d[], int num, int row_stride) {
  eval_cuda(c, pos_d, true, (void *const *)vals_d, (void *const *)grad_lapl_d, nullptr, num, true,
            "eval_multi_multi_UBspline_3d_d_vgl_cuda", 1, nullptr, Linv_d, row_stride);
}
// Complex rows are row_stride complex values apart: 2 * row_stride reals
// (src/multi_bspline_cuda_c_impl.h:612-622).
void eval_multi_multi_UBspline_3d_c_vgl_cuda(multi_UBspline_3d_c_cuda *c, float *pos_d, float *Linv_d,
                                             complex_float *vals_d[], complex_float *grad_lapl_d[], int num,
                                             int row_stride) {
  eval_cuda(c, pos_d, false, (void *const *)vals_d, (void *const *)grad_lapl_d, nullptr, num, true,
            "eval_multi_multi_UBspline_3d_c_vgl_cuda", 1, nullptr, Linv_d, 2 * (int64_t)row_stride);
}
void eval_multi_multi_UBspline_3d_z_vgl_cuda(multi_UBspline_3d_z_cuda *c, double *pos_d, double *Linv_d,
                                             complex_double *vals_d[], complex_double *grad_lapl_d[], int num,
                                             int row_stride) {
  eval_cuda(c, pos_d, true, (void *const *)vals_d, (void *const *)grad_lapl_d, nullptr, num, true,
            "eval_multi_multi_UBspline_3d_z_vgl_cuda", 1, nullptr, Linv_d, 2 * (int64_t)row_stride);
}

void eval_multi_multi_UBspline_3d_s_cuda(multi_UBspline_3d_s_cuda *c, float *pos_d, float *vals_d[], int num) {
  eval_cuda(c, pos_d, false, (void *const *)vals_d, nullptr, nullptr, num, false, "eval_multi_multi_UBspline_3d_s_cuda");
}
void eval_multi_multi_UBspline_3d_s_vgh_cuda(multi_UBspline_3d_s_cuda *c, float *pos_d, float *vals_d[],
                                             float *grads_d[], float *hess_d[], int num) {
  eval_cuda(c, pos_d, false, (void *const *)vals_d, (void *const *)grads_d, (void *const *)hess_d, num, true,
            "eval_multi_multi_UBspline_3d_s_vgh_cuda");
}
void eval_multi_multi_UBspline_3d_d_cuda(multi_UBspline_3d_d_cuda *c, double *pos_d, double *vals_d[], int num) {
  eval_cuda(c, pos_d, true, (void *const *)vals_d, nullptr, nullptr, num, false, "eval_multi_multi_UBspline_3d_d_cuda");
}
void eval_multi_multi_UBspline_3d_d_vgh_cuda(multi_UBspline_3d_d_cuda *c, double *pos_d, double *vals_d[],
                                             double *grads_d[], double *hess_d[], int num) {
  eval_cuda(c, pos_d, true, (void *const *)vals_d, (void *const *)grads_d, (void *const *)hess_d, num, true,
            "eval_multi_multi_UBspline_3d_d_vgh_cuda");
}
void eval_multi_multi_UBspline_3d_c_cuda(multi_UBspline_3d_c_cuda *c, float *pos_d, complex_float *vals_d[], int num) {
  eval_cuda(c, pos_d, false, (void *const *)vals_d, nullptr, nullptr, num, false, "eval_multi_multi_UBspline_3d_c_cuda");
}
void eval_multi_multi_UBspline_3d_c_vgh_cuda(multi_UBspline_3d_c_cuda *c, float *pos_d, complex_float *vals_d[],
                                             complex_float *grads_d[], complex_float *hess_d[], int num) {
  eval_cuda(c, pos_d, false, (void *const *)vals_d, (void *const *)grads_d, (void *const *)hess_d, num, true,
            "eval_multi_multi_UBspline_3d_c_vgh_cuda");
}
void eval_multi_multi_UBspline_3d_z_cuda(multi_UBspline_3d_z_cuda *c, double *pos_d, complex_double *vals_d[],
                                         int num) {
  eval_cuda(c, pos_d, true, (void *const *)vals_d, nullptr, nullptr, num, false, "eval_multi_multi_UBspline_3d_z_cuda");
}
void eval_multi_multi_UBspline_3d_z_vgh_cuda(multi_UBspline_3d_z_cuda *c, double *pos_d, complex_double *vals_d[],
                                             complex_double *grads_d[], complex_double *hess_d[], int num) {
  eval_cuda(c, pos_d, true, (void *const *)vals_d, (void *const *)grads_d, (void *const *)hess_d, num, true,
            "eval_multi_multi_UBspline_3d_z_vgh_cuda");
}

}  // extern "C"
