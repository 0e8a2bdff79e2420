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
// are deterministic.  k_det_tc does the same for F16 and BF16 tables on the
// tensor cores (their default load mode 5).
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

// ------------------------------------------------------------ tensor cores
// k_det_tc: the ratio of F16 and BF16 tables in their default load mode 5,
// with the evaluation kernel's tensor-core contraction (k_eval_tc, eval.cu):
// per walker and tile of 128 orbitals, D[128 orbitals x NC] = A[128 x 64] *
// B[64 x NC] in four tcgen05.mma (K = 16, one per x-plane), A the stencil as
// a TMA box copies it (128-byte swizzle), B the walker's weights of seven
// outputs (value, gradient, the Hessian's diagonal) split into the table
// type's parts, each part in its own column.  Instead of storing the
// outputs, the epilogue dots them with the inverse column.
//
// A block takes pb walkers and all N orbitals: unit u = p * TT + t is tile
// t of walker p.  Warp 0 (one lane) keeps kDtStages stencil copies in
// flight, one unit a stage; warp 1 (one lane) issues a unit's MMAs into
// one of the block's accumulator slots (unit u into slot u modulo their
// number) once its stencil, the walker's weights and the slot are there,
// and commits the unit to the barriers that free its
// stage and fill its slot; warps 2-5 (one orbital of each tile a thread)
// read a slot, free it, add the weight parts, scale, and accumulate the
// products with the thread's inverse entries; at a walker's last tile (its
// MMAs then all complete) they build the weights of the walker two ahead in
// its buffer and fold their five sums with a fixed shuffle tree into shared
// memory, which one thread per walker adds up in order after the loop, so
// the results are deterministic.  The value row, on request, equals the
// flat evaluation's mode-5 values bit for bit.  Every wait is bounded, as
// in k_eval_tc.
//
// Two stencil stages and five blocks an SM: more walkers in flight than four
// stages and three blocks (2,048 walkers: 0.047 against 0.052 ms; 16,384:
// 0.285 against 0.298 ms).
constexpr int kDtStages = 2, kDtSlots = 4, kDtMaxWalkers = 7, kDtBlocksPerSM = 5;
__host__ __device__ __forceinline__ size_t dt_ptr_off(int pb) { return align_up(smem_total(pb, 4), 16); }
__host__ __device__ __forceinline__ size_t dt_red_off(int pb) { return dt_ptr_off(pb) + (size_t)pb * 8; }
__host__ __device__ __forceinline__ size_t dt_head(int pb) { return dt_red_off(pb) + (size_t)pb * 4 * 5 * 4; }
// the head, slack to align the operand area to 1024 bytes, the stages, two
// weight buffers, the mbarriers and the TMEM address / abort flag / count;
// at kDtMaxWalkers walkers kDtBlocksPerSM blocks share an SM
__host__ __device__ __forceinline__ size_t dt_smem(int pb) {
  return dt_head(pb) + 1024 + (size_t)kDtStages * 16384 + 2 * 4096 + 8 * (2 * kDtStages + 2 + 2 * kDtSlots) + 16;
}

template <int ST, bool GL>
__global__ void __launch_bounds__(kTcThreads, kDtBlocksPerSM) k_det_tc(const __grid_constant__ DetArgs d) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int NS = kDtStages, NP = TcCfg<ST>::parts, NQ = GL ? 7 : 1;
  constexpr int NC = NQ * NP <= 16 ? 16 : 32;  // accumulator columns a unit (the MMA's N)
  // accumulator slots: 64 TMEM columns a block, so five blocks hold 320 of 512
  constexpr int RA = NC == 16 ? kDtSlots : kDtSlots / 2;
  constexpr unsigned kB = 4096u, kStage = 16384u;
  constexpr int NW = 4;  // output warps
  const EvalArgs &a = d.e;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int64_t p0 = (int64_t)blockIdx.x * a.pb;
  const int pn = (int)min((int64_t)a.pb, a.npts - p0);
  const int TT = (d.n + 127) >> 7;
  float *sw = reinterpret_cast<float *>(smem);
  int *sidx = reinterpret_cast<int *>(smem + smem_w_bytes(a.pb, 4));
  int64_t *ssrc = reinterpret_cast<int64_t *>(smem + smem_w_bytes(a.pb, 4) + align_up((size_t)a.pb * 12, 8));
  const float **sptr = reinterpret_cast<const float **>(smem + dt_ptr_off(a.pb));
  float *red = reinterpret_cast<float *>(smem + dt_red_off(a.pb));
  // cells and the unscaled basis weights (delta_inv applied in the epilogue)
  for (int q = tid; q < pn * 3; q += kTcThreads) {
    const int pp = q / 3, ax = q - 3 * pp;
    const int64_t src = p0 + pp;
    const double xd = a.pos_f64 ? reinterpret_cast<const double *>(a.pos)[3 * src + ax]
                                : (double)reinterpret_cast<const float *>(a.pos)[3 * src + ax];
    int idx;
    float t;
    cell(a, ax, xd, idx, t);
    bspline_weights<float>(t, sw + pp * 36 + ax * 12, 1.0f);
    sidx[pp * 3 + ax] = idx;
    if (ax == 0) ssrc[pp] = src;
  }
  for (int q = tid; q < pn; q += kTcThreads) sptr[q] = d.ainv[p0 + q];
  const unsigned base_s = (unsigned)__cvta_generic_to_shared(smem);
  const unsigned a_s = (base_s + (unsigned)dt_head(a.pb) + 1023u) & ~1023u;
  const unsigned b_s = a_s + NS * kStage;
  const unsigned full_s = b_s + 2 * kB, empty_s = full_s + 8 * NS, bfull_s = empty_s + 8 * NS;
  const unsigned tfull_s = bfull_s + 16, tempty_s = tfull_s + 8 * RA, slot_s = tempty_s + 8 * RA;
  unsigned char *bgen = smem + (b_s - base_s);
  volatile int *abort_flag = reinterpret_cast<volatile int *>(smem + (slot_s + 4 - base_s));
  volatile int *consumed = reinterpret_cast<volatile int *>(smem + (slot_s + 8 - base_s));
  // weight columns past the outputs' parts stay zero
  for (int e = tid; e < 2 * (int)kB / 16; e += kTcThreads) reinterpret_cast<uint4 *>(bgen)[e] = make_uint4(0, 0, 0, 0);
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_s), "n"(RA * NC)
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
    for (int b = 0; b < 2; b++) mbar_init(bfull_s + 8 * b, 128);
#pragma unroll
    for (int r = 0; r < RA; r++) {
      mbar_init(tfull_s + 8 * r, 1);
      mbar_init(tempty_s + 8 * r, 128);
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
  const unsigned long long lim = a.wait_ns ? a.wait_ns : kWaitNs;
  auto wait = [&](unsigned bar, unsigned parity) -> bool {
    if (*abort_flag) return false;
    if (mbar_wait(bar, parity, lim)) return true;
    *abort_flag = 1;
    return false;
  };
  const int U = pn * TT;
  int issued = 0, skipped = -1, last_commit = -1;
  if (warp == 0) {
    if (lane == 0) {
      tma_prefetch_map(&a.tmap);
      for (int u = 0; u < U; u++) {
        const int s = u % NS, p = u / TT, t = u - p * TT;
        if (u >= NS && !wait(empty_s + 8 * s, (unsigned)((u / NS - 1) & 1))) break;
        issued = u + 1;
        // test hook: no copy for this walker, so its wait runs out
        if (a.test_skip == p + 1 && blockIdx.x == 0) { skipped = p; continue; }
        mbar_arrive_expect_tx(full_s + 8 * s, kStage);
#pragma unroll
        for (int mg = 0; mg < 2; mg++)
          tma_load_4d(a_s + s * kStage + mg * 8192u, &a.tmap, full_s + 8 * s, 128 * t + 64 * mg, sidx[3 * p + 2],
                      sidx[3 * p + 1], sidx[3 * p]);
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = umma_idesc_16(128, NC, TcCfg<ST>::fmt);
      bool go = true;
      for (int p = 0; p < pn && go; p++) {
        const int bb = p & 1;
        if (!wait(bfull_s + 8 * bb, (unsigned)((p >> 1) & 1))) break;
        for (int t = 0; t < TT; t++) {
          const int u = p * TT + t, s = u % NS, r = u % RA;
          if (u >= RA && !wait(tempty_s + 8 * r, (unsigned)((u / RA - 1) & 1))) { go = false; break; }
          if (!wait(full_s + 8 * s, (unsigned)((u / NS) & 1))) { go = false; break; }
          *consumed = u + 1;
          tc_fence_after();
#pragma unroll
          for (int i = 0; i < 4; i++)
            umma_f16(tmem + r * NC, umma_desc(a_s + s * kStage + i * 2048u, 8192u, 1024u, 2),
                     umma_desc(b_s + bb * kB + i * 1024u, 128u, 256u, 0), idesc, i > 0);
          umma_commit(empty_s + 8 * s);
          umma_commit(tfull_s + 8 * r);
          last_commit = u;
        }
      }
    }
  } else {
    const int et = tid - 64;
    const int colr = (warp & 3) * 32 + lane;  // this thread's orbital (TMEM lane) in every tile
    // this thread's share of a weight matrix: stencil row k, outputs 0-3
    // (even threads) or 4-6 (odd threads)
    const int k = et >> 1;
    const int ki = k >> 4, kj = (k >> 2) & 3, km = k & 3, kk = k & 15;
    const unsigned boff = ki * 1024 + (kk >> 3) * 128 + (kk & 7) * 2;
    // derivative orders in x, y, z of each output (v, gx, gy, gz, hxx, hyy, hzz)
    static constexpr int OA[7] = {0, 1, 0, 0, 2, 0, 0};
    static constexpr int OB[7] = {0, 0, 1, 0, 0, 2, 0};
    static constexpr int OC[7] = {0, 0, 0, 1, 0, 0, 2};
    auto build_b = [&](int p) {
      const float *w = sw + p * 36;
      unsigned char *bm = bgen + (p & 1) * kB + boff;
      float wx[3], wy[3], wz[3];
#pragma unroll
      for (int dd = 0; dd < 3; dd++) {
        wx[dd] = w[4 * dd + ki];
        wy[dd] = w[12 + 4 * dd + kj];
        wz[dd] = w[24 + 4 * dd + km];
      }
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
        if constexpr (GL) {
          put(std::integral_constant<int, 1>());
          put(std::integral_constant<int, 2>());
          put(std::integral_constant<int, 3>());
        }
      } else if constexpr (GL) {
        put(std::integral_constant<int, 4>());
        put(std::integral_constant<int, 5>());
        put(std::integral_constant<int, 6>());
      }
      fence_proxy_async();
      mbar_arrive(bfull_s + 8 * (p & 1));
    };
    const float dx = a.dinvf[0], dy = a.dinvf[1], dz = a.dinvf[2];
    float acc[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
    build_b(0);
    if (pn > 1) build_b(1);
    // the inverse entry and the spline's factor of unit u, loaded during
    // unit u - 1 (the reference layout's entries are scattered 4-byte reads)
    auto load_av = [&](int u, float &av, float &sc) {
      const int p = u / TT, col = (u - p * TT) * 128 + colr;
      av = 0.f;
      sc = 1.f;
      if (u < U && col < d.n) {
        av = d.trans ? sptr[p][(int64_t)d.k * d.ld + col] : sptr[p][(int64_t)col * d.ld + d.k];
        if (a.scale) sc = a.scale[col];
      }
    };
    float av_n, sc_n;
    load_av(0, av_n, sc_n);
    for (int u = 0; u < U; u++) {
      const int p = u / TT, t = u - p * TT, r = u % RA;
      const int col = t * 128 + colr;
      const bool live = col < d.n;
      const float av = av_n, sc = sc_n;
      load_av(u + 1, av_n, sc_n);
      if (!wait(tfull_s + 8 * r, (unsigned)((u / RA) & 1))) break;
      // walker p's MMAs are all complete after its last tile: its weight
      // buffer takes walker p + 2's weights
      if (t == TT - 1 && p + 2 < pn) build_b(p + 2);
      tc_fence_after();
      uint32_t rr[32];
      if constexpr (NC == 16) tmem_ld16(tmem + ((unsigned)((warp & 3) * 32) << 16) + r * NC, rr);
      else tmem_ld32(tmem + ((unsigned)((warp & 3) * 32) << 16) + r * NC, rr);
      tc_fence_before();
      mbar_arrive(tempty_s + 8 * r);
      float o[NQ];
#pragma unroll
      for (int q = 0; q < NQ; q++) {
        float v = __uint_as_float(rr[NP * q]);
#pragma unroll
        for (int h = 1; h < NP; h++) v += __uint_as_float(rr[NP * q + h]);
        o[q] = v;
      }
      if (live) {
        const float v = o[0] * (sc * 1.f);  // as the flat kernel's value: (sum of parts) x (factor x 1)
        acc[0] = fmaf(v, av, acc[0]);
        if constexpr (GL) {
          acc[1] = fmaf(o[1] * (sc * dx), av, acc[1]);
          acc[2] = fmaf(o[2] * (sc * dy), av, acc[2]);
          acc[3] = fmaf(o[3] * (sc * dz), av, acc[3]);
          const float lap = (o[4] * (sc * (dx * dx)) + o[5] * (sc * (dy * dy))) + o[6] * (sc * (dz * dz));
          acc[4] = fmaf(lap, av, acc[4]);
        }
        if (d.row_out) d.row_out[ssrc[p]][col] = v;
      }
      if (t == TT - 1) {
#pragma unroll
        for (int q = 0; q < 5; q++) {
#pragma unroll
          for (int off = 16; off > 0; off >>= 1) acc[q] += __shfl_xor_sync(0xffffffffu, acc[q], off);
          if (lane == 0) red[(p * NW + (warp - 2)) * 5 + q] = acc[q];
          acc[q] = 0.f;
        }
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
        if (u / TT != skipped) mbar_wait(full_s + 8 * (u % NS), (unsigned)((u / NS) & 1), lim);
    }
    if (tid == 32 && last_commit >= 0) {
      const int u = *consumed - 1;
      mbar_wait(empty_s + 8 * (u % NS), (unsigned)((u / NS) & 1), lim);
    }
  } else if (tid < pn) {
    const int pp = tid;
    float s[5];
#pragma unroll
    for (int q = 0; q < 5; q++) {
      s[q] = red[pp * NW * 5 + q];
#pragma unroll
      for (int w = 1; w < NW; w++) s[q] += red[(pp * NW + w) * 5 + q];
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
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "n"(RA * NC) : "memory");
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

template <int ST, bool GL>
cudaError_t launch_det_tc_k(const DetArgs &d, unsigned grid, cudaStream_t s) {
  const size_t sm = dt_smem(d.e.pb);
  const void *f = (const void *)k_det_tc<ST, GL>;
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k_det_tc<ST, GL><<<grid, kTcThreads, sm, s>>>(d);
  return cudaGetLastError();
}

template <int ST>
cudaError_t launch_det_tc(const DetArgs &d, bool gl, unsigned grid, cudaStream_t s) {
  return gl ? launch_det_tc_k<ST, true>(d, grid, s) : launch_det_tc_k<ST, false>(d, grid, s);
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
  if ((t->storage == ST_F16 || t->storage == ST_BF16) && pick_mode(t, true) == 5) {
    // tensor cores, as the table's vgh evaluation: kDtBlocksPerSM blocks of at most
    // kDtMaxWalkers walkers an SM, the walkers spread evenly over whole waves
    if (int r = tc_table_map(t, d.e)) return r;
    d.e.wait_err = t->wait_err_d;
    if (t->test_skip.load(std::memory_order_relaxed)) {
      d.e.test_skip = t->test_skip.exchange(0);
      d.e.wait_ns = t->test_wait_ns;
    }
    const int64_t slots = kDtBlocksPerSM * (int64_t)num_sms();
    const int64_t waves = (nwalkers + slots * kDtMaxWalkers - 1) / (slots * kDtMaxWalkers);
    const int pb = (int)((nwalkers + slots * waves - 1) / (slots * waves));
    d.e.pb = pb;
    const unsigned grid = (unsigned)((nwalkers + pb - 1) / pb);
    EG_CUDA(t->storage == ST_F16 ? launch_det_tc<ST_F16>(d, gl, grid, s) : launch_det_tc<ST_BF16>(d, gl, grid, s));
    count_launch();
    return 0;
  }
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
