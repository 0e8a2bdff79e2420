// Library extensions: batched evaluation into flat device buffers on a
// caller's stream, cell-sorted evaluation, a host-buffer entry with
// copy/compute overlap, launch-shape control and autotuning, and the
// device-side splitmix64 generator used for synthetic inputs.
#include <cub/device/device_radix_sort.cuh>
#include <limits.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <chrono>

#include "eg_internal.h"

namespace eg {

// ------------------------------------------------------------------ sorting
// Morton key of a point's cell (same cell rule as the evaluation) and its
// index; sorting the pairs gives a visiting order in which consecutive
// points share stencil rows.
__device__ __forceinline__ uint64_t spread3(uint64_t v) {
  v &= 0x1FFFFF;
  v = (v | (v << 32)) & 0x1F00000000FFFFull;
  v = (v | (v << 16)) & 0x1F0000FF0000FFull;
  v = (v | (v << 8)) & 0x100F00F00F00F00Full;
  v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
  v = (v | (v << 2)) & 0x1249249249249249ull;
  return v;
}

__global__ void k_cell_keys(const EvalArgs a, uint64_t *keys, int *idx) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= a.npts) return;
  int c[3];
  for (int ax = 0; ax < 3; ax++) {
    const double xd = a.pos_f64 ? reinterpret_cast<const double *>(a.pos)[3 * p + ax]
                                : (double)reinterpret_cast<const float *>(a.pos)[3 * p + ax];
    double u = (a.rule == 0) ? (xd - a.start[ax]) * a.dinv[ax] : xd * a.dinv[ax];
    int i = (int)floor(u);
    c[ax] = i < 0 ? 0 : (i > a.lim[ax] ? a.lim[ax] : i);
  }
  keys[p] = (spread3(c[0]) << 2) | (spread3(c[1]) << 1) | spread3(c[2]);
  idx[p] = (int)p;
}

__global__ void k_iota(int *p, int64_t n) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = (int)i;
}

// Batches of up to kSmallSort points are ordered by a counting sort on the
// Morton key of coarse cells (the cell index shifted right by `shift`, at
// most 16 per axis, 4096 keys), in two launches of S blocks (16, or one per
// kSortSlice points beyond that), block b owning the b-th slice of the
// points.  k_sort_keys keys its slice and writes the slice's key counts
// (row b of `hist`); k_sort_scatter gives key k of slice b the offset
// (points with smaller keys) + (points with key k in earlier slices) and
// places the slice's points with shared-memory atomics.
// Points of one key within a slice come out in the order the atomics place
// them; each point still writes its own output slot, so the results do not
// depend on that order.  (One block doing all of it was latency-bound at
// ~28 us for 17k points, an 8-block cluster no faster; the radix sort below,
// for larger batches, takes three launches, ~40 us at 17k points.)
constexpr int kSortSlice = 2048;  // most points a slice holds
constexpr int kSortMinBlocks = 16;
constexpr int kSortThreads = 1024;
constexpr int kCoarseKeys = 4096;
constexpr int kKeysPerThread = kCoarseKeys / kSortThreads;

// Morton interleave of three 4-bit coarse coordinates (12 bits).
__device__ __forceinline__ unsigned spread4(unsigned v) {
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4) | ((v & 8u) << 6);
}

// Coarse cell of one coordinate: FP32 is exact enough, since a point on the
// wrong side of a coarse-cell edge only changes the visiting order.
__device__ __forceinline__ unsigned coarse_cell(const EvalArgs &a, int ax, float x, int shift) {
  const float u = a.rule == 0 ? (x - (float)a.start[ax]) * a.dinvf[ax] : x * a.dinvf[ax];
  const int i = (int)floorf(u);
  return (unsigned)(i < 0 ? 0 : (i > a.lim[ax] ? a.lim[ax] : i)) >> shift;
}

__device__ __forceinline__ void slice_of(int n, int b, int &lo, int &hi) {
  const int chunk = (n + (int)gridDim.x - 1) / (int)gridDim.x;
  lo = min(n, b * chunk);
  hi = min(n, lo + chunk);
}

__global__ void __launch_bounds__(kSortThreads) k_sort_keys(const EvalArgs a, int shift, unsigned short *key,
                                                            unsigned *hist) {
  __shared__ unsigned count[kCoarseKeys];
  const int tid = threadIdx.x;
  int lo, hi;
  slice_of((int)a.npts, blockIdx.x, lo, hi);
  for (int k = tid; k < kCoarseKeys; k += kSortThreads) count[k] = 0;
  __syncthreads();
  for (int p = lo + tid; p < hi; p += kSortThreads) {
    float x[3];
#pragma unroll
    for (int ax = 0; ax < 3; ax++)
      x[ax] = a.pos_f64 ? (float)reinterpret_cast<const double *>(a.pos)[3 * (int64_t)p + ax]
                        : reinterpret_cast<const float *>(a.pos)[3 * (int64_t)p + ax];
    const unsigned k = (spread4(coarse_cell(a, 0, x[0], shift)) << 2) |
                       (spread4(coarse_cell(a, 1, x[1], shift)) << 1) | spread4(coarse_cell(a, 2, x[2], shift));
    key[p] = (unsigned short)k;
    atomicAdd(&count[k], 1u);
  }
  __syncthreads();
  uint4 c;
  c.x = count[kKeysPerThread * tid]; c.y = count[kKeysPerThread * tid + 1];
  c.z = count[kKeysPerThread * tid + 2]; c.w = count[kKeysPerThread * tid + 3];
  reinterpret_cast<uint4 *>(hist + (size_t)blockIdx.x * kCoarseKeys)[tid] = c;
}

__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(int n, const unsigned short *key,
                                                               const unsigned *hist, int *perm) {
  static_assert(kKeysPerThread == 4, "one uint4 of counts a thread");
  __shared__ unsigned count[kCoarseKeys];
  __shared__ unsigned warp_sum[kSortThreads / 32];
  const int tid = threadIdx.x, b = blockIdx.x;
  // this thread's 4 keys: their totals and the counts of earlier slices
  unsigned tot[4] = {0, 0, 0, 0}, before[4] = {0, 0, 0, 0};
#pragma unroll 4
  for (int r = 0; r < (int)gridDim.x; r++) {
    const uint4 c = reinterpret_cast<const uint4 *>(hist + (size_t)r * kCoarseKeys)[tid];
    tot[0] += c.x; tot[1] += c.y; tot[2] += c.z; tot[3] += c.w;
    if (r < b) { before[0] += c.x; before[1] += c.y; before[2] += c.z; before[3] += c.w; }
  }
  // exclusive prefix sum of the totals over the keys: within the thread,
  // then across lanes and warps
  const unsigned sum = tot[0] + tot[1] + tot[2] + tot[3];
  unsigned incl = sum;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const unsigned v = __shfl_up_sync(0xffffffffu, incl, d);
    if ((tid & 31) >= d) incl += v;
  }
  if ((tid & 31) == 31) warp_sum[tid >> 5] = incl;
  __syncthreads();
  if (tid < 32) {
    const unsigned w = warp_sum[tid];
    unsigned wi = w;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const unsigned v = __shfl_up_sync(0xffffffffu, wi, d);
      if (tid >= d) wi += v;
    }
    warp_sum[tid] = wi - w;
  }
  __syncthreads();
  unsigned run = warp_sum[tid >> 5] + incl - sum;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    count[4 * tid + j] = run + before[j];
    run += tot[j];
  }
  __syncthreads();
  int lo, hi;
  slice_of(n, b, lo, hi);
  for (int p = lo + tid; p < hi; p += kSortThreads) perm[atomicAdd(&count[key[p]], 1u)] = p;
}

static int coarse_shift(const EvalArgs &a) {
  int bits = 0;
  for (int ax = 0; ax < 3; ax++) {
    int b = 1;
    while ((1 << b) <= a.lim[ax]) b++;
    bits = std::max(bits, b);
  }
  return std::max(0, bits - 4);
}

static int sort_slices(int64_t n) { return (int)std::max<int64_t>(kSortMinBlocks, (n + kSortSlice - 1) / kSortSlice); }

// Scratch of the counting sort of n <= kSmallSort points: perm, the keys,
// then the slices' key counts.
size_t small_sort_bytes(int64_t n) {
  return align_up_sz(n * 4, 256) + align_up_sz(n * 2, 256) + (size_t)sort_slices(n) * kCoarseKeys * 4;
}

int small_sort_into(const EvalArgs &a, void *scratch, int **perm_out, cudaStream_t s) {
  const int64_t n = a.npts;
  const int S = sort_slices(n);
  char *base = (char *)scratch;
  int *perm = (int *)base;
  unsigned short *key = (unsigned short *)(base + align_up_sz(n * 4, 256));
  unsigned *hist = (unsigned *)(base + align_up_sz(n * 4, 256) + align_up_sz(n * 2, 256));
  k_sort_keys<<<S, kSortThreads, 0, s>>>(a, coarse_shift(a), key, hist);
  k_sort_scatter<<<S, kSortThreads, 0, s>>>((int)n, key, hist, perm);
  count_launch(2);
  EG_CUDA(cudaGetLastError());
  *perm_out = perm;
  return 0;
}

// With CUDA's lazy module loading a kernel's code is brought to the device
// on its first launch; asking for its attributes brings it there now.
int load_sort_kernels() {
  cudaFuncAttributes fa;
  EG_CUDA(cudaFuncGetAttributes(&fa, k_cell_keys));
  EG_CUDA(cudaFuncGetAttributes(&fa, k_sort_keys));
  EG_CUDA(cudaFuncGetAttributes(&fa, k_sort_scatter));
  return 0;
}

int sort_points(Table *t, const EvalArgs &a, int **perm_out, cudaStream_t s) {
  const int64_t n = a.npts;
  if (n > INT_MAX) return fail(EINSPLINE_GB300_ESIZE, "sorted evaluation takes at most %d points", INT_MAX);
  int bits = 0;
  for (int ax = 0; ax < 3; ax++) {
    int b = 1;
    while ((1 << b) <= a.lim[ax]) b++;
    bits = std::max(bits, b);
  }
  if (n <= kSmallSort) {
    const size_t need = small_sort_bytes(n);
    if (t->sort_bytes < need) {
      cudaFree(t->sort_dev);
      t->sort_dev = nullptr;
      t->sort_bytes = 0;
      if (cudaMalloc(&t->sort_dev, need) != cudaSuccess) {
        cudaGetLastError();
        return fail(EINSPLINE_GB300_ENOMEM, "cannot allocate %zu bytes for point sorting", need);
      }
      t->sort_bytes = need;
    }
    return small_sort_into(a, t->sort_dev, perm_out, s);
  }
  const int end_bit = std::min(63, 3 * bits);
  size_t temp = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, temp, (uint64_t *)nullptr, (uint64_t *)nullptr, (int *)nullptr,
                                  (int *)nullptr, (int)n, 0, end_bit, s);
  const size_t need = align_up_sz(n * 8, 256) * 2 + align_up_sz(n * 4, 256) * 2 + align_up_sz(temp, 256);
  if (t->sort_bytes < need) {
    cudaFree(t->sort_dev);
    t->sort_dev = nullptr;
    t->sort_bytes = 0;
    if (cudaMalloc(&t->sort_dev, need) != cudaSuccess) {
      cudaGetLastError();
      return fail(EINSPLINE_GB300_ENOMEM, "cannot allocate %zu bytes for point sorting", need);
    }
    t->sort_bytes = need;
  }
  char *p = (char *)t->sort_dev;
  uint64_t *k_in = (uint64_t *)p; p += align_up_sz(n * 8, 256);
  uint64_t *k_out = (uint64_t *)p; p += align_up_sz(n * 8, 256);
  int *v_in = (int *)p; p += align_up_sz(n * 4, 256);
  int *v_out = (int *)p; p += align_up_sz(n * 4, 256);
  void *tmp = p;
  k_cell_keys<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, k_in, v_in);
  count_launch();
  EG_CUDA(cudaGetLastError());
  EG_CUDA(cub::DeviceRadixSort::SortPairs(tmp, temp, k_in, k_out, v_in, v_out, (int)n, 0, end_bit, s));
  count_launch();
  *perm_out = v_out;
  return 0;
}

// ------------------------------------------------------------------ helpers
__global__ void k_scale_box(double *pos, int64_t n, double lx, double ly, double lz) {
  const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  pos[3 * p] *= lx; pos[3 * p + 1] *= ly; pos[3 * p + 2] *= lz;
}

static int check_opts(Table *t, const einspline_gb300_eval_opts *o) {
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle");
  if (!o) return fail(EINSPLINE_GB300_EINVAL, "opts is NULL");
  if (o->rule < 0 || o->rule > 1 || o->layout < 0 || o->layout > 1)
    return fail(EINSPLINE_GB300_EINVAL, "opts.rule and opts.layout must be 0 or 1");
  return 0;
}

static void setup_args(Table *t, const einspline_gb300_eval_opts *o, EvalArgs &a) {
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(t, a);
  a.pos_f64 = o->pos_f64;
  a.rule = o->rule;
  a.layout = o->layout;
  a.vstride = o->vstride ? o->vstride : t->ncol;
  a.gstride = o->gstride ? o->gstride : 3 * (int64_t)t->ncol;
  a.hstride = o->hstride ? o->hstride : (o->layout ? 9 : 6) * (int64_t)t->ncol;
}

static int eval_device(Table *t, const einspline_gb300_eval_opts *o, int64_t npts, const void *pos_d, void *v,
                       void *g, void *h, cudaStream_t s) {
  EvalArgs a;
  setup_args(t, o, a);
  a.npts = npts;
  a.pos = pos_d;
  a.vals = v; a.grads = g; a.hess = h;
  if (o->sort && npts > 1) {
    int *perm = nullptr;
    if (int r = sort_points(t, a, &perm, s)) return r;
    a.perm = perm;
  }
  int tx, ty, pb;
  pick_tile(t, o->vgh != 0, npts, tx, ty, pb, a.perm != nullptr);
  return launch_eval(t, a, o->vgh != 0, s, tx, ty, pb);
}

// n rows of `width` bytes from packed device rows into host rows `pitch`
// bytes apart: one linear copy when the host rows are packed too (the usual
// case), a strided one otherwise.
cudaError_t copy_rows(char *dst, size_t pitch, const char *src, size_t width, int64_t n, cudaStream_t s) {
  if (pitch == width) return cudaMemcpyAsync(dst, src, width * (size_t)n, cudaMemcpyDeviceToHost, s);
  return cudaMemcpy2DAsync(dst, pitch, src, width, width, (size_t)n, cudaMemcpyDeviceToHost, s);
}

}  // namespace eg

using namespace eg;

extern "C" {

int einspline_gb300_eval_3d(einspline_gb300_table *t, const einspline_gb300_eval_opts *o, int64_t npts,
                            const void *pos_d, void *vals_d, void *grads_d, void *hess_d, void *stream) {
  clear();
  if (int r = check_opts(t, o)) return r;
  if (npts < 0) return fail(EINSPLINE_GB300_EINVAL, "npts < 0");
  if (npts == 0) return 0;
  if (!pos_d || !vals_d || (o->vgh && (!grads_d || !hess_d)))
    return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_eval_3d: NULL buffer");
  if (int r = table_flush(t)) return r;
  cudaStream_t s = stream ? (cudaStream_t)stream : cudaStreamLegacy;
  return eval_device(t, o, npts, pos_d, vals_d, grads_d, hess_d, s);
}

// Device address of a pinned, mapped host buffer, or NULL.
static void *mapped_address(const void *h) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, h) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return (at.type == cudaMemoryTypeHost && at.devicePointer) ? at.devicePointer : nullptr;
}

int einspline_gb300_set_fp64_mode(einspline_gb300_table *t, int mode) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle (3D tables only)");
  if (mode != 0 && mode != 1) return fail(EINSPLINE_GB300_EINVAL, "mode must be 0 or 1");
  if (t->storage != ST_F64) return mode ? fail(EINSPLINE_GB300_EINVAL, "not an FP64 (d/z) table") : 0;
  {
    std::lock_guard<std::mutex> lock(t->mu);
    if (t->servers > 0 && mode != t->fp64_mode)
      return fail(EINSPLINE_GB300_EBUSY, "a request server uses this table: set the mode before creating it");
  }
  if (int r = table_flush(t)) return r;
  {
    std::lock_guard<std::mutex> lock(t->mu);
    t->fp64_mode = mode;
    t->df_stale = true;
    // the kernels differ between the modes: forget the tuned launch shapes
    for (int v = 0; v < 2; v++) {
      t->tuned_tx[v] = t->tuned_ty[v] = t->tuned_pb[v] = t->tuned_mode[v] = 0;
      t->tuned_s_tx[v] = t->tuned_s_ty[v] = t->tuned_s_pb[v] = t->tuned_s_mode[v] = 0;
    }
    if (mode == 0) {
      cudaFree(t->df_coefs);  // synchronises the device: no launch still reads it
      t->df_coefs = nullptr;
      return 0;
    }
  }
  if (int r = table_df_refresh(t)) {
    // No double-float copy (its allocation failed): the table stays in IEEE
    // mode, so no later flush tries to allocate the copy again.
    std::lock_guard<std::mutex> lock(t->mu);
    if (!t->df_coefs) t->fp64_mode = 0;
    return r;
  }
  return 0;
}

int einspline_gb300_get_fp64_mode(einspline_gb300_table *t) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle (3D tables only)");
  return t->fp64_mode;
}

int einspline_gb300_set_host_direct(einspline_gb300_table *t, int mode) {
  clear();
  if (!table_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle");
  if (mode < -1 || mode > 1) return fail(EINSPLINE_GB300_EINVAL, "mode must be -1, 0 or 1");
  t->host_direct = mode < 0 ? 0 : mode;
  return 0;
}

int einspline_gb300_eval_3d_host(einspline_gb300_table *t, const einspline_gb300_eval_opts *o, int64_t npts,
                                 const void *pos_h, void *vals_h, void *grads_h, void *hess_h) {
  clear();
  if (int r = check_opts(t, o)) return r;
  if (npts < 0) return fail(EINSPLINE_GB300_EINVAL, "npts < 0");
  if (npts == 0) return 0;
  if (!pos_h || !vals_h || (o->vgh && (!grads_h || !hess_h)))
    return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_eval_3d_host: NULL buffer");
  if (int r = table_flush(t)) return r;
  std::lock_guard<std::mutex> lock(t->mu);
  if (t->host_direct == 1) {
    // Pinned host buffers mapped into the device address space: one launch
    // reads the positions and writes the results through NVLink-C2C / PCIe,
    // with no staging copies.  (On GB300 machines this measured 1.3 G vgh
    // evals/s against 4.5 G for the copy pipeline below, so it is opt-in.)
    void *pd = mapped_address(pos_h), *vd = mapped_address(vals_h);
    void *gd = o->vgh ? mapped_address(grads_h) : nullptr, *hd = o->vgh ? mapped_address(hess_h) : nullptr;
    if (pd && vd && (!o->vgh || (gd && hd))) {
      cudaStream_t s = t->stream;
      if (int r = eval_device(t, o, npts, pd, vd, gd, hd, s)) return r;
      EG_CUDA(cudaStreamSynchronize(s));
      return 0;
    }
    return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_eval_3d_host: direct mode needs pinned, mapped buffers");
  }
  const size_t rb = t->storage == ST_F64 ? 8 : 4;
  const int hq = o->layout ? 9 : 6;
  const size_t per_pt_out = (size_t)t->ncol * rb * (o->vgh ? (4 + hq) : 1);
  const size_t pos_b = o->pos_f64 ? 24 : 12;
  // Chunks of output, two in flight: the first about 8 MB, so that the
  // device-to-host link starts early, then doubling up to about 128 MB, so
  // that few copies carry the rest (the link, ~193 GB/s, is the bound).
  int64_t chunk = std::max<int64_t>(1, (int64_t)((128u << 20) / per_pt_out));
  chunk = std::min(chunk, npts);
  int64_t cur = std::max<int64_t>(1, (int64_t)((8u << 20) / per_pt_out));
  const size_t slot = align_up_sz(chunk * pos_b, 256) + align_up_sz(chunk * per_pt_out, 256);
  if (t->pipe_bytes < 2 * slot) {
    cudaFree(t->pipe_dev);
    t->pipe_dev = nullptr;
    t->pipe_bytes = 0;
    if (cudaMalloc(&t->pipe_dev, 2 * slot) != cudaSuccess) {
      cudaGetLastError();
      return fail(EINSPLINE_GB300_ENOMEM, "cannot allocate %zu bytes of pipeline buffers", 2 * slot);
    }
    t->pipe_bytes = 2 * slot;
  }
  for (int i = 0; i < 2; i++)
    if (!t->pipe_stream[i]) EG_CUDA(cudaStreamCreateWithFlags(&t->pipe_stream[i], cudaStreamNonBlocking));
  const int64_t vs = o->vstride ? o->vstride : t->ncol;
  const int64_t gs = o->gstride ? o->gstride : 3 * (int64_t)t->ncol;
  const int64_t hs = o->hstride ? o->hstride : hq * (int64_t)t->ncol;
  einspline_gb300_eval_opts od = *o;
  od.vstride = t->ncol; od.gstride = 3 * (int64_t)t->ncol; od.hstride = hq * (int64_t)t->ncol;
  od.sort = 0;
  int k = 0;
  int64_t n = 0;
  for (int64_t p0 = 0; p0 < npts; p0 += n, k++) {
    n = std::min(std::min(cur, chunk), npts - p0);
    cur = std::min(2 * cur, chunk);
    cudaStream_t s = t->pipe_stream[k & 1];
    char *base = (char *)t->pipe_dev + (size_t)(k & 1) * slot;
    char *pos_d = base;
    char *out_d = base + align_up_sz(chunk * pos_b, 256);
    char *v_d = out_d;
    char *g_d = v_d + (size_t)chunk * t->ncol * rb;
    char *h_d = g_d + (size_t)chunk * 3 * t->ncol * rb;
    EG_CUDA(cudaMemcpyAsync(pos_d, (const char *)pos_h + p0 * pos_b, n * pos_b, cudaMemcpyHostToDevice, s));
    if (int r = eval_device(t, &od, n, pos_d, v_d, g_d, h_d, s)) return r;
    EG_CUDA(copy_rows((char *)vals_h + p0 * vs * rb, vs * rb, v_d, t->ncol * rb, n, s));
    if (o->vgh) {
      EG_CUDA(copy_rows((char *)grads_h + p0 * gs * rb, gs * rb, g_d, 3 * t->ncol * rb, n, s));
      EG_CUDA(copy_rows((char *)hess_h + p0 * hs * rb, hs * rb, h_d, hq * t->ncol * rb, n, s));
    }
  }
  EG_CUDA(cudaStreamSynchronize(t->pipe_stream[0]));
  EG_CUDA(cudaStreamSynchronize(t->pipe_stream[1]));
  return wait_status(t, "einspline_gb300_eval_3d_host");
}

int einspline_gb300_set_load_mode(einspline_gb300_table *t, int mode) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle");
  if (mode < -1 || mode > 5) return fail(EINSPLINE_GB300_EINVAL, "load mode must be -1, 0, 1, 2, 3, 4 or 5");
  t->tile_mode = mode;
  return 0;
}

int einspline_gb300_wait_status(einspline_gb300_table *t) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle");
  return wait_status(t, "einspline_gb300_wait_status");
}

int einspline_gb300_test_wait_timeout(einspline_gb300_table *t, int stage, double seconds) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle");
  if (stage < 0) {
    t->test_skip.store(0);
    return 0;
  }
  if (!(seconds >= 1e-6 && seconds <= 1.0))
    return fail(EINSPLINE_GB300_EINVAL, "the wait limit must lie in [1 us, 1 s] (got %g s)", seconds);
  t->test_wait_ns = (unsigned long long)(seconds * 1e9);
  t->test_skip.store(stage + 1);
  return 0;
}

int einspline_gb300_set_tile(einspline_gb300_table *t, int tx, int ty, int pb) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle");
  if (tx == 0 && ty == 0 && pb == 0) { t->tile_tx = t->tile_ty = t->tile_pb = 0; return 0; }
  if (tx < 32 || tx % 32 || ty < 1 || tx * ty > 256 || pb < 1 || pb > 64)
    return fail(EINSPLINE_GB300_EINVAL, "tile must have tx a multiple of 32, tx*ty <= 256, 1 <= pb <= 64");
  t->tile_tx = tx; t->tile_ty = ty; t->tile_pb = pb;
  return 0;
}

int einspline_gb300_get_tile(einspline_gb300_table *t, int *tx, int *ty, int *pb) {
  clear();
  if (!table3_ok(t) || !tx || !ty || !pb) return fail(EINSPLINE_GB300_EINVAL, "bad argument");
  pick_tile(t, true, 0, *tx, *ty, *pb);
  return 0;
}

int einspline_gb300_get_launch_shape(einspline_gb300_table *t, int sorted, int vgh, int *tx, int *ty, int *pb,
                                     int *mode) {
  clear();
  if (!table3_ok(t) || !tx || !ty || !pb || !mode) return fail(EINSPLINE_GB300_EINVAL, "bad argument");
  pick_tile(t, vgh != 0, 0, *tx, *ty, *pb, sorted != 0);
  *mode = pick_mode(t, vgh != 0, sorted != 0);
  return 0;
}

int einspline_gb300_get_load_mode(einspline_gb300_table *t) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle");
  return pick_mode(t, true);
}

}  // extern "C"

namespace eg {

__global__ void k_gather_pos(const double *pos, const int *perm, int64_t n, double *out) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t s = perm[i];
  out[3 * i] = pos[3 * s];
  out[3 * i + 1] = pos[3 * s + 1];
  out[3 * i + 2] = pos[3 * s + 2];
}

// npts points uniform in the table's box (rule 1 measures positions from the
// grid origin), double, into pos.
static void uniform_points(Table *t, double *pos, int64_t npts) {
  einspline_gb300_fill_uniform(pos, 3 * npts, 1, 0x5eed5eedull, 0, 0.0, 1.0, t->stream);
  k_scale_box<<<(unsigned)((npts + 255) / 256), 256, 0, t->stream>>>(pos, npts, t->end[0] - t->start[0],
                                                                     t->end[1] - t->start[1], t->end[2] - t->start[2]);
  count_launch();
}

// A launch over npts points at pos (double, rule 1, GPU layout) writing to
// out (room for npts points' outputs).
static EvalArgs tuning_args(Table *t, const double *pos, int64_t npts, void *out) {
  const size_t rb = t->storage == ST_F64 ? 8 : 4;
  EvalArgs a;
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(t, a);
  a.pos = pos;
  a.pos_f64 = 1;
  a.rule = 1;
  a.layout = 0;
  a.npts = npts;
  a.vals = out;
  a.grads = (char *)out + (size_t)npts * t->ncol * rb;
  a.hess = (char *)out + (size_t)npts * 4 * t->ncol * rb;
  a.vstride = t->ncol; a.gstride = 3 * (int64_t)t->ncol; a.hstride = 6 * (int64_t)t->ncol;
  return a;
}

// Times every load mode and tile shape on launch a (three launches each,
// after one warm launch) and returns the fastest as {tx, ty, pb, mode}.
static int tune_shapes(Table *t, const EvalArgs &a, bool vgh, int best_shape[4]) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  const int VW = elems_per_thread(t);
  const int saved_pf = t->tile_mode;
  // Load modes worth timing: IEEE FP64 has the direct kernels only, the wide
  // pipeline (3) is for 16-bit tables.
  const int ks = t->storage == ST_F64 ? (t->fp64_mode == 1 && t->df_coefs ? (int)ST_DF : (int)ST_F64) : t->storage;
  std::vector<int> modes = {0, 1};
  if (ks != ST_F64) {
    modes.push_back(2);
    if (is16(ks)) modes.push_back(3);
    modes.push_back(4);
  }
  // F16 and BF16 vgh use the tensor-core reduction (mode 5), whose results
  // differ from the other modes' by FP32 rounding: only its points per block
  // are tuned, so tuning never changes a result.
  if ((ks == ST_F16 || ks == ST_BF16) && vgh) modes = {5};
  int rc = 0;
  for (int pf : modes) {
    t->tile_mode = pf;
    if (pf == 5) {
      // every count from 8 up to 11, the most at which three blocks share an
      // SM (11 was 0.3-1 % faster than 10 on cell-sorted batches)
      for (int pb = 2; pb <= 11 && !rc; pb += pb < 8 ? 2 : 1) {
        EvalArgs b = a;
        if ((rc = launch_eval(t, b, vgh, t->stream, 128, 1, pb))) break;
        cudaEventRecord(e0, t->stream);
        for (int r = 0; r < 3; r++) {
          b = a;
          launch_eval(t, b, vgh, t->stream, 128, 1, pb);
        }
        cudaEventRecord(e1, t->stream);
        cudaEventSynchronize(e1);
        float ms = 0;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          best_shape[0] = 128; best_shape[1] = 1; best_shape[2] = pb; best_shape[3] = pf;
        }
      }
      continue;
    }
    const int vw = VW * ((pf == 3 || (pf == 4 && is16(ks))) ? 2 : 1);
    for (int tx = 32; tx <= 256 && !rc; tx *= 2) {
      if (tx > 32 && (tx / 2) * vw >= t->ncol) break;  // wider tiles only idle threads
      if (pf == 3 && tx > 32) break;                   // the wide pipeline is one warp per block
      for (int ty = 1; tx * ty <= 256 && (pf < 2 || ty == 1) && !rc; ty *= 2)
        for (int m = 1; m <= 8 && !rc; m *= 2) {
          const int pb = ty * m;
          if (pb > 64) continue;
          EvalArgs b = a;
          if ((rc = launch_eval(t, b, vgh, t->stream, tx, ty, pb))) break;
          cudaEventRecord(e0, t->stream);
          for (int r = 0; r < 3; r++) {
            b = a;
            launch_eval(t, b, vgh, t->stream, tx, ty, pb);
          }
          cudaEventRecord(e1, t->stream);
          cudaEventSynchronize(e1);
          float ms = 0;
          cudaEventElapsedTime(&ms, e0, e1);
          if (ms < best) {
            best = ms;
            best_shape[0] = tx; best_shape[1] = ty; best_shape[2] = pb; best_shape[3] = pf;
          }
        }
    }
    if (rc) break;
  }
  t->tile_mode = saved_pf;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  cudaError_t e = cudaStreamSynchronize(t->stream);
  if (e != cudaSuccess) return cuda_check(e, "autotune");
  return 0;
}

}  // namespace eg

extern "C" {

int einspline_gb300_autotune(einspline_gb300_table *t, int64_t npts, int vgh) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle");
  if (npts < 1) return fail(EINSPLINE_GB300_EINVAL, "npts must be >= 1");
  if (int r = table_flush(t)) return r;
  const size_t rb = t->storage == ST_F64 ? 8 : 4;
  const size_t out_b = (size_t)npts * t->ncol * rb * (vgh ? 10 : 1);
  void *buf = nullptr;
  if (cudaMalloc(&buf, out_b + (size_t)npts * 24) != cudaSuccess) {
    cudaGetLastError();
    return fail(EINSPLINE_GB300_ENOMEM, "autotune scratch");
  }
  double *pos = (double *)((char *)buf + out_b);
  uniform_points(t, pos, npts);
  const EvalArgs a = tuning_args(t, pos, npts, buf);
  int shape[4] = {0, 0, 0, 0};
  const int r = tune_shapes(t, a, vgh != 0, shape);
  cudaFree(buf);
  if (r) return r;
  const int v = vgh ? 1 : 0;
  t->tuned_tx[v] = shape[0]; t->tuned_ty[v] = shape[1]; t->tuned_pb[v] = shape[2]; t->tuned_mode[v] = shape[3];
  return 0;
}

int einspline_gb300_autotune_sorted(einspline_gb300_table *t, int64_t npts, int vgh) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "bad table handle");
  if (npts < 1 || npts > INT_MAX) return fail(EINSPLINE_GB300_EINVAL, "npts must be in [1, %d]", INT_MAX);
  if (int r = table_flush(t)) return r;
  // The batch's points in cell order; shapes are timed on a window of
  // consecutive sorted points, which has the batch's local density.
  const int64_t W = std::min<int64_t>(npts, 32768);
  const size_t rb = t->storage == ST_F64 ? 8 : 4;
  const size_t out_b = align_up_sz((size_t)W * t->ncol * rb * (vgh ? 10 : 1), 256);
  void *buf = nullptr;
  if (cudaMalloc(&buf, out_b + align_up_sz((size_t)npts * 24, 256) + (size_t)W * 24) != cudaSuccess) {
    cudaGetLastError();
    return fail(EINSPLINE_GB300_ENOMEM, "autotune scratch");
  }
  double *all = (double *)((char *)buf + out_b);
  double *win = (double *)((char *)all + align_up_sz((size_t)npts * 24, 256));
  uniform_points(t, all, npts);
  EvalArgs s = tuning_args(t, all, npts, buf);
  int *perm = nullptr;
  int r = sort_points(t, s, &perm, t->stream);
  if (!r) {
    k_gather_pos<<<(unsigned)((W + 255) / 256), 256, 0, t->stream>>>(all, perm, W, win);
    count_launch();
    const EvalArgs a = tuning_args(t, win, W, buf);
    int shape[4] = {0, 0, 0, 0};
    r = tune_shapes(t, a, vgh != 0, shape);
    if (!r) {
      const int v = vgh ? 1 : 0;
      t->tuned_s_tx[v] = shape[0]; t->tuned_s_ty[v] = shape[1]; t->tuned_s_pb[v] = shape[2];
      t->tuned_s_mode[v] = shape[3];
    }
  }
  cudaFree(buf);
  return r;
}

}  // extern "C"

// ------------------------------------------------------------------ synth
namespace {
__global__ void k_fill_uniform(void *dst, int64_t n, int f64, uint64_t seed, int64_t offset, double lo, double hi) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t z = seed + (uint64_t)(offset + i + 1) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z = z ^ (z >> 31);
  const double u = __dmul_rn((double)(z >> 11), 1.0 / 9007199254740992.0);
  const double v = __dadd_rn(lo, __dmul_rn(__dsub_rn(hi, lo), u));
  if (f64) ((double *)dst)[i] = v;
  else ((float *)dst)[i] = __double2float_rn(v);
}
}  // namespace

extern "C" int einspline_gb300_fill_uniform(void *dst_d, int64_t n, int f64, uint64_t seed, int64_t offset, double lo,
                                            double hi, void *stream) {
  clear();
  if (!dst_d || n < 0) return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_fill_uniform: bad argument");
  if (n == 0) return 0;
  const int64_t blocks = (n + 255) / 256;
  if (blocks > INT_MAX) return fail(EINSPLINE_GB300_ESIZE, "fill too large");
  k_fill_uniform<<<(unsigned)blocks, 256, 0, stream ? (cudaStream_t)stream : cudaStreamLegacy>>>(dst_d, n, f64, seed,
                                                                                                 offset, lo, hi);
  count_launch();
  EG_CUDA(cudaGetLastError());
  return 0;
}
