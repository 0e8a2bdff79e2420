// Cell-sorted batched evaluation that allocates no memory.
//
// einspline_gb300_eval_3d with opts.sort = 1 sorts the points by cell in a
// scratch area (keys, key counts and the visiting order, or the radix sort's
// work space for large batches) that it allocates with cudaMalloc and keeps
// on the table.  Some callers cannot let
// a library allocate device memory while they run: QMC drivers that hand the
// whole device to their own pool allocator and account for every byte, code
// that runs while another component holds the device's allocation lock, or
// callers that must not trigger the implicit device synchronisation that
// cudaMalloc/cudaFree can cause in the middle of a timed or captured region.
// This entry gives them the same result with the scratch in a fixed
// file-scope device array instead.
#include <cub/device/device_radix_sort.cuh>
#include <string.h>

#include <mutex>

#include "eg_internal.h"

namespace eg {
namespace {

// Largest batch the fixed scratch holds.
constexpr int64_t kNoAllocMaxPoints = 262144;
constexpr size_t kKeyBytes = (size_t)kNoAllocMaxPoints * 8;
constexpr size_t kIdxBytes = (size_t)kNoAllocMaxPoints * 4;
constexpr size_t kSortTempBytes = (size_t)4 << 20;
constexpr size_t kScratchBytes = 2 * kKeyBytes + 2 * kIdxBytes + kSortTempBytes;  // 10 MiB

// One copy per device that loads this library, alive until the process
// exits.  Device code could name it directly; host code must not use its
// name as an address (on the host it is only a stand-in for the symbol), so
// the host looks the device address up once per device below.
static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
void *g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch on the current device, looked up on the
// first call made with that device current.
int scratch_for_current_device(void **out) {
  int dev = 0;
  EG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(EINSPLINE_GB300_EINVAL, "device index %d out of range", dev);
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
    if (e != cudaSuccess || !p) return cuda_check(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return 0;
}

}  // namespace
}  // namespace eg

using namespace eg;

extern "C" int einspline_gb300_eval_3d_sorted_noalloc(einspline_gb300_table *t, const einspline_gb300_eval_opts *o,
                                                      int64_t npts, const void *pos_d, void *vals_d, void *grads_d,
                                                      void *hess_d, void *stream) {
  clear();
  if (!table3_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_eval_3d_sorted_noalloc: bad table handle");
  if (!o || o->rule < 0 || o->rule > 1 || o->layout < 0 || o->layout > 1)
    return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_eval_3d_sorted_noalloc: bad options");
  if (npts < 0) return fail(EINSPLINE_GB300_EINVAL, "npts < 0");
  if (npts > kNoAllocMaxPoints)
    return fail(EINSPLINE_GB300_ESIZE,
                "einspline_gb300_eval_3d_sorted_noalloc: %lld points exceed its fixed scratch of %lld points; "
                "split the batch or use einspline_gb300_eval_3d",
                (long long)npts, (long long)kNoAllocMaxPoints);
  if (npts == 0) return 0;
  if (!pos_d || !vals_d || (o->vgh && (!grads_d || !hess_d)))
    return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_eval_3d_sorted_noalloc: NULL buffer");
  void *scratch = nullptr;
  if (int r = scratch_for_current_device(&scratch)) return r;
  // Queued set_* calls are solved first; the solve's work space was made when
  // they were queued, so this allocates nothing either.
  if (int r = table_flush(t)) return r;
  cudaStream_t s = stream ? (cudaStream_t)stream : cudaStreamLegacy;

  EvalArgs a;
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(t, a);
  a.pos_f64 = o->pos_f64;
  a.rule = o->rule;
  a.layout = o->layout;
  a.vstride = o->vstride ? o->vstride : t->ncol;
  a.gstride = o->gstride ? o->gstride : 3 * (int64_t)t->ncol;
  a.hstride = o->hstride ? o->hstride : (o->layout ? 9 : 6) * (int64_t)t->ncol;
  a.npts = npts;
  a.pos = pos_d;
  a.vals = vals_d; a.grads = grads_d; a.hess = hess_d;

  int tx, ty, pb;
  pick_tile(t, o->vgh != 0, npts, tx, ty, pb, true);
  // Batches of up to kSmallSort points: the two-launch counting sort, whose
  // scratch (under 2 MB) is written before it is read.
  if (npts <= kSmallSort && small_sort_bytes(npts) <= kScratchBytes) {
    int *perm = nullptr;
    if (int r = small_sort_into(a, scratch, &perm, s)) return r;
    a.perm = perm;
    return launch_eval(t, a, o->vgh != 0, s, tx, ty, pb);
  }
  char *p = (char *)scratch;
  uint64_t *k_in = (uint64_t *)p;
  uint64_t *k_out = (uint64_t *)(p + kKeyBytes);
  int *v_in = (int *)(p + 2 * kKeyBytes);
  int *v_out = (int *)(p + 2 * kKeyBytes + kIdxBytes);
  void *temp = p + 2 * kKeyBytes + 2 * kIdxBytes;
  int bits = 0;
  for (int ax = 0; ax < 3; ax++) {
    int b = 1;
    while ((1 << b) <= a.lim[ax]) b++;
    if (b > bits) bits = b;
  }
  const int end_bit = 3 * bits < 63 ? 3 * bits : 63;
  size_t temp_bytes = 0;
  EG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, k_in, k_out, v_in, v_out, (int)npts, 0, end_bit, s));
  if (temp_bytes > kSortTempBytes)
    return fail(EINSPLINE_GB300_ESIZE, "sort work space of %zu bytes exceeds the fixed %zu", temp_bytes, kSortTempBytes);
  // Every key and index used below is written first: nothing in the scratch
  // has to start at zero, and the previous call's contents do not matter.
  k_cell_keys<<<(unsigned)((npts + 255) / 256), 256, 0, s>>>(a, k_in, v_in);
  count_launch();
  EG_CUDA(cudaGetLastError());
  EG_CUDA(cub::DeviceRadixSort::SortPairs(temp, temp_bytes, k_in, k_out, v_in, v_out, (int)npts, 0, end_bit, s));
  count_launch();
  a.perm = v_out;
  return launch_eval(t, a, o->vgh != 0, s, tx, ty, pb);
}
