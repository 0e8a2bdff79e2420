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
//
// Set-up: the first call on a device (per CUDA context) looks the array's
// device address up and brings this entry's kernels to the device.  CUDA
// loads modules lazily by default, so that is when the 10 MiB array and the
// kernels' code take device memory: make the first call -- an empty one,
// npts = 0, with the table and options of later calls, does the whole
// set-up -- before a pool allocator takes the device's free memory, and
// before any stream capture.
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
// the host looks the device address up in each context it is used in.
static __device__ __align__(256) unsigned char g_sort_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;

// Per device: the context the set-up below was made in and the array's
// device address there.  A new context on the device (after
// cudaDeviceReset, say) loads the module again, possibly elsewhere, so the
// set-up is redone whenever the current context differs.
struct DeviceSetup {
  CUcontext ctx = nullptr;
  void *scratch = nullptr;
};
std::mutex g_mu;
DeviceSetup g_setup[kMaxDevices];

using CtxGetCurrent = CUresult (*)(CUcontext *);
CtxGetCurrent ctx_get_current() {
  static CtxGetCurrent fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      p = nullptr;
    }
    return reinterpret_cast<CtxGetCurrent>(p);
  }();
  return fn;
}

// Radix-sort bit range of the cell keys of a table's launches.
int key_end_bit(const EvalArgs &a) {
  int bits = 0;
  for (int ax = 0; ax < 3; ax++) {
    int b = 1;
    while ((1 << b) <= a.lim[ax]) b++;
    if (b > bits) bits = b;
  }
  return 3 * bits < 63 ? 3 * bits : 63;
}

// The once-per-device (per context) set-up, made by the first call on a
// device with that device current: the array's device address, and every
// kernel this entry launches brought to the device now, since with CUDA's
// lazy module loading a module's code and its file-scope arrays are given
// device memory when it is first used.  The radix sort's kernels are loaded
// by sorting the array's own contents once; the largest work space the sort
// can need (at the most points, widest keys) is checked against the fixed
// one here.
int device_setup(cudaStream_t s, void **out) {
  int dev = 0;
  EG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return fail(EINSPLINE_GB300_EINVAL, "device index %d out of range", dev);
  CtxGetCurrent get = ctx_get_current();
  CUcontext ctx = nullptr;
  if (!get || get(&ctx) != CUDA_SUCCESS || !ctx)
    return fail(EINSPLINE_GB300_ECUDA, "einspline_gb300_eval_3d_sorted_noalloc: no current CUDA context");
  std::lock_guard<std::mutex> g(g_mu);
  DeviceSetup &d = g_setup[dev];
  if (d.ctx == ctx && d.scratch) {
    *out = d.scratch;
    return 0;
  }
  void *p = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&p, g_sort_scratch);
  if (e != cudaSuccess || !p) return cuda_check(e != cudaSuccess ? e : cudaErrorInvalidSymbol, "cudaGetSymbolAddress");
  if (int r = load_sort_kernels()) return r;
  char *base = (char *)p;
  uint64_t *k_in = (uint64_t *)base, *k_out = (uint64_t *)(base + kKeyBytes);
  int *v_in = (int *)(base + 2 * kKeyBytes), *v_out = (int *)(base + 2 * kKeyBytes + kIdxBytes);
  size_t temp_bytes = 0;
  EG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, temp_bytes, k_in, k_out, v_in, v_out, (int)kNoAllocMaxPoints, 0,
                                          63, s));
  if (temp_bytes > kSortTempBytes)
    return fail(EINSPLINE_GB300_ESIZE, "sort work space of %zu bytes exceeds the fixed %zu", temp_bytes,
                kSortTempBytes);
  EG_CUDA(cub::DeviceRadixSort::SortPairs(base + 2 * kKeyBytes + 2 * kIdxBytes, temp_bytes, k_in, k_out, v_in, v_out,
                                          (int)kNoAllocMaxPoints, 0, 63, s));
  count_launch();
  d.ctx = ctx;
  d.scratch = p;
  *out = p;
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
  cudaStream_t s = stream ? (cudaStream_t)stream : cudaStreamLegacy;
  void *scratch = nullptr;
  if (int r = device_setup(s, &scratch)) return r;
  {
    // Refuse what would need memory: the double-float copy of an FP64 table
    // in double-float mode is made on demand by a flush.
    std::lock_guard<std::mutex> g(t->mu);
    if (t->storage == ST_F64 && t->fp64_mode == 1 && !t->df_coefs)
      return fail(EINSPLINE_GB300_ENOMEM,
                  "einspline_gb300_eval_3d_sorted_noalloc: the table's double-float copy is missing and would have "
                  "to be allocated; set the FP64 mode again first");
  }
  // An empty call is the warm-up: it also brings the evaluation kernel of
  // this table and these options to the device.
  if (npts == 0) return load_eval_kernel(t, o->vgh != 0, true);
  if (!pos_d || !vals_d || (o->vgh && (!grads_d || !hess_d)))
    return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_eval_3d_sorted_noalloc: NULL buffer");
  // Queued set_* calls are solved first; the solve's work space was made when
  // they were queued, so this allocates nothing either (it synchronises the
  // table's stream when there was something to solve).
  if (int r = table_flush(t)) return r;

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
  const int end_bit = key_end_bit(a);
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
