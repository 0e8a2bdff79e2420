// Internal declarations shared by the library's translation units.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <mutex>
#include <unordered_map>
#include <vector>

#include "einspline_gb300.h"

namespace eg {

constexpr uint32_t kMagic = 0x45473330u;  // "EG30"

enum Storage { ST_NATIVE = 0, ST_F32 = 1, ST_F16 = 2, ST_BF16 = 3, ST_F64 = 4, ST_I16 = 5,
               // kernel-only: an FP64 table read from its double-float shadow
               ST_DF = 6 };
__host__ __device__ constexpr bool is16(int st) { return st == ST_F16 || st == ST_BF16 || st == ST_I16; }
// I16 values are stored with this bias so that a 16-bit pattern u becomes
// the float 2^23 + u by inserting it under the exponent of 2^23.
constexpr int kI16Bias = 32768;

// ---------------------------------------------------------------- errors
// Records a status for the calling thread; aborts when abort mode is on.
int fail(int code, const char *fmt, ...);
void clear();
// Records a failed CUDA status e (call it only when e != cudaSuccess) and
// returns ECUDA.
int cuda_check(cudaError_t e, const char *what);
#define EG_CUDA(call)                                                  \
  do {                                                                 \
    cudaError_t eg_e_ = (call);                                        \
    if (eg_e_ != cudaSuccess) return ::eg::cuda_check(eg_e_, #call);   \
  } while (0)
void count_launch(int n = 1);
inline size_t align_up_sz(size_t v, size_t a) { return (v + a - 1) / a * a; }

// --------------------------------------------------------- line factors
// Data-independent part of the 1D interpolation solve for one axis, found
// once on the host by running the reference elimination on the band
// coefficients alone.  The device kernels then only push right-hand sides
// through the recorded multipliers and divisors, in the reference's order.
struct LineFactors {
  int M = 0;
  int cyclic = 1;   // periodic/antiperiodic (1) or boundary-row system (0)
  int anti = 0;     // antiperiodic wrap sign
  int lcode = 0, rcode = 0;
  // Packed arrays, each of length M+2:
  //  cyclic: P (divisors), L (sub-diagonal multipliers), E (last-row
  //          multipliers), U (super-diagonal), LC (wrap column); scalars F, Q
  //  bc:     P, L, U; scalars R0, R1, Q (last row), U0a, U0b (first row),
  //          and the boundary rows' own divisor P[0]
  std::vector<double> P, L, E, U, LC;
  double F = 0, Q = 0, R0 = 0, R1 = 0, U0a = 0, U0b = 0;
};
void build_line_factors(int M, int lcode, int rcode, double delta_inv, LineFactors &f);
// Offsets of the arrays inside the packed device copy.
struct PackedFactors {
  int M, cyclic, anti, pad_;
  double F, Q, R0, R1, U0a, U0b;
  double QH, QL;  // Q's reciprocal as hi + lo (QH = 0: divide Q directly)
};
size_t packed_factor_doubles(int M);
void pack_line_factors(const LineFactors &f, std::vector<double> &out);

// ----------------------------------------------------------------- table
}  // namespace eg

struct einspline_gb300_table {
  uint32_t magic = eg::kMagic;
  char kind = 's';        // 's','d','c','z'
  int dims = 3;           // 1, 2 or 3 axes (1D/2D/3D multi-splines); axes
                          // beyond dims hold one point and one coefficient
  int storage = eg::ST_F32;
  int ncomp = 1;          // 1 real, 2 complex
  int num_splines = 0;
  int ncol = 0;           // ncomp * num_splines real columns
  int ncol_pad = 0;       // real columns per stored row (128-byte rows)
  int elem_bytes = 4;
  int M[3] = {0, 0, 0};   // data points per axis
  int Nc[3] = {0, 0, 0};  // coefficients per axis
  double start[3], end[3], delta[3], dinv[3];
  int lcode[3], rcode[3];
  double lval[3][2], rval[3][2];
  int64_t xs = 0, ys = 0, zs = 0;  // strides in stored reals
  size_t table_bytes = 0;
  void *coefs = nullptr;            // device
  float *scale = nullptr;           // device, ncol_pad floats (16-bit storage)
  // FP64 tables: 0 evaluate in IEEE FP64; 1 in double-float arithmetic from
  // a shadow copy holding each coefficient as (hi, lo) floats
  int fp64_mode = 0;
  void *df_coefs = nullptr;         // device, table_bytes
  bool df_stale = true;
  int servers = 0;                  // request servers built on this table
  bool owns = true;

  // queued set calls
  std::mutex mu;
  int cap = 0;                      // splines per batched solve
  std::vector<int> pend_spline;     // slot -> spline index
  std::unordered_map<int, int> slot_of;
  void *staging = nullptr;          // device, cap * points * ncomp values of the input type
  int in_bytes = 4;                 // bytes per input real (4 for s/c, 8 for d/z)
  double *work_a = nullptr;         // device FP64 [Mx][My][Mz][cap*ncomp]
  double *work_w = nullptr;         // device FP64 [Nx][Ny][Nz][cap*ncomp]
  float *colmax = nullptr;          // device, cap*ncomp
  int *slot_spline_d = nullptr;     // device, cap
  double *factors_d = nullptr;      // device, 3 packed factor sets
  size_t factor_off[3] = {0, 0, 0};
  cudaStream_t stream = nullptr;

  // single-point entry scratch: 40 * ncol output reals in mapped pinned
  // host memory, which the kernels write directly
  void *pt_host = nullptr;
  void *pt_dev = nullptr;           // its device address

  // host-buffer pipeline scratch (einspline_gb300_eval_3d_host)
  void *pipe_dev = nullptr;
  size_t pipe_bytes = 0;
  cudaStream_t pipe_stream[2] = {nullptr, nullptr};
  cudaEvent_t pipe_event[2] = {nullptr, nullptr};

  // host-buffer entry: 0 copy through device memory (default), 1 kernels
  // read/write mapped pinned host buffers directly
  int host_direct = 0;

  // host mirror of the coefficients in the value type (einspline_gb300_host_coefs):
  // pinned, mapped host memory of table_bytes / elem_bytes reals
  void *host_coefs = nullptr;
  size_t host_coefs_bytes = 0;

  // cell-sorted evaluation scratch
  void *sort_dev = nullptr;
  size_t sort_bytes = 0;

  // launch shape and load mode (-1: not forced)
  int tile_tx = 0, tile_ty = 0, tile_pb = 0, tile_mode = -1;
  // set by a TMA-staged evaluation whose bounded barrier wait ran out
  // (mapped pinned host word and its device address)
  int *wait_err_h = nullptr, *wait_err_d = nullptr;
  // test hook for the next mode-4 launch (einspline_gb300_test_wait_timeout):
  // the stage block 0 leaves without copies, plus one (0: off), and the
  // launch's wait limit
  std::atomic<int> test_skip{0};
  unsigned long long test_wait_ns = 0;
  int tuned_tx[2] = {0, 0}, tuned_ty[2] = {0, 0}, tuned_pb[2] = {0, 0}, tuned_mode[2] = {0, 0};
  // the same for launches that visit points in cell order (sorted batches)
  int tuned_s_tx[2] = {0, 0}, tuned_s_ty[2] = {0, 0}, tuned_s_pb[2] = {0, 0}, tuned_s_mode[2] = {0, 0};
};

namespace eg {

using Table = einspline_gb300_table;

struct GridDesc {
  double start, end;
  int num;
  int lcode, rcode;
  double lval[2], rval[2];
};

// Creates a table object with its device storage (zero-filled).  Only the
// first dims entries of g are read.
Table *table_create(char kind, const GridDesc g[3], int num_splines, int storage, int dims = 3);
void table_destroy(Table *t);
// Copy of src converted to another storage (device to device), with new
// private storage; used by the *_cuda creators.
Table *table_clone(Table *src, int storage);
// Queue set calls; data on host (from_device=0) or device.
int table_set(Table *t, int first, int count, const void *data, bool from_device);
// One spline of a 1D table solved with its own x boundary condition
// (set_multi_UBspline_1d_{d,z}_BC); host data.
int table_set_bc(Table *t, int spline, const void *data, int lcode, int rcode, const double lval[2],
                 const double rval[2]);
int table_flush(Table *t);
// Rebuilds the double-float shadow of an FP64 table when fp64_mode is 1 and
// the table changed since it was made.
int table_df_refresh(Table *t);
inline bool table_ok(const Table *t) { return t && t->magic == kMagic; }
// A 3D table: what every 3D entry point and extension takes.
inline bool table3_ok(const Table *t) { return table_ok(t) && t->dims == 3; }

// ---------------------------------------------------------------- eval
struct EvalArgs {
  const void *coefs;
  const float *scale;
  int64_t xs, ys, zs;         // stored reals
  int ncol;                   // real columns to evaluate
  int ncol_pad;
  int lim[3];                 // largest first-cell index per axis (N-4)
  double start[3], dinv[3];
  float dinvf[3];
  const void *pos;            // device positions (or null: inline)
  double inl[3];              // inline position for the single-point entry
  int pos_f64;
  int rule;                   // 0 CPU-entry rule, 1 reference GPU rule
  const int *perm;            // optional visiting order
  int64_t npts;
  // outputs: pointer arrays (per point) or flat bases with strides
  void *const *vals_pp;
  void *const *grads_pp;
  void *const *hess_pp;
  void *vals, *grads, *hess;
  void *ghess;                // vghgh: third derivatives [N][27] (CPU layout)
  int64_t vstride, gstride, hstride;
  int layout;                 // 0 GPU layout, 1 CPU layout
  int is_complex;
  int ntiles;                 // column tiles per point group
  int pb;                     // points per block (shared-memory layout)
  int pb_tail;                // > 0: point groups from g_tail on hold pb_tail points
  int64_t g_tail;             //      (shorter blocks for the launch's last wave)
  int mode;                   // load mode: 0 direct loads, 1 L2 bulk prefetch first,
                              // 2/3 shared-memory pipeline of async copies,
                              // 4 shared-memory pipeline of tensor-map (TMA) copies
  int out;                    // 0 vgh; 1 vgl with lattice transform (GPU entries):
                              // 4 rows G.grad and Tr(G^T G H) at lrow apart in gl_pp;
                              // 2 vgl (CPU entries): grads and lapl = trace(H) in hess;
                              // 3 vg: value and gradient only
  const void *sign;           // optional per-point factor (output type) on every output
  int unscaled;               // 1D/2D kernels: derivatives in cell units (no delta_inv),
                              // as the reference's 1D GPU vgl kernels return them
  const void *linv;           // out 1: 3x3 row-major G (output type)
  int64_t lrow;               // out 1: row stride of the gradient/laplacian rows (reals)
  int *wait_err;              // mode 4: set to 1 when a bounded barrier wait ran out
  unsigned long long wait_ns; // mode 4: limit of each bounded wait (0: kWaitNs, 0.5 s)
  int test_skip;              // mode 4 test hook: s + 1 makes block 0 issue no copy for
                              // its stage s, so that stage's wait runs out (0: off)
  int box_bytes;              // mode 4: bytes of one box row (<= 256 stored reals)
  // mode 4: the table as a 4D tensor [x][y][z][column] (column innermost);
  // CUtensorMap is 128-byte aligned, and so is EvalArgs
  CUtensorMap tmap;
};

// mode >= 0 forces a load mode (EvalArgs::mode) instead of the table's choice.
int launch_eval(Table *t, EvalArgs &a, bool vgh, cudaStream_t s, int tx, int ty, int pb, int mode = -1);
// One point of a single-point entry (a.npts = 1, outputs in the point scratch).
int launch_point(Table *t, EvalArgs &a, bool vgh);
// ETIMEOUT (and clears the word) when a TMA-staged evaluation on t gave up a
// bounded wait since the last check; call after the launches completed.
int wait_status(Table *t, const char *fn);
// Mapped pinned output scratch of the single-point entries (40 * ncol reals).
int point_scratch(Table *t, const char *fn);
void fill_eval_geometry(const Table *t, EvalArgs &a);
// Kernel, grid, block and shared memory of a launch without launching it
// (for graph kernel nodes); fills a.pb and a.ntiles.
int prepare_eval(Table *t, EvalArgs &a, bool vgh, int tx, int ty, int pb, const void **func, dim3 *grid,
                 dim3 *block, size_t *smem);
// sorted: the launch visits its points in cell order (a visiting order is
// set), which has its own tuned shape.
void pick_tile(Table *t, bool vgh, int64_t npts, int &tx, int &ty, int &pb, bool sorted = false);
// Load mode of launches on this table (see EvalArgs::mode).
int pick_mode(Table *t, bool vgh, bool sorted = false);
// Tensor map of a 16-bit table for the tensor-core kernels (load mode 5).
int tc_table_map(const Table *t, EvalArgs &a);
int elems_per_thread(const Table *t);

// sorting
int sort_points(Table *t, const EvalArgs &a, int **perm_out, cudaStream_t s);
// The counting sort of batches of up to kSmallSort points into caller-given
// scratch of small_sort_bytes(npts) bytes (16-byte aligned; nothing in it
// has to start at zero).
constexpr int64_t kSmallSort = 131072;
size_t small_sort_bytes(int64_t n);
int small_sort_into(const EvalArgs &a, void *scratch, int **perm_out, cudaStream_t s);
// Morton key of each point's cell and its index (defined in api_ext.cu).
__global__ void k_cell_keys(const EvalArgs a, uint64_t *keys, int *idx);
// Bring kernels' code to the current device now rather than at their first
// launch (CUDA loads modules lazily by default): the sort kernels, and the
// evaluation kernel that a launch on t with these options would use.
int load_sort_kernels();
int load_eval_kernel(Table *t, bool vgh, bool sorted);

}  // namespace eg
