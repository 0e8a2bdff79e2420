/*
 * einspline_gb300.h -- additions to the einspline API for the GB300 library.
 *
 * The drop-in entry points (create/set/eval and the *_cuda batched calls) are
 * declared in the reference-named headers next to this one.  This header adds
 * what a GPU-resident library needs and the reference has no counterpart for:
 * error status instead of abort(), a choice of table storage (FP32, or
 * FP16/BF16 with a per-spline scale), batched evaluation into flat device
 * buffers on a caller's stream, cell-sorted evaluation, a host-buffer entry
 * that pipelines copies with compute, tile tuning, and a request server.
 *
 * Every object here is reached through the table handle that each spline
 * struct carries in its appended field: spline->gb300.
 */
#ifndef EINSPLINE_GB300_H
#define EINSPLINE_GB300_H

#include <stdint.h>
#include "multi_bspline.h"
#include "multi_bspline_structs_cuda.h"
#include "multi_bspline_create_cuda.h"
#include "multi_bspline_eval_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct einspline_gb300_table einspline_gb300_table;

/* ---------------------------------------------------------------- errors */
/* Status codes.  The reference returns void and aborts on any error
 * (src/multi_bspline_cuda_s_impl.h:556-562); here every call also leaves a
 * thread-local status behind. */
enum {
  EINSPLINE_GB300_OK = 0,
  EINSPLINE_GB300_EINVAL = 1,   /* bad argument                          */
  EINSPLINE_GB300_ENOMEM = 2,   /* host or device allocation failed      */
  EINSPLINE_GB300_ECUDA = 3,    /* a CUDA call failed                    */
  EINSPLINE_GB300_ESIZE = 4,    /* size beyond a stated limit            */
  EINSPLINE_GB300_EBUSY = 5,    /* server full / request not admitted    */
  EINSPLINE_GB300_ETIMEOUT = 6  /* a bounded wait ran out                */
};
int einspline_gb300_last_error(void);
const char *einspline_gb300_last_error_message(void);
void einspline_gb300_clear_error(void);
/* 1 (default): print and abort() on error, as the reference does.
 * 0: return with the status set (void entry points just return). */
void einspline_gb300_set_abort_on_error(int enable);

/* --------------------------------------------------------------- storage */
enum {
  EINSPLINE_GB300_STORE_NATIVE = 0, /* FP32 for s/c, FP64 for d/z */
  EINSPLINE_GB300_STORE_F32 = 1,
  EINSPLINE_GB300_STORE_F16 = 2,    /* IEEE half with a scale per spline        */
  EINSPLINE_GB300_STORE_BF16 = 3,   /* bfloat16 with a power-of-two scale      */
  EINSPLINE_GB300_STORE_F64 = 4,
  EINSPLINE_GB300_STORE_I16 = 5     /* 16-bit fixed point with a scale per spline */
};

/* create_multi_UBspline_3d_{s,c} with a chosen table storage (s/c only:
 * NATIVE, F32, F16, BF16 or I16).  The FP64 solve result of each spline is
 * multiplied by a per-spline factor and rounded once to the storage type;
 * evaluation multiplies the inverse back after the FP32 reduction.
 *   F16: the largest |coefficient| maps to just under 65504 (full half range);
 *   I16: coefficients map to integers in [-32767, 32767] (uniform step
 *        max|c|/32767, the smallest absolute error of the 16-bit formats);
 *   BF16: a power of two puts the largest |coefficient| in [2^14, 2^15).
 * For complex splines the real and imaginary parts share one factor. */
multi_UBspline_3d_s *einspline_gb300_create_3d_s(Ugrid x_grid, Ugrid y_grid, Ugrid z_grid,
                                                 BCtype_s xBC, BCtype_s yBC, BCtype_s zBC,
                                                 int num_splines, int storage);
multi_UBspline_3d_c *einspline_gb300_create_3d_c(Ugrid x_grid, Ugrid y_grid, Ugrid z_grid,
                                                 BCtype_c xBC, BCtype_c yBC, BCtype_c zBC,
                                                 int num_splines, int storage);

/* A device copy of a table in another storage: an FP64 d table to s storage
 * (F32/F16/BF16) or a z table to c storage, rounded once from FP64. */
multi_UBspline_3d_s_cuda *einspline_gb300_create_3d_s_cuda_from_d(multi_UBspline_3d_d *spline,
                                                                  int storage);
multi_UBspline_3d_c_cuda *einspline_gb300_create_3d_c_cuda_from_z(multi_UBspline_3d_z *spline,
                                                                  int storage);

/* Bulk set_multi_UBspline_3d_*: count splines first..first+count-1 from a
 * DEVICE array [count][Mx][My][Mz] of the value type (float for s/c, double
 * for d/z; complex interleaved).  Queued like set_*; data_d may be reused
 * once the call returns. */
int einspline_gb300_set_3d_device(einspline_gb300_table *t, int first, int count, const void *data_d);
/* Solve every queued spline now. */
int einspline_gb300_flush(einspline_gb300_table *t);

typedef struct {
  int kind;            /* 's', 'd', 'c' or 'z' */
  int storage;         /* EINSPLINE_GB300_STORE_* actually used */
  int num_splines;
  int ncol;            /* real columns: num_splines (x2 for complex) */
  int ncol_pad;        /* real columns per table row, padded to 128 bytes */
  int elem_bytes;      /* bytes per stored real */
  int nx, ny, nz;      /* coefficients per axis */
  int64_t x_stride, y_stride, z_stride; /* in stored reals */
  uint64_t table_bytes;
  const void *coefs;   /* device */
  const float *scale;  /* device, per real column (16-bit storage), else NULL */
} einspline_gb300_table_info;
int einspline_gb300_get_table_info(einspline_gb300_table *t, einspline_gb300_table_info *out);
/* Copy the stored table (padded layout, storage type) to host memory of
 * table_bytes bytes; the scales (ncol floats) too when scale_host != NULL. */
int einspline_gb300_copy_table(einspline_gb300_table *t, void *host_dst, float *scale_host);
/* For callers that read or write spline->coefs on the host, as the
 * reference's host table allows (src/multi_bspline_structs.h:155-164: coefs
 * is host memory there; checkpoint reads and writes, broadcasts): a pinned
 * host mirror of the coefficients in the reference's layout and value type
 * (float for s/c, double for d/z; the struct's x/y/z strides apply),
 * refreshed from the device table by each call (16-bit tables dequantised);
 * *coefs_out may be stored in spline->coefs for such code.  After host
 * edits, push_host_coefs uploads the mirror into the device table (FP32 and
 * FP64 storage; EINVAL for 16-bit tables, which set_* builds from data);
 * evaluation always reads the device table.  The mirror lives until
 * release_host_coefs or the spline's destruction. */
int einspline_gb300_host_coefs(einspline_gb300_table *t, void **coefs_out);
int einspline_gb300_push_host_coefs(einspline_gb300_table *t);
int einspline_gb300_release_host_coefs(einspline_gb300_table *t);

/* ------------------------------------------------------------ evaluation */
typedef struct {
  int vgh;        /* 1: value + gradient + Hessian; 0: value only            */
  int pos_f64;    /* positions are double (1) or float (0), xyz interleaved   */
  int rule;       /* 0: CPU-entry rule ((x-start)*delta_inv, modf, edge cells
                     extrapolated); 1: the reference GPU-entry rule
                     (x*delta_inv, floor, cell clamped)                       */
  int layout;     /* 0: GPU layout -- hess [N][6] (xx,xy,xz,yy,yz,zz), complex
                     grads [N][re,im][3]; 1: CPU layout -- hess [N][3][3],
                     complex grads [N][3][re,im]                              */
  int sort;       /* 1: visit points in cell (Morton) order for L2 reuse; the
                     results are bit-identical to sort = 0.  The ordering
                     uses the table's sort scratch: sorted calls on one
                     table on different streams must not overlap          */
  int64_t vstride, gstride, hstride; /* per-point output strides in output
                     reals (float for s/c, double for d/z); 0 = packed       */
} einspline_gb300_eval_opts;

/* Evaluate npts points, inputs and outputs in DEVICE memory, on a CUDA
 * stream (NULL = legacy default stream); returns without synchronizing.
 * Output reals are float for s/c tables (any storage) and double for d/z. */
int einspline_gb300_eval_3d(einspline_gb300_table *t, const einspline_gb300_eval_opts *opts,
                            int64_t npts, const void *pos_d, void *vals_d, void *grads_d,
                            void *hess_d, void *stream);

/* The same with HOST buffers (pinned memory recommended): positions are
 * copied in and results copied out in chunks on two streams so copies
 * overlap compute.  Returns when the outputs are in host memory. */
int einspline_gb300_eval_3d_host(einspline_gb300_table *t, const einspline_gb300_eval_opts *opts,
                                 int64_t npts, const void *pos_h, void *vals_h, void *grads_h,
                                 void *hess_h);
/* 0 (default, also -1): copy through device memory as above.  1: the
 * kernel reads positions from and writes results into the host buffers
 * directly; every buffer must be pinned and mapped into the device's address
 * space (cudaHostAlloc / cudaMallocHost memory).  Measured on GB300: 1.3 G
 * vgh evals/s direct against 4.5 G with the copy pipeline (whose 191 GB/s
 * device-to-host copies are the limit). */
int einspline_gb300_set_host_direct(einspline_gb300_table *t, int mode);

/* Cell-sorted evaluation (as einspline_gb300_eval_3d with opts->sort = 1,
 * whose sort scratch is allocated with cudaMalloc) that allocates nothing.
 * No counterpart in the reference.  For callers that cannot let a library
 * allocate device memory while they run -- a driver whose pool allocator owns
 * the device's memory, or code that must not trigger the device-wide
 * synchronisation cudaMalloc/cudaFree may cause.  The sort scratch is a fixed
 * 10 MiB file-scope device array that every GPU loading the library holds
 * until the process exits; npts above 262,144 is refused with ESIZE.  The
 * first call on a device (per CUDA context) is its set-up: it looks the
 * array's device address up (cudaGetSymbolAddress) and loads this entry's
 * kernels.  CUDA loads modules lazily by default, so this first call is when
 * the 10 MiB array and the kernels' code take device memory: make it before
 * a pool allocator takes the device's free memory, and before any stream
 * capture.  An empty call (npts = 0) with the table and options of later
 * calls does the whole set-up and nothing else.  A call may synchronise the
 * table's stream when set_* calls are still queued (their solve runs
 * first); an FP64 table in double-float mode whose double-float copy is
 * missing is refused (ENOMEM) rather than given one.  All calls share the
 * array: calls that overlap on the GPU (different streams or threads
 * without ordering between them) race and must be serialised.  Results are
 * bit-identical to einspline_gb300_eval_3d with sorting. */
int einspline_gb300_eval_3d_sorted_noalloc(einspline_gb300_table *t, const einspline_gb300_eval_opts *opts,
                                           int64_t npts, const void *pos_d, void *vals_d, void *grads_d,
                                           void *hess_d, void *stream);

/* Launch shape: tx threads along the spline axis (multiple of 32), ty point
 * lanes per block, pb points per block.  0,0,0 restores the default. */
int einspline_gb300_set_tile(einspline_gb300_table *t, int tx, int ty, int pb);
int einspline_gb300_get_tile(einspline_gb300_table *t, int *tx, int *ty, int *pb);
/* How the kernel brings stencil rows in:
 *   0: direct 16/8-byte loads into registers;
 *   1: each block first bulk-prefetches the rows of all its points into L2
 *      (more DRAM requests in flight without holding registers);
 *   2: a three-stage pipeline of asynchronous copies into shared memory
 *      (FP32 and 16-bit tables; one point lane per block);
 *   3: as 2 with 8 columns and one 16-byte copy per thread and row (16-bit
 *      tables; others use 2);
 *   4: a three-stage shared-memory pipeline fed by tensor-map (TMA) copies:
 *      one copy brings the 4x4 stencil rows of a point's x-plane for the
 *      whole block, completion is tracked by mbarriers; 8 columns a thread
 *      for 16-bit tables, 4 for FP32, 2 for double-float (IEEE FP64 uses 0);
 *   5: F16 and BF16 tables: the reduction runs on the tensor cores (tcgen05.mma):
 *      a block owns 256 columns, one TMA copy per 64 columns brings a
 *      point's whole 4x4x4 stencil in the MMA operand layout, and
 *      the point's weights, split into f16 high and low parts (bf16 high,
 *      middle and low parts for BF16 tables), are the other operand; FP32
 *      accumulation in tensor memory.  Results agree with the
 *      other modes to FP32 rounding, not bit for bit.  It is the default of
 *      vgh on F16 and BF16 tables, whose vgh autotuning only tunes its
 *      points per block, so tuning changes no result.  Other tables, and
 *      complex tables in the CPU layout, use their pipeline (3 or 2) instead;
 *  -1: the autotuned choice; untuned, vgh uses 5 for F16 and BF16 tables, 3
 *      for I16 tables and 2 for FP32 (the choices the autotuner makes on
 *      GB300); value-only uses 3 for 16-bit tables and 0 for FP32; FP64
 *      uses 0.  Results are identical in modes 0-4, and within mode 5. */
int einspline_gb300_set_load_mode(einspline_gb300_table *t, int mode);
int einspline_gb300_get_load_mode(einspline_gb300_table *t);
/* Every wait of the mode-4 and mode-5 kernels on their mbarriers is bounded (0.5 s);
 * one that runs out makes the block stop early and sets a word that this
 * call reads and clears: EINSPLINE_GB300_ETIMEOUT when some launch on t since
 * the last check gave up (its results are incomplete), else 0.  Call it
 * after the launches have completed (synchronised stream).  The blocking
 * entries (single-point, host-buffer) check it themselves. */
int einspline_gb300_wait_status(einspline_gb300_table *t);
/* Testing the bounded waits without a fault: the next mode-4 or mode-5 launch
 * on t (an evaluation, or a determinant ratio on the tensor cores) has its
 * first block issue no copy for its stage `stage` (stages count a block's
 * point x-planes from 0 in mode 4, its points or walkers in mode 5), and every
 * wait of that launch gives up
 * after `seconds` (1 us .. 1 s) instead of 0.5 s.  That stage's barrier
 * then never completes, its wait runs out, the block stops early and the
 * launch reports ETIMEOUT through einspline_gb300_wait_status; no copy is
 * left in flight and the next launch is unaffected.  Applies to one launch
 * only; stage < 0 cancels it.  No counterpart in the reference, which
 * aborts on a CUDA error instead. */
int einspline_gb300_test_wait_timeout(einspline_gb300_table *t, int stage, double seconds);
/* Time every candidate tile in every load mode on this table for npts
 * random points and keep the fastest (for vgh when vgh != 0); the choice is
 * cached per table. */
int einspline_gb300_autotune(einspline_gb300_table *t, int64_t npts, int vgh);
/* The same for launches that visit their points in cell order (opts.sort,
 * the allocation-free sorted entry): npts random points are sorted by cell
 * and the shapes are timed on a window of up to 32,768 consecutive sorted
 * points, so a batch's density (npts per grid cell) is what is tuned for.
 * Sorted launches then use this choice; set_tile / set_load_mode still
 * override both; get_tile and get_load_mode report the random-order one. */
int einspline_gb300_autotune_sorted(einspline_gb300_table *t, int64_t npts, int vgh);
/* The tile and load mode a launch takes (random order or cell-sorted, vgh
 * or value-only), after set_tile / set_load_mode, tuning and defaults. */
int einspline_gb300_get_launch_shape(einspline_gb300_table *t, int sorted, int vgh, int *tx, int *ty, int *pb,
                                     int *mode);

/* --------------------------------------------------------------- serving */
/* A request server over one table: QMC-walker-shaped requests (a set of
 * points each) arrive at any time; a worker thread admits them while their
 * outputs fit in a device-memory budget, packs admitted requests into
 * batches and keeps several batches in flight on separate streams, each
 * launched through a CUDA graph.  Requests that arrive while others are on
 * the GPU join the next batch as slots and memory free up.  A request's
 * outputs stay in device memory until it is released.  Every point is
 * computed independently in a fixed order, so a request's results are
 * bit-identical alone and in any mix. */
typedef struct einspline_gb300_server einspline_gb300_server;
typedef struct {
  int vgh;                   /* 1: value+gradient+Hessian (default), 0: value */
  int pos_f64;               /* positions are double (1) or float (0) */
  int rule;                  /* cell rule, as einspline_gb300_eval_opts.rule */
  int use_graphs;            /* 1: launch batches through CUDA graphs */
  int max_inflight;          /* batches on the GPU at once (1..8), default 3 */
  int max_batch_points;      /* points per batch, default 16384; also the
                                largest request accepted */
  uint64_t hbm_budget_bytes; /* device memory for request outputs; 0 = 4 GiB
                                or half of the free memory, whichever is less */
  int sort;                  /* 1: visit each batch's points in cell order (a
                                counting sort per batch, in scratch of each
                                slot; batches are then launched without
                                graphs; max_batch_points <= 131072); results
                                are bit-identical to sort = 0 */
} einspline_gb300_server_opts;

/* Output layout per request: vals [npts][N], grads [npts][N][3],
 * hess [npts][N][6] (GPU layout; complex as float/double pairs per entry). */
einspline_gb300_server *einspline_gb300_server_create(einspline_gb300_table *t,
                                                      const einspline_gb300_server_opts *opts);
int einspline_gb300_server_destroy(einspline_gb300_server *s);
/* Queue a request (positions copied from host memory); returns its id >= 0,
 * or -1 with the status set (ESIZE when it can never fit). */
int64_t einspline_gb300_server_submit(einspline_gb300_server *s, const void *pos_host, int npts);
/* Wait up to timeout_s seconds for a request; 0 when done, ETIMEOUT else. */
int einspline_gb300_server_wait(einspline_gb300_server *s, int64_t id, double timeout_s);
/* Device addresses of a finished request's outputs and its latency
 * (submit to results ready, seconds). */
int einspline_gb300_server_result(einspline_gb300_server *s, int64_t id, void **vals_d, void **grads_d,
                                  void **hess_d, double *latency_s);
/* Copy a finished request's outputs to host memory (any may be NULL). */
int einspline_gb300_server_copy_result(einspline_gb300_server *s, int64_t id, void *vals_h, void *grads_h,
                                       void *hess_h);
/* Give a finished request's device memory back (admits waiting requests). */
int einspline_gb300_server_release(einspline_gb300_server *s, int64_t id);

typedef struct {
  int64_t submitted, completed, released, batches;
  int64_t evals;              /* (point, spline) pairs computed */
  uint64_t budget_bytes, peak_bytes_in_use;
  int peak_inflight;          /* most batches seen on the GPU at once */
  double busy_seconds;        /* first launch to last completion */
} einspline_gb300_server_stats;
int einspline_gb300_server_get_stats(einspline_gb300_server *s, einspline_gb300_server_stats *out);

/* Replay an open-loop arrival trace natively: request i (npts[i] points at
 * pos_host + offsets[i] positions) is submitted at arrival_s[i] seconds after
 * the call starts, released as soon as it completes, and its latency (submit
 * to results ready) stored in latency_s[i].  Returns when all are done. */
int einspline_gb300_server_replay(einspline_gb300_server *s, int nreq, const double *arrival_s,
                                  const int *npts, const int64_t *offsets, const void *pos_host,
                                  double *latency_s, double *wall_s);

/* ------------------------------------------------- QMC determinant step
 * The consumer of the orbital row in the reference's QMC prototype
 * (src/cuda_walker.cu): every walker moves electron k; the N orbitals are
 * evaluated at its new position (calc_new_row, :69-88), dotted with column k
 * of the walker's inverse Slater matrix (calc_ratios, :171-201) and, when the
 * move is accepted, the inverse gets a Sherman-Morrison update
 * (update_inverse_cuda1/2, src/determinant_update.h:9-111, launched at
 * src/cuda_walker.cu:92-136).  No single reference entry point corresponds:
 * these replace that kernel sequence.  Real float tables only (s kind, any
 * float or 16-bit storage); A and Ainv are float. */
typedef struct {
  int nelec;       /* N: determinant size, orbitals 0..N-1 of the table      */
  int k;           /* the moved electron: row k of A, column k of Ainv       */
  int ld;          /* leading dimension of every A and Ainv, floats (>= N)   */
  int ainv_trans;  /* 0: Ainv[j*ld + e] (orbital j, electron e), the
                      reference's layout, column k strided in memory;
                      1: the transpose, Ainv[e*ld + j]: column k contiguous,
                      fewer bytes per ratio.  A is always A[e*ld + j].      */
  int pos_f64;     /* positions double (1) or float (0), xyz interleaved     */
  int rule;        /* cell rule, as in einspline_gb300_eval_opts             */
} einspline_gb300_det_opts;

/* For each of nwalkers walkers w (all buffers in device memory; ainv_d and
 * row_d are device arrays of device pointers, one per walker):
 *   ratio_d[w]    = sum_j phi_j(r_w) Ainv_w[j][k]
 *   grad_d[3w..]  = sum_j grad phi_j(r_w) Ainv_w[j][k] / ratio   (optional)
 *   lapl_d[w]     = sum_j lapl phi_j(r_w) Ainv_w[j][k] / ratio   (optional)
 *   row_d[w][j]   = phi_j(r_w), j < N                           (optional)
 * with r_w = pos_d[3w..3w+2].  The orbital values, gradients and Laplacians
 * are never written to memory (except the value row when row_d != NULL); the
 * row equals einspline_gb300_eval_3d's values bit for bit in the table's load
 * mode (F16 and BF16 tables default to the tensor-core mode 5, whose ratio
 * kernel is the tensor-core contraction too; modes 0-4 run the FMA
 * reduction; the two agree to FP32 rounding).  Sums run in a
 * fixed order, so results do not vary from run to run.  Bounded waits of
 * the tensor-core kernel report through einspline_gb300_wait_status.
 * Asynchronous on stream (NULL = legacy default stream). */
int einspline_gb300_det_ratio(einspline_gb300_table *t, const einspline_gb300_det_opts *opts, int nwalkers,
                              const void *pos_d, const float *const *ainv_d, float *ratio_d,
                              float *grad_d, float *lapl_d, float *const *row_d, void *stream);

/* Sherman-Morrison update of naccept walkers' inverses after row k of A is
 * replaced by row_d[w] (device pointer arrays, as above):
 *   x    = (u - A[k,:]) Ainv,   Ainv -= Ainv[:,k] x / (1 + x[k]),
 *   A[k,:] = u.
 * work_d: device scratch of 2 * nelec * naccept floats.  At most 65535
 * walkers per call.  Asynchronous on stream. */
int einspline_gb300_det_update(const einspline_gb300_det_opts *opts, int naccept, float *const *a_d,
                               float *const *ainv_d, const float *const *row_d, float *work_d, void *stream);

/* FP64 (d and z) tables: how evaluations compute.
 *   0 (default): IEEE FP64 fused multiply-adds.  On GB300 the FP64 pipe is a
 *     small fraction of the FP32 one, and this path is bound by it, far below
 *     the memory roofline.
 *   1: double-float arithmetic on the FP32 pipes: each coefficient and basis
 *     weight as an unevaluated sum of two floats (hi + lo, ~48 significant
 *     bits), error-free products by FMA residuals and two-sum accumulation;
 *     results within ~1e-14 relative of FP64 (tested to 1e-12 against the
 *     FP64 oracle).  Keeps a (hi, lo) copy of the table in device memory (the
 *     table's size again), rebuilt after set_* / flush.
 * Applies to every 3D evaluation of the table (flat, host-buffer, server,
 * single-point and *_cuda entries of a handle made from it take the handle's
 * own table: set the mode on c->gb300).  Not for 1D/2D tables.  A request
 * server captures the table's kernel in its graphs: set the mode before
 * creating one (changing it while a server exists fails with EBUSY). */
int einspline_gb300_set_fp64_mode(einspline_gb300_table *t, int mode);
int einspline_gb300_get_fp64_mode(einspline_gb300_table *t);

/* Kernel launches (and graph launches) this library has issued so far. */
int64_t einspline_gb300_launch_count(void);

/* Fill a device array with the splitmix64 uniform stream used by the
 * tests and benchmark: dst[i] = lo + (hi-lo) * u(seed, offset + i). */
int einspline_gb300_fill_uniform(void *dst_d, int64_t n, int f64, uint64_t seed, int64_t offset,
                                 double lo, double hi, void *stream);

#ifdef __cplusplus
}
#endif

#endif
