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
  EINSPLINE_GB300_STORE_F16 = 2,    /* IEEE half, power-of-two scale per spline */
  EINSPLINE_GB300_STORE_BF16 = 3,   /* bfloat16, power-of-two scale per spline  */
  EINSPLINE_GB300_STORE_F64 = 4
};

/* create_multi_UBspline_3d_{s,c} with a chosen table storage (s/c only:
 * NATIVE, F32, F16 or BF16).  The FP64 solve result of each spline is scaled
 * by a power of two so its largest coefficient lies in [2^14, 2^15), rounded
 * once to the storage type, and evaluation multiplies the scale back. */
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
  const float *scale;  /* device, per real column (F16/BF16), else NULL */
} einspline_gb300_table_info;
int einspline_gb300_get_table_info(einspline_gb300_table *t, einspline_gb300_table_info *out);
/* Copy the stored table (padded layout, storage type) to host memory of
 * table_bytes bytes; the scales (ncol floats) too when scale_host != NULL. */
int einspline_gb300_copy_table(einspline_gb300_table *t, void *host_dst, float *scale_host);

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
                     results are bit-identical to sort = 0                    */
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

/* Launch shape: tx threads along the spline axis (multiple of 32), ty point
 * lanes per block, pb points per block.  0,0,0 restores the default. */
int einspline_gb300_set_tile(einspline_gb300_table *t, int tx, int ty, int pb);
int einspline_gb300_get_tile(einspline_gb300_table *t, int *tx, int *ty, int *pb);
/* Time every candidate tile on this table for npts random points and keep
 * the fastest (for vgh when vgh != 0); the choice is cached per table. */
int einspline_gb300_autotune(einspline_gb300_table *t, int64_t npts, int vgh);

/* Kernel launches this library issued on the calling thread so far. */
int64_t einspline_gb300_launch_count(void);

/* Fill a device array with the splitmix64 uniform stream used by the
 * tests and benchmark: dst[i] = lo + (hi-lo) * u(seed, offset + i). */
int einspline_gb300_fill_uniform(void *dst_d, int64_t n, int f64, uint64_t seed, int64_t offset,
                                 double lo, double hi, void *stream);

#ifdef __cplusplus
}
#endif

#endif
