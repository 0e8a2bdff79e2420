/*
 * multi_bspline_eval_cuda.h -- batched multi-point evaluation on the GPU.
 *
 * Replaces the 1D value and vgl entries and the 3D value, sign, vgh and vgl
 * entries of src/multi_bspline_eval_cuda.h:12-137
 * (kernels and launchers in src/multi_bspline_cuda_{s,d,c,z}_impl.h).
 * Same arguments and meaning:
 *   pos_d   device array of num points, xyz interleaved (float for s/c,
 *           double for d/z), measured from the grid origin: the cell of
 *           coordinate r is clamp(floor(r * gridInv), 0, dim-1), exactly the
 *           reference's rule (src/multi_bspline_cuda_s_impl.h:370-384)
 *   vals_d  device array of num device pointers; point i writes N values
 *           (complex: N complex) at vals_d[i]
 *   grads_d point i writes [N][3] at grads_d[i]; complex: [N][re,im][3] floats
 *   hess_d  point i writes [N][6] (xx, xy, xz, yy, yz, zz) at hess_d[i];
 *           complex: [N][re,im][6]
 * Calls run on the legacy default stream and return when the results are
 * ready, as the reference's did.  num has no 65,535 limit here.  On a CUDA
 * error the call reports through einspline_gb300_last_error() and, in the
 * default mode, prints and aborts like the reference.
 */
#ifndef EINSPLINE_GB300_MULTI_BSPLINE_EVAL_CUDA_H
#define EINSPLINE_GB300_MULTI_BSPLINE_EVAL_CUDA_H

#include "multi_bspline_structs_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- 1D (src/multi_bspline_eval_cuda.h:12-55; the reference implements s
 * and c, src/multi_bspline_cuda_s_impl.h:10-175, src/multi_bspline_cuda_c_impl.h:9-175).
 * pos_d holds one coordinate per point; vals_d, grads_d and lapl_d are
 * device arrays of num device pointers, each to N reals (2N for complex,
 * re/im interleaved).  As in the reference's kernels, the gradient and
 * second derivative are taken with respect to the cell coordinate
 * u = r * gridInv: they are NOT multiplied by gridInv and gridInv^2
 * (multiply them yourself for derivatives in position units).  The
 * reference leaves grads/lapl of the last N mod 64 columns unwritten; here
 * every column is written. */
void eval_multi_multi_UBspline_1d_s_cuda(multi_UBspline_1d_s_cuda *spline, float *pos_d, float *vals_d[], int num);
void eval_multi_multi_UBspline_1d_s_vgl_cuda(multi_UBspline_1d_s_cuda *spline, float *pos_d, float *vals_d[],
                                             float *grads_d[], float *lapl_d[], int num);
void eval_multi_multi_UBspline_1d_d_cuda(multi_UBspline_1d_d_cuda *spline, double *pos_d, double *vals_d[],
                                         int num);
void eval_multi_multi_UBspline_1d_d_vgl_cuda(multi_UBspline_1d_d_cuda *spline, double *pos_d, double *vals_d[],
                                             double *grads_d[], double *lapl_d[], int num);
void eval_multi_multi_UBspline_1d_c_cuda(multi_UBspline_1d_c_cuda *spline, float *pos_d, complex_float *vals_d[],
                                         int num);
void eval_multi_multi_UBspline_1d_c_vgl_cuda(multi_UBspline_1d_c_cuda *spline, float *pos_d,
                                             complex_float *vals_d[], complex_float *grads_d[],
                                             complex_float *lapl_d[], int num);
void eval_multi_multi_UBspline_1d_z_cuda(multi_UBspline_1d_z_cuda *spline, double *pos_d, complex_double *vals_d[],
                                         int num);
void eval_multi_multi_UBspline_1d_z_vgl_cuda(multi_UBspline_1d_z_cuda *spline, double *pos_d,
                                             complex_double *vals_d[], complex_double *grads_d[],
                                             complex_double *lapl_d[], int num);

/* ---- 3D */
/* src/multi_bspline_eval_cuda.h:62-64; src/multi_bspline_cuda_s_impl.h:488 */
void eval_multi_multi_UBspline_3d_s_cuda(multi_UBspline_3d_s_cuda *spline, float *pos_d,
                                         float *vals_d[], int num);
/* src/multi_bspline_eval_cuda.h:71-74; src/multi_bspline_cuda_s_impl.h:542 */
void eval_multi_multi_UBspline_3d_s_vgh_cuda(multi_UBspline_3d_s_cuda *spline, float *pos_d,
                                             float *vals_d[], float *grads_d[], float *hess_d[],
                                             int num);

/* src/multi_bspline_eval_cuda.h:67-68; src/multi_bspline_cuda_s_impl.h:515: values times
 * a per-point factor sign_d[i] (device array of num floats). */
void eval_multi_multi_UBspline_3d_s_sign_cuda(multi_UBspline_3d_s_cuda *spline, float *pos_d, float *sign_d,
                                              float *vals_d[], int num);
/* src/multi_bspline_eval_cuda.h:77-79; src/multi_bspline_cuda_s_impl.h:566-760: value, and
 * four rows at grad_lapl_d[i] + r*row_stride: G.grad (r = 0,1,2) and the laplacian
 * Tr(G^T G H) (r = 3), with G = Linv_d (device, 3x3 row-major). */
void eval_multi_multi_UBspline_3d_s_vgl_cuda(multi_UBspline_3d_s_cuda *spline, float *pos_d, float *Linv_d,
                                             float *vals_d[], float *grad_lapl_d[], int num, int row_stride);
/* src/multi_bspline_eval_cuda.h:82-84; src/multi_bspline_cuda_s_impl.h:763-933: vgl times
 * the per-point factor sign_d[i]. */
void eval_multi_multi_UBspline_3d_s_vgl_sign_cuda(multi_UBspline_3d_s_cuda *spline, float *pos_d, float *sign_d,
                                                  float *Linv_d, float *vals_d[], float *grad_lapl_d[], int num,
                                                  int row_stride);

/* src/multi_bspline_eval_cuda.h:89-91; src/multi_bspline_cuda_d_impl.h:229 */
void eval_multi_multi_UBspline_3d_d_cuda(multi_UBspline_3d_d_cuda *spline, double *pos_d,
                                         double *vals_d[], int num);
/* src/multi_bspline_eval_cuda.h:93-96; src/multi_bspline_cuda_d_impl.h:254 */
void eval_multi_multi_UBspline_3d_d_vgh_cuda(multi_UBspline_3d_d_cuda *spline, double *pos_d,
                                             double *vals_d[], double *grads_d[],
                                             double *hess_d[], int num);

/* src/multi_bspline_eval_cuda.h:99-101; src/multi_bspline_cuda_d_impl.h:278-452 */
void eval_multi_multi_UBspline_3d_d_vgl_cuda(multi_UBspline_3d_d_cuda *spline, double *pos_d, double *Linv_d,
                                             double *vals_d[], double *grad_lapl_d[], int num, int row_stride);

/* src/multi_bspline_eval_cuda.h:105-108; src/multi_bspline_cuda_c_impl.h:417 */
void eval_multi_multi_UBspline_3d_c_cuda(multi_UBspline_3d_c_cuda *spline, float *pos_d,
                                         complex_float *vals_d[], int num);
/* src/multi_bspline_eval_cuda.h:110-114; src/multi_bspline_cuda_c_impl.h:442 */
void eval_multi_multi_UBspline_3d_c_vgh_cuda(multi_UBspline_3d_c_cuda *spline, float *pos_d,
                                             complex_float *vals_d[], complex_float *grads_d[],
                                             complex_float *hess_d[], int num);

/* src/multi_bspline_eval_cuda.h:117-119; src/multi_bspline_cuda_c_impl.h:467-660: rows are
 * row_stride complex values apart. */
void eval_multi_multi_UBspline_3d_c_vgl_cuda(multi_UBspline_3d_c_cuda *spline, float *pos_d, float *Linv_d,
                                             complex_float *vals_d[], complex_float *grad_lapl_d[], int num,
                                             int row_stride);

/* src/multi_bspline_eval_cuda.h:123-126; src/multi_bspline_cuda_z_impl.h:233 */
void eval_multi_multi_UBspline_3d_z_cuda(multi_UBspline_3d_z_cuda *spline, double *pos_d,
                                         complex_double *vals_d[], int num);
/* src/multi_bspline_eval_cuda.h:128-132; src/multi_bspline_cuda_z_impl.h:259 */
void eval_multi_multi_UBspline_3d_z_vgh_cuda(multi_UBspline_3d_z_cuda *spline, double *pos_d,
                                             complex_double *vals_d[], complex_double *grads_d[],
                                             complex_double *hess_d[], int num);

/* src/multi_bspline_eval_cuda.h:135-137; src/multi_bspline_cuda_z_impl.h:284-458 */
void eval_multi_multi_UBspline_3d_z_vgl_cuda(multi_UBspline_3d_z_cuda *spline, double *pos_d, double *Linv_d,
                                             complex_double *vals_d[], complex_double *grad_lapl_d[], int num,
                                             int row_stride);

#ifdef __cplusplus
}
#endif

#endif
