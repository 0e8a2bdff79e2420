/*
 * multi_bspline_eval_z.h -- single-point evaluation of a uniform 1D/2D/3D
 * multi-spline of type z (complex_double), host output buffers.
 *
 * Replaces the 3D value, vg, vgl and vgh entries of src/multi_bspline_eval_z.h:87-110
 * and the std backend's vghgh entry.
 * Output layout is the reference CPU layout: vals[N], grads[N][3],
 * hess[N][3][3] (full symmetric matrix, row-major).  The point may be given
 * anywhere; the reference reads outside its table when a point leaves
 * [start, end], this library extrapolates the edge cell instead.
 * Each call runs one GPU launch plus a device-to-host copy: for many points
 * use eval_multi_multi_UBspline_3d_z*_cuda or einspline_gb300_eval_3d.
 */
#ifndef EINSPLINE_GB300_MULTI_BSPLINE_EVAL_Z_H
#define EINSPLINE_GB300_MULTI_BSPLINE_EVAL_Z_H

#include "multi_bspline_structs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- 1D and 2D (src/multi_bspline_eval_z.h:29-77; std backend
 * src/multi_bspline_eval_std_z_impl.h).  1D: grads[N], lapl[N] and hess[N]
 * are first and second derivatives (the 1D vgh equals the vgl, as in the
 * reference).  2D: grads[N][2], lapl[N] = d2/dx2 + d2/dy2, hess[N][2][2]. */
void eval_multi_UBspline_1d_z(multi_UBspline_1d_z *spline, double x, complex_double *vals);
void eval_multi_UBspline_1d_z_vg(multi_UBspline_1d_z *spline, double x, complex_double *vals, complex_double *grads);
void eval_multi_UBspline_1d_z_vgl(multi_UBspline_1d_z *spline, double x, complex_double *vals, complex_double *grads, complex_double *lapl);
void eval_multi_UBspline_1d_z_vgh(multi_UBspline_1d_z *spline, double x, complex_double *vals, complex_double *grads, complex_double *hess);
void eval_multi_UBspline_2d_z(multi_UBspline_2d_z *spline, double x, double y, complex_double *vals);
void eval_multi_UBspline_2d_z_vg(multi_UBspline_2d_z *spline, double x, double y, complex_double *vals, complex_double *grads);
void eval_multi_UBspline_2d_z_vgl(multi_UBspline_2d_z *spline, double x, double y, complex_double *vals, complex_double *grads,
                                   complex_double *lapl);
void eval_multi_UBspline_2d_z_vgh(multi_UBspline_2d_z *spline, double x, double y, complex_double *vals, complex_double *grads,
                                   complex_double *hess);

/* ---- 3D */
void eval_multi_UBspline_3d_z(multi_UBspline_3d_z *spline, double x, double y, double z,
                               complex_double *vals);

/* src/multi_bspline_eval_z.h:92-103: value and gradient, grads[N][3]. */
void eval_multi_UBspline_3d_z_vg(multi_UBspline_3d_z *spline, double x, double y, double z,
                                  complex_double *vals, complex_double *grads);

/* src/multi_bspline_eval_z.h:92-103: value, gradient and laplacian (d2/dx2 + d2/dy2 + d2/dz2), lapl[N]. */
void eval_multi_UBspline_3d_z_vgl(multi_UBspline_3d_z *spline, double x, double y, double z,
                                   complex_double *vals, complex_double *grads, complex_double *lapl);

void eval_multi_UBspline_3d_z_vgh(multi_UBspline_3d_z *spline, double x, double y, double z,
                                   complex_double *vals, complex_double *grads, complex_double *hess);

/* src/multi_bspline_eval_std_z_impl.h:868 (the reference declares it in its
 * std/sse backend headers only): value, gradient, Hessian and third
 * derivatives, gradhess[N][3][3][3] (all 27 entries, symmetric copies filled). */
void eval_multi_UBspline_3d_z_vghgh(multi_UBspline_3d_z *spline, double x, double y, double z,
                                     complex_double *vals, complex_double *grads, complex_double *hess, complex_double *gradhess);

#ifdef __cplusplus
}
#endif

#endif
