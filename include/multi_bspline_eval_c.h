/*
 * multi_bspline_eval_c.h -- single-point evaluation of a uniform 1D/2D/3D
 * multi-spline of type c (complex_float), host output buffers.
 *
 * Replaces the 3D value, vg, vgl and vgh entries of src/multi_bspline_eval_c.h:92-115
 * and the std backend's vghgh entry.
 * Output layout is the reference CPU layout: vals[N], grads[N][3],
 * hess[N][3][3] (full symmetric matrix, row-major).  The point may be given
 * anywhere; the reference reads outside its table when a point leaves
 * [start, end], this library extrapolates the edge cell instead.
 * Each call runs one GPU launch plus a device-to-host copy: for many points
 * use eval_multi_multi_UBspline_3d_c*_cuda or einspline_gb300_eval_3d.
 */
#ifndef EINSPLINE_GB300_MULTI_BSPLINE_EVAL_C_H
#define EINSPLINE_GB300_MULTI_BSPLINE_EVAL_C_H

#include "multi_bspline_structs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- 1D and 2D (src/multi_bspline_eval_c.h:32-81; std backend
 * src/multi_bspline_eval_std_c_impl.h).  1D: grads[N], lapl[N] and hess[N]
 * are first and second derivatives (the 1D vgh equals the vgl, as in the
 * reference).  2D: grads[N][2], lapl[N] = d2/dx2 + d2/dy2, hess[N][2][2]. */
void eval_multi_UBspline_1d_c(multi_UBspline_1d_c *spline, double x, complex_float *vals);
void eval_multi_UBspline_1d_c_vg(multi_UBspline_1d_c *spline, double x, complex_float *vals, complex_float *grads);
void eval_multi_UBspline_1d_c_vgl(multi_UBspline_1d_c *spline, double x, complex_float *vals, complex_float *grads, complex_float *lapl);
void eval_multi_UBspline_1d_c_vgh(multi_UBspline_1d_c *spline, double x, complex_float *vals, complex_float *grads, complex_float *hess);
void eval_multi_UBspline_2d_c(multi_UBspline_2d_c *spline, double x, double y, complex_float *vals);
void eval_multi_UBspline_2d_c_vg(multi_UBspline_2d_c *spline, double x, double y, complex_float *vals, complex_float *grads);
void eval_multi_UBspline_2d_c_vgl(multi_UBspline_2d_c *spline, double x, double y, complex_float *vals, complex_float *grads,
                                   complex_float *lapl);
void eval_multi_UBspline_2d_c_vgh(multi_UBspline_2d_c *spline, double x, double y, complex_float *vals, complex_float *grads,
                                   complex_float *hess);

/* ---- 3D */
void eval_multi_UBspline_3d_c(multi_UBspline_3d_c *spline, double x, double y, double z,
                               complex_float *vals);

/* src/multi_bspline_eval_c.h:97-108: value and gradient, grads[N][3]. */
void eval_multi_UBspline_3d_c_vg(multi_UBspline_3d_c *spline, double x, double y, double z,
                                  complex_float *vals, complex_float *grads);

/* src/multi_bspline_eval_c.h:97-108: value, gradient and laplacian (d2/dx2 + d2/dy2 + d2/dz2), lapl[N]. */
void eval_multi_UBspline_3d_c_vgl(multi_UBspline_3d_c *spline, double x, double y, double z,
                                   complex_float *vals, complex_float *grads, complex_float *lapl);

void eval_multi_UBspline_3d_c_vgh(multi_UBspline_3d_c *spline, double x, double y, double z,
                                   complex_float *vals, complex_float *grads, complex_float *hess);

/* src/multi_bspline_eval_std_c_impl.h:864 (the reference declares it in its
 * std/sse backend headers only): value, gradient, Hessian and third
 * derivatives, gradhess[N][3][3][3] (all 27 entries, symmetric copies filled). */
void eval_multi_UBspline_3d_c_vghgh(multi_UBspline_3d_c *spline, double x, double y, double z,
                                     complex_float *vals, complex_float *grads, complex_float *hess, complex_float *gradhess);

#ifdef __cplusplus
}
#endif

#endif
