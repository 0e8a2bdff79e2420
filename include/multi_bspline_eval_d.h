/*
 * multi_bspline_eval_d.h -- single-point evaluation of a uniform 3D
 * multi-spline of type d (double), host output buffers.
 *
 * Replaces the 3D value and vgh entries of src/multi_bspline_eval_d.h:88-111.
 * Output layout is the reference CPU layout: vals[N], grads[N][3],
 * hess[N][3][3] (full symmetric matrix, row-major).  The point may be given
 * anywhere; the reference reads outside its table when a point leaves
 * [start, end], this library extrapolates the edge cell instead.
 * Each call runs one GPU launch plus a device-to-host copy: for many points
 * use eval_multi_multi_UBspline_3d_d*_cuda or einspline_gb300_eval_3d.
 */
#ifndef EINSPLINE_GB300_MULTI_BSPLINE_EVAL_D_H
#define EINSPLINE_GB300_MULTI_BSPLINE_EVAL_D_H

#include "multi_bspline_structs.h"

#ifdef __cplusplus
extern "C" {
#endif

void eval_multi_UBspline_3d_d(multi_UBspline_3d_d *spline, double x, double y, double z,
                               double *vals);

void eval_multi_UBspline_3d_d_vgh(multi_UBspline_3d_d *spline, double x, double y, double z,
                                   double *vals, double *grads, double *hess);

#ifdef __cplusplus
}
#endif

#endif
