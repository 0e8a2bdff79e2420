/*
 * multi_bspline_create.h -- create / set / destroy for uniform 1D, 2D and
 * 3D multi-splines.
 *
 * Replaces the entries of src/multi_bspline_create.h:41-171: 1D/2D at
 * :41-62 (s), :74-101 (d), :109-130 (c), :141-166 (z), and 3D
 * (create_multi_UBspline_3d_{s,d,c,z} at :60-63, :88-91, :120-123, :150-153;
 *  set_multi_UBspline_3d_{s,d,c,z} at :75, :105, :136, :170).
 *
 * Behaviour kept: same names, argument meaning and grid set-up (N = M+3 for
 * periodic/antiperiodic, M+2 otherwise; delta = (end-start)/(N-3)).
 * Behaviour changed, by design:
 *   * the table is allocated in GPU memory and the interpolating solve runs
 *     on the GPU in FP64 for every type (the reference solves s/c in float);
 *     results are rounded once, on store, to the table's storage type;
 *   * set_* copies the caller's data and queues the spline; queued splines are
 *     solved together, in one batched launch, when the queue is full or
 *     before the next evaluation (einspline_gb300_flush forces it).  The
 *     caller may reuse or free data as soon as set_* returns.
 * Errors (bad arguments, out of GPU memory, CUDA errors) are reported through
 * einspline_gb300_last_error(); in the default mode they also print and
 * abort() as the reference does.
 */
#ifndef EINSPLINE_GB300_MULTI_BSPLINE_CREATE_H
#define EINSPLINE_GB300_MULTI_BSPLINE_CREATE_H

#include "bspline_base.h"
#include "multi_bspline_structs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---- 1D and 2D multi-splines (src/multi_bspline_create.c:88-248 s,
 * :389-575 c, :767-940 d, :1091-1316 z).  Same rules as 3D: FP64 solve on
 * the GPU, rounded once on store; data is [Mx] or [Mx][My], C order. */
multi_UBspline_1d_s *create_multi_UBspline_1d_s(Ugrid x_grid, BCtype_s xBC, int num_splines);
multi_UBspline_2d_s *create_multi_UBspline_2d_s(Ugrid x_grid, Ugrid y_grid, BCtype_s xBC, BCtype_s yBC,
                                                 int num_splines);
void set_multi_UBspline_1d_s(multi_UBspline_1d_s *spline, int spline_num, float *data);
void set_multi_UBspline_2d_s(multi_UBspline_2d_s *spline, int spline_num, float *data);
multi_UBspline_1d_d *create_multi_UBspline_1d_d(Ugrid x_grid, BCtype_d xBC, int num_splines);
multi_UBspline_2d_d *create_multi_UBspline_2d_d(Ugrid x_grid, Ugrid y_grid, BCtype_d xBC, BCtype_d yBC,
                                                 int num_splines);
void set_multi_UBspline_1d_d(multi_UBspline_1d_d *spline, int spline_num, double *data);
void set_multi_UBspline_2d_d(multi_UBspline_2d_d *spline, int spline_num, double *data);
multi_UBspline_1d_c *create_multi_UBspline_1d_c(Ugrid x_grid, BCtype_c xBC, int num_splines);
multi_UBspline_2d_c *create_multi_UBspline_2d_c(Ugrid x_grid, Ugrid y_grid, BCtype_c xBC, BCtype_c yBC,
                                                 int num_splines);
void set_multi_UBspline_1d_c(multi_UBspline_1d_c *spline, int spline_num, complex_float *data);
void set_multi_UBspline_2d_c(multi_UBspline_2d_c *spline, int spline_num, complex_float *data);
multi_UBspline_1d_z *create_multi_UBspline_1d_z(Ugrid x_grid, BCtype_z xBC, int num_splines);
multi_UBspline_2d_z *create_multi_UBspline_2d_z(Ugrid x_grid, Ugrid y_grid, BCtype_z xBC, BCtype_z yBC,
                                                 int num_splines);
void set_multi_UBspline_1d_z(multi_UBspline_1d_z *spline, int spline_num, complex_double *data);
void set_multi_UBspline_2d_z(multi_UBspline_2d_z *spline, int spline_num, complex_double *data);
/* src/multi_bspline_create.h:94 and :161: one spline solved with its
 * own x boundary condition.  The codes must be periodic (or antiperiodic)
 * exactly when the table's are (the table size depends on it); otherwise
 * the call fails with EINVAL (the reference would write past the table). */
void set_multi_UBspline_1d_d_BC(multi_UBspline_1d_d *spline, int spline_num, double *data, BCtype_d xBC);
void set_multi_UBspline_1d_z_BC(multi_UBspline_1d_z *spline, int spline_num, complex_double *data, BCtype_z xBC);

/* src/multi_bspline_create.h:60-63; src/multi_bspline_create.c:252-321 */
multi_UBspline_3d_s *
create_multi_UBspline_3d_s(Ugrid x_grid, Ugrid y_grid, Ugrid z_grid,
                           BCtype_s xBC, BCtype_s yBC, BCtype_s zBC, int num_splines);
/* src/multi_bspline_create.h:75; src/multi_bspline_create.c:324-373.
 * data: host array [Mx][My][Mz], C order. */
void set_multi_UBspline_3d_s(multi_UBspline_3d_s *spline, int spline_num, float *data);

/* src/multi_bspline_create.h:88-91; src/multi_bspline_create.c:942-1018 */
multi_UBspline_3d_d *
create_multi_UBspline_3d_d(Ugrid x_grid, Ugrid y_grid, Ugrid z_grid,
                           BCtype_d xBC, BCtype_d yBC, BCtype_d zBC, int num_splines);
/* src/multi_bspline_create.h:105; src/multi_bspline_create.c:1021-1073 */
void set_multi_UBspline_3d_d(multi_UBspline_3d_d *spline, int spline_num, double *data);

/* src/multi_bspline_create.h:120-123; src/multi_bspline_create.c:577-648 */
multi_UBspline_3d_c *
create_multi_UBspline_3d_c(Ugrid x_grid, Ugrid y_grid, Ugrid z_grid,
                           BCtype_c xBC, BCtype_c yBC, BCtype_c zBC, int num_splines);
/* src/multi_bspline_create.h:136; src/multi_bspline_create.c:651-732.
 * data: host array [Mx][My][Mz] of complex (re, im interleaved). */
void set_multi_UBspline_3d_c(multi_UBspline_3d_c *spline, int spline_num, complex_float *data);

/* src/multi_bspline_create.h:150-153; src/multi_bspline_create.c:1318-1390 */
multi_UBspline_3d_z *
create_multi_UBspline_3d_z(Ugrid x_grid, Ugrid y_grid, Ugrid z_grid,
                           BCtype_z xBC, BCtype_z yBC, BCtype_z zBC, int num_splines);
/* src/multi_bspline_create.h:170; src/multi_bspline_create.c:1393-1478 */
void set_multi_UBspline_3d_z(multi_UBspline_3d_z *spline, int spline_num, complex_double *data);

/* src/multi_bspline_create.c:1480-1485 (reached through destroy_Bspline). */
void destroy_multi_UBspline(Bspline *spline);

#ifdef __cplusplus
}
#endif

#endif
