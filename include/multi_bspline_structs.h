/*
 * multi_bspline_structs.h -- uniform 1D, 2D and 3D multi-spline structs.
 *
 * Replaces src/multi_bspline_structs.h:155-164 (3d_s), :192-201 (3d_d),
 * :232-243 (3d_c), :273-284 (3d_z) and the 1D/2D structs of the same file
 * (:28-51 s, :66-89 d, :103-128 c, :142-168 z).  Every public field keeps
 * its name, type and offset.  Two differences a caller must know:
 *   * coefs is a DEVICE pointer: the table lives in GPU memory (HBM) as
 *     coefs[Nx][Ny][Nz][z_stride].  Use einspline_gb300_copy_table() to read
 *     it on the host, or einspline_gb300_host_coefs() for a host mirror in
 *     the reference's layout and value type (pushed back to the device by
 *     einspline_gb300_push_host_coefs()).  The storage type may be narrower
 *     than the value type for s/c tables made with einspline_gb300_create_3d_{s,c}.
 *   * a private pointer (gb300) is appended after the public fields.  The
 *     structs are only ever made by this library's create functions, as in
 *     the reference, so appending does not change any public offset.
 * The innermost stride (z_stride in 3D, y_stride in 2D, x_stride in 1D) is
 * num_splines padded so that every table row starts on a 128-byte boundary
 * (the reference pads to the SIMD width).  The 2D complex structs keep the
 * reference's lapl2 scratch pointer for layout; it is NULL here.
 */
#ifndef EINSPLINE_GB300_MULTI_BSPLINE_STRUCTS_H
#define EINSPLINE_GB300_MULTI_BSPLINE_STRUCTS_H

#include <stdint.h>
#include "bspline_base.h"

struct einspline_gb300_table;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  float *coefs;
  intptr_t x_stride;
  Ugrid x_grid;
  BCtype_s xBC;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_1d_s;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  float *coefs;
  intptr_t x_stride, y_stride;
  Ugrid x_grid, y_grid;
  BCtype_s xBC, yBC;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_2d_s;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  double *coefs;
  intptr_t x_stride;
  Ugrid x_grid;
  BCtype_d xBC;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_1d_d;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  double *coefs;
  intptr_t x_stride, y_stride;
  Ugrid x_grid, y_grid;
  BCtype_d xBC, yBC;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_2d_d;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  complex_float *coefs;
  intptr_t x_stride;
  Ugrid x_grid;
  BCtype_c xBC;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_1d_c;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  complex_float *coefs;
  intptr_t x_stride, y_stride;
  Ugrid x_grid, y_grid;
  BCtype_c xBC, yBC;
  int num_splines;
  /* temporary storage for laplacian components (unused here; kept for layout) */
  complex_float *lapl2;
  struct einspline_gb300_table *gb300;
} multi_UBspline_2d_c;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  complex_double *coefs;
  intptr_t x_stride;
  Ugrid x_grid;
  BCtype_z xBC;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_1d_z;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  complex_double *coefs;
  intptr_t x_stride, y_stride;
  Ugrid x_grid, y_grid;
  BCtype_z xBC, yBC;
  int num_splines;
  /* temporary storage for laplacian components (unused here; kept for layout) */
  complex_double *lapl2;
  struct einspline_gb300_table *gb300;
} multi_UBspline_2d_z;


typedef struct
{
  spline_code spcode;
  type_code    tcode;
  float *coefs;
  intptr_t x_stride, y_stride, z_stride;
  Ugrid x_grid, y_grid, z_grid;
  BCtype_s xBC, yBC, zBC;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_3d_s;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  double *coefs;
  intptr_t x_stride, y_stride, z_stride;
  Ugrid x_grid, y_grid, z_grid;
  BCtype_d xBC, yBC, zBC;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_3d_d;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  complex_float *coefs;
  intptr_t x_stride, y_stride, z_stride;
  Ugrid x_grid, y_grid, z_grid;
  BCtype_c xBC, yBC, zBC;
  int num_splines;
  /* temporary storage for laplacian components (unused here; kept for layout) */
  complex_float *lapl3;
  struct einspline_gb300_table *gb300;
} multi_UBspline_3d_c;

typedef struct
{
  spline_code spcode;
  type_code    tcode;
  complex_double *coefs;
  intptr_t x_stride, y_stride, z_stride;
  Ugrid x_grid, y_grid, z_grid;
  BCtype_z xBC, yBC, zBC;
  int num_splines;
  /* temporary storage for laplacian components (unused here; kept for layout) */
  complex_double *lapl3;
  struct einspline_gb300_table *gb300;
} multi_UBspline_3d_z;

#endif
