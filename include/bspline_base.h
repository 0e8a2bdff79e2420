/*
 * bspline_base.h -- basic types of the einspline C API, kept layout-compatible
 * with the reference so that callers compile and link unchanged.
 *
 * Replaces the reference's src/bspline_base.h:49-102 (bc_code, spline_code,
 * type_code, BCtype_{s,d,c,z}, Ugrid, Bspline, destroy_Bspline).
 */
#ifndef EINSPLINE_GB300_BSPLINE_BASE_H
#define EINSPLINE_GB300_BSPLINE_BASE_H

#ifdef __cplusplus
#include <complex>
typedef std::complex<float>  complex_float;
typedef std::complex<double> complex_double;
#else
#include <complex.h>
typedef complex float  complex_float;
typedef complex double complex_double;
#endif

/* Boundary conditions (src/bspline_base.h:49). */
typedef enum { PERIODIC, DERIV1, DERIV2, FLAT, NATURAL, ANTIPERIODIC } bc_code;
/* Spline kinds (src/bspline_base.h:50-53); this library builds MULTI_U1D, MULTI_U2D and MULTI_U3D. */
typedef enum { U1D, U2D, U3D,
               NU1D, NU2D, NU3D,
               MULTI_U1D, MULTI_U2D, MULTI_U3D,
               MULTI_NU1D, MULTI_NU2D, MULTI_NU3D } spline_code;
/* Value types (src/bspline_base.h:54-55). */
typedef enum { SINGLE_REAL, DOUBLE_REAL, SINGLE_COMPLEX, DOUBLE_COMPLEX } type_code;

typedef struct { bc_code lCode, rCode; float lVal, rVal; } BCtype_s;
typedef struct { bc_code lCode, rCode; double lVal, rVal; } BCtype_d;
typedef struct { bc_code lCode, rCode; float lVal_r, lVal_i, rVal_r, rVal_i; } BCtype_c;
typedef struct { bc_code lCode, rCode; double lVal_r, lVal_i, rVal_r, rVal_i; } BCtype_z;

/* Uniform grid: the caller sets start, end, num; create fills delta and
 * delta_inv (src/bspline_base.h:81-88). */
typedef struct
{
  double start, end;
  int num;
  /* private */
  double delta, delta_inv;
} Ugrid;

/* Common header of every spline struct (src/bspline_base.h:90-95). */
typedef struct
{
  spline_code sp_code;
  type_code   t_code;
  void *coefs;
} Bspline;

#ifdef __cplusplus
extern "C"
#endif
/* Frees any spline made by this library's create functions
 * (src/bspline_base.h:98-102; src/bspline_create.c:1865-1877). */
void destroy_Bspline(void *spline);

#endif
