/*
 * multi_bspline_structs_cuda.h -- device-side 1D and 3D multi-spline handles.
 *
 * Replaces the 1D and 3D structs of src/multi_bspline_structs_cuda.h:14-48
 * and :90-124 (the reference has no 2D evaluation on the GPU).  Public
 * fields keep names, types and offsets; a private pointer (gb300) is appended.
 * Handles come only from create_multi_UBspline_{1d,3d}_*_cuda*.
 *   coefs   device table, rows padded to 128 bytes (the reference pads N to 16)
 *   stride  element strides (x, y, z) -- in float units for c and double units
 *           for z, as in the reference; 0 when a stride exceeds 32 bits
 *           (the library itself uses 64-bit strides held privately)
 *   gridInv 1/delta per axis
 *   dim     number of cells per axis (M for periodic grids, as the reference)
 */
#ifndef EINSPLINE_GB300_MULTI_BSPLINE_STRUCTS_CUDA_H
#define EINSPLINE_GB300_MULTI_BSPLINE_STRUCTS_CUDA_H

#include <vector_types.h>
#include "bspline_base.h"

/* Threads per block of the reference kernels (src/multi_bspline_structs_cuda.h:4).
 * Kept for callers that size their own launches from it. */
#define SPLINE_BLOCK_SIZE 64

struct einspline_gb300_table;

/* 1D handles (src/multi_bspline_structs_cuda.h:14-48): stride is the row
 * stride in reals, dim the number of cells (M for periodic grids). */
typedef struct
{
  float *coefs;
  unsigned int stride;
  float gridInv;
  int num_splines;
  int dim;
  struct einspline_gb300_table *gb300;
} multi_UBspline_1d_s_cuda;

typedef struct
{
  complex_float *coefs;
  unsigned int stride;
  float gridInv;
  int num_splines;
  int dim;
  struct einspline_gb300_table *gb300;
} multi_UBspline_1d_c_cuda;

typedef struct
{
  double *coefs;
  unsigned int stride;
  double gridInv;
  int num_splines;
  int dim;
  struct einspline_gb300_table *gb300;
} multi_UBspline_1d_d_cuda;

typedef struct
{
  complex_double *coefs;
  unsigned int stride;
  double gridInv;
  int num_splines;
  int dim;
  struct einspline_gb300_table *gb300;
} multi_UBspline_1d_z_cuda;


typedef struct
{
  float *coefs;
  uint3 stride;
  float3 gridInv;
  uint3 dim;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_3d_s_cuda;

typedef struct
{
  complex_float *coefs;
  uint3 stride;
  float3 gridInv;
  uint3 dim;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_3d_c_cuda;

typedef struct
{
  double *coefs;
  uint3 stride;
  double3 gridInv;
  uint3 dim;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_3d_d_cuda;

typedef struct
{
  complex_double *coefs;
  uint3 stride;
  double3 gridInv;
  uint3 dim;
  int num_splines;
  struct einspline_gb300_table *gb300;
} multi_UBspline_3d_z_cuda;

#endif
