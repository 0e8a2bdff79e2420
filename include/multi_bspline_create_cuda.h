/*
 * multi_bspline_create_cuda.h -- make device handles from host-API splines.
 *
 * Replaces the 3D entries of src/multi_bspline_create_cuda.h:60-78
 * (src/multi_bspline_create_cuda.cu:245, :328, :427, :500, :590, :662).
 * Each call makes an independent device copy of the table, as the
 * reference does, so either object may be destroyed first.  The _conv forms
 * round an FP64 table to FP32 on the GPU (d -> s, z -> c).  Unlike the
 * reference these accept every boundary condition, not only periodic ones.
 * destroy_multi_UBspline_3d_*_cuda is new: the reference has no destructor
 * (its test frees ->coefs with cudaFree, which also works here).
 */
#ifndef EINSPLINE_GB300_MULTI_BSPLINE_CREATE_CUDA_H
#define EINSPLINE_GB300_MULTI_BSPLINE_CREATE_CUDA_H

#include "multi_bspline_structs.h"
#include "multi_bspline_structs_cuda.h"

#ifdef __cplusplus
extern "C" {
#endif

/* 1D (src/multi_bspline_create_cuda.h:10-28; the reference implements s and
 * c, src/multi_bspline_create_cuda.cu:17-237, and declares d and z). */
multi_UBspline_1d_s_cuda *create_multi_UBspline_1d_s_cuda(multi_UBspline_1d_s *spline);
multi_UBspline_1d_s_cuda *create_multi_UBspline_1d_s_cuda_conv(multi_UBspline_1d_d *spline);
multi_UBspline_1d_c_cuda *create_multi_UBspline_1d_c_cuda(multi_UBspline_1d_c *spline);
multi_UBspline_1d_c_cuda *create_multi_UBspline_1d_c_cuda_conv(multi_UBspline_1d_z *spline);
multi_UBspline_1d_d_cuda *create_multi_UBspline_1d_d_cuda(multi_UBspline_1d_d *spline);
multi_UBspline_1d_z_cuda *create_multi_UBspline_1d_z_cuda(multi_UBspline_1d_z *spline);
void destroy_multi_UBspline_1d_s_cuda(multi_UBspline_1d_s_cuda *spline);
void destroy_multi_UBspline_1d_c_cuda(multi_UBspline_1d_c_cuda *spline);
void destroy_multi_UBspline_1d_d_cuda(multi_UBspline_1d_d_cuda *spline);
void destroy_multi_UBspline_1d_z_cuda(multi_UBspline_1d_z_cuda *spline);

/* 3D */
multi_UBspline_3d_s_cuda *create_multi_UBspline_3d_s_cuda(multi_UBspline_3d_s *spline);
multi_UBspline_3d_s_cuda *create_multi_UBspline_3d_s_cuda_conv(multi_UBspline_3d_d *spline);
multi_UBspline_3d_c_cuda *create_multi_UBspline_3d_c_cuda(multi_UBspline_3d_c *spline);
multi_UBspline_3d_c_cuda *create_multi_UBspline_3d_c_cuda_conv(multi_UBspline_3d_z *spline);
multi_UBspline_3d_d_cuda *create_multi_UBspline_3d_d_cuda(multi_UBspline_3d_d *spline);
multi_UBspline_3d_z_cuda *create_multi_UBspline_3d_z_cuda(multi_UBspline_3d_z *spline);

void destroy_multi_UBspline_3d_s_cuda(multi_UBspline_3d_s_cuda *spline);
void destroy_multi_UBspline_3d_c_cuda(multi_UBspline_3d_c_cuda *spline);
void destroy_multi_UBspline_3d_d_cuda(multi_UBspline_3d_d_cuda *spline);
void destroy_multi_UBspline_3d_z_cuda(multi_UBspline_3d_z_cuda *spline);

#ifdef __cplusplus
}
#endif

#endif
