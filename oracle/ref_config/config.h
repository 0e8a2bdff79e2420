/* Hand-written config.h for compiling the reference's portable ("std") CPU
 * sources directly with gcc, without its autotools build.  No SIMD backend,
 * no HIGH_PRECISION: the same choices as a default ./configure on a machine
 * without SSE. */
#ifndef EINSPLINE_REF_CONFIG_H
#define EINSPLINE_REF_CONFIG_H
#define HAVE_POSIX_MEMALIGN 1
#define HAVE_C_VARARRAYS 1
#endif
