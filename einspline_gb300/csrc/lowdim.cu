// 1D and 2D multi-splines: the CPU entries eval_multi_UBspline_{1d,2d}_*
// [_vg, _vgl, _vgh] (src/multi_bspline_eval_std_s_impl.h:38-480, d/c/z
// alike) and the batched 1D GPU entries eval_multi_multi_UBspline_1d_*[_vgl]_cuda
// (src/multi_bspline_cuda_s_impl.h:10-175, src/multi_bspline_cuda_c_impl.h:9-175).
//
// A block takes kLdPoints points and kLdThreads * VW consecutive real columns; each
// thread reads its columns of the 4 (1D) or 16 (2D) stencil rows with one
// vector load per row and reduces them separably (y first, then x), the
// basis weights computed by every thread from the point's cell (a handful
// of multiply-adds, no shared memory).  The tables are small next to the 3D
// ones: these paths are for API completeness and latency, not bandwidth.
#include <string.h>

#include "eval_core.h"

namespace eg {

constexpr int kLdThreads = 128;
constexpr int kLdPoints = 4;

template <typename A>
__device__ __forceinline__ void ld_axis(const EvalArgs &a, int64_t p, int ax, int dims, int &idx, A *w) {
  double xd;
  if (!a.pos) xd = a.inl[ax];
  else if (a.pos_f64) xd = reinterpret_cast<const double *>(a.pos)[dims * p + ax];
  else xd = (double)reinterpret_cast<const float *>(a.pos)[dims * p + ax];
  A t;
  cell(a, ax, xd, idx, t);
  const A d = a.unscaled ? A(1) : (sizeof(A) == 4 ? (A)a.dinvf[ax] : (A)a.dinv[ax]);
  bspline_weights<A>(t, w, d);
}

// Stores VW values at p (16-byte vector stores when aligned and complete).
template <typename A, int VW>
__device__ __forceinline__ void st_row(A *p, int col0, int ncol, const A (&v)[VW]) {
  if (col0 + VW <= ncol && al16(p)) {
#pragma unroll
    for (int c = 0; c < VW * (int)sizeof(A) / 16; c++) {
      float4 q;
      memcpy(&q, reinterpret_cast<const char *>(v) + 16 * c, 16);
      reinterpret_cast<float4 *>(p)[c] = q;
    }
  } else {
#pragma unroll
    for (int e = 0; e < VW; e++)
      if (col0 + e < ncol) p[e] = v[e];
  }
}

template <int ST, int D, bool DER>
__device__ __forceinline__ void eval_ld_point(const EvalArgs &a, int64_t p, int col0);

template <int ST, int D, bool DER>
__global__ void __launch_bounds__(kLdThreads) k_eval_ld(const EvalArgs a) {
  constexpr int VW = CT<ST>::VW;
  const int col0 = (blockIdx.y * kLdThreads + threadIdx.x) * VW;
  if (col0 >= a.ncol) return;
  // kLdPoints consecutive points per block: more loads in flight per warp
  const int64_t p0 = (int64_t)blockIdx.x * kLdPoints;
#pragma unroll 1
  for (int q = 0; q < kLdPoints; q++)
    if (p0 + q < a.npts) eval_ld_point<ST, D, DER>(a, p0 + q, col0);
}

// o (D = 1): value, first, second derivative.
// o (D = 2): value, d/dx, d/dy, d2/dx2, d2/dxdy, d2/dy2.
// a.out: 0 value, 1 vg, 2 vgl, 3 vgh; a.layout: 1 the CPU API's layouts at
// flat bases with per-point strides, 0 the 1D GPU entries' pointer arrays
// (value, gradient, second derivative per real column).
template <int ST, int D, bool DER>
__device__ __forceinline__ void eval_ld_point(const EvalArgs &a, int64_t p, int col0) {
  using A = typename CT<ST>::A;
  constexpr int VW = CT<ST>::VW;
  A wx[12], wy[12];
  int ix, iy = 0;
  ld_axis<A>(a, p, 0, D, ix, wx);
  if (D == 2) ld_axis<A>(a, p, 1, D, iy, wy);
  const int64_t xsb = a.xs * CT<ST>::BYTES, ysb = a.ys * CT<ST>::BYTES;
  const char *base = reinterpret_cast<const char *>(a.coefs) + (int64_t)col0 * CT<ST>::BYTES + ix * xsb + iy * ysb;
  A o[6][VW];
#pragma unroll
  for (int q = 0; q < 6; q++)
#pragma unroll
    for (int e = 0; e < VW; e++) o[q][e] = A(0);
  if (D == 1) {
#pragma unroll
    for (int i = 0; i < 4; i++) {
      A c[VW];
      load_row<ST>(base + i * xsb, c);
#pragma unroll
      for (int e = 0; e < VW; e++) {
        o[0][e] = fmaT(wx[i], c[e], o[0][e]);
        if (DER) {
          o[1][e] = fmaT(wx[4 + i], c[e], o[1][e]);
          o[2][e] = fmaT(wx[8 + i], c[e], o[2][e]);
        }
      }
    }
  } else {
#pragma unroll
    for (int i = 0; i < 4; i++) {
      A y[3][VW];
#pragma unroll
      for (int q = 0; q < 3; q++)
#pragma unroll
        for (int e = 0; e < VW; e++) y[q][e] = A(0);
#pragma unroll
      for (int j = 0; j < 4; j++) {
        A c[VW];
        load_row<ST>(base + i * xsb + j * ysb, c);
#pragma unroll
        for (int e = 0; e < VW; e++) {
          y[0][e] = fmaT(wy[j], c[e], y[0][e]);
          if (DER) {
            y[1][e] = fmaT(wy[4 + j], c[e], y[1][e]);
            y[2][e] = fmaT(wy[8 + j], c[e], y[2][e]);
          }
        }
      }
#pragma unroll
      for (int e = 0; e < VW; e++) {
        o[0][e] = fmaT(wx[i], y[0][e], o[0][e]);
        if (DER) {
          o[1][e] = fmaT(wx[4 + i], y[0][e], o[1][e]);
          o[2][e] = fmaT(wx[i], y[1][e], o[2][e]);
          o[3][e] = fmaT(wx[8 + i], y[0][e], o[3][e]);
          o[4][e] = fmaT(wx[4 + i], y[1][e], o[4][e]);
          o[5][e] = fmaT(wx[i], y[2][e], o[5][e]);
        }
      }
    }
  }
  if (a.scale) {
#pragma unroll
    for (int e = 0; e < VW; e++) {
      const A sc = (A)a.scale[col0 + e];
#pragma unroll
      for (int q = 0; q < 6; q++) o[q][e] *= sc;
    }
  }
  if (a.layout == 0) {
    st_row<A, VW>(reinterpret_cast<A *>(a.vals_pp[p]) + col0, col0, a.ncol, o[0]);
    if (DER && a.out >= 1) st_row<A, VW>(reinterpret_cast<A *>(a.grads_pp[p]) + col0, col0, a.ncol, o[1]);
    if (DER && a.out >= 2) st_row<A, VW>(reinterpret_cast<A *>(a.hess_pp[p]) + col0, col0, a.ncol, o[2]);
    return;
  }
  const int nc = a.is_complex ? 2 : 1;
#pragma unroll
  for (int e = 0; e < VW; e++) {
    const int col = col0 + e;
    if (col >= a.ncol) break;
    // complex columns interleave re/im of one spline: entry m of spline n
    // sits at nc * (K * n + m) + part for a K-entry output
    const int n = col / nc, part = col - n * nc;
    reinterpret_cast<A *>(a.vals)[p * a.vstride + col] = o[0][e];
    if (!DER || a.out == 0) continue;
    A *gp = reinterpret_cast<A *>(a.grads) + p * a.gstride;
    A *hp = reinterpret_cast<A *>(a.hess) + p * a.hstride;
    if (D == 1) {
      gp[col] = o[1][e];
      if (a.out >= 2) hp[col] = o[2][e];
    } else {
      gp[nc * (2 * n) + part] = o[1][e];
      gp[nc * (2 * n + 1) + part] = o[2][e];
      if (a.out == 2) hp[col] = o[3][e] + o[5][e];
      if (a.out == 3) {
        hp[nc * (4 * n) + part] = o[3][e];
        hp[nc * (4 * n + 1) + part] = o[4][e];
        hp[nc * (4 * n + 2) + part] = o[4][e];
        hp[nc * (4 * n + 3) + part] = o[5][e];
      }
    }
  }
}

template <int ST>
void launch_ld_st(const EvalArgs &a, int dims, dim3 grid, cudaStream_t s) {
  const bool der = a.out > 0;
  if (dims == 1) {
    if (der) k_eval_ld<ST, 1, true><<<grid, kLdThreads, 0, s>>>(a);
    else k_eval_ld<ST, 1, false><<<grid, kLdThreads, 0, s>>>(a);
  } else {
    if (der) k_eval_ld<ST, 2, true><<<grid, kLdThreads, 0, s>>>(a);
    else k_eval_ld<ST, 2, false><<<grid, kLdThreads, 0, s>>>(a);
  }
}

int launch_ld(Table *t, const EvalArgs &a, cudaStream_t s) {
  const int VW = t->storage == ST_F64 ? 2 : 4;
  const unsigned tiles = (unsigned)((t->ncol + kLdThreads * VW - 1) / (kLdThreads * VW));
  const int64_t blocks = (a.npts + kLdPoints - 1) / kLdPoints;
  if (blocks > 0x7FFFFFFF) return fail(EINSPLINE_GB300_ESIZE, "too many points in one call");
  const dim3 grid((unsigned)blocks, tiles);
  switch (t->storage) {
    case ST_F32: launch_ld_st<ST_F32>(a, t->dims, grid, s); break;
    case ST_F16: launch_ld_st<ST_F16>(a, t->dims, grid, s); break;
    case ST_BF16: launch_ld_st<ST_BF16>(a, t->dims, grid, s); break;
    case ST_I16: launch_ld_st<ST_I16>(a, t->dims, grid, s); break;
    default: launch_ld_st<ST_F64>(a, t->dims, grid, s); break;
  }
  EG_CUDA(cudaGetLastError());
  count_launch();
  return 0;
}

}  // namespace eg

using namespace eg;

namespace {

template <typename S>
Table *ld_table(S *s, int dims, const char *fn) {
  if (!s || !table_ok(s->gb300) || s->gb300->dims != dims) {
    fail(EINSPLINE_GB300_EINVAL, "%s: not a %dD spline made by this library", fn, dims);
    return nullptr;
  }
  return s->gb300;
}

// One point, host outputs in the CPU layouts.  form: 0 value, 1 vg, 2 vgl,
// 3 vgh; lh receives the second derivative (1D), the laplacian (2D vgl) or
// the Hessian (2D vgh).
template <typename S, typename V>
void eval_point_ld(S *s, int dims, double x, double y, V *vals, V *grads, V *lh, int form, const char *fn) {
  clear();
  Table *t = ld_table(s, dims, fn);
  if (!t) return;
  if (!vals || (form >= 1 && !grads) || (form >= 2 && !lh)) {
    fail(EINSPLINE_GB300_EINVAL, "%s: NULL output", fn);
    return;
  }
  if (table_flush(t)) return;
  std::lock_guard<std::mutex> g(t->mu);
  if (point_scratch(t, fn)) return;
  const size_t rb = t->storage == ST_F64 ? 8 : 4;
  const size_t n = (size_t)t->ncol;
  const size_t ng = (size_t)dims, nh = (dims == 2 && form == 3) ? 4 : 1;
  EvalArgs a;
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(t, a);
  a.inl[0] = x; a.inl[1] = y;
  a.rule = 0;
  a.layout = 1;
  a.out = form;
  a.npts = 1;
  a.vals = t->pt_dev;
  a.grads = (char *)t->pt_dev + n * rb;
  a.hess = (char *)t->pt_dev + (1 + ng) * n * rb;
  if (launch_ld(t, a, t->stream)) return;
  // the kernel wrote into the mapped host scratch directly
  if (cudaError_t e = cudaStreamSynchronize(t->stream)) {
    cuda_check(e, fn);
    return;
  }
  memcpy(vals, t->pt_host, n * rb);
  if (form >= 1) memcpy(grads, (char *)t->pt_host + n * rb, ng * n * rb);
  if (form >= 2) memcpy(lh, (char *)t->pt_host + (1 + ng) * n * rb, nh * n * rb);
}

// Batched 1D GPU entries: reference GPU cell rule, derivatives in cell units,
// pointer-array outputs; returns when the results are ready.
template <typename CS>
void eval_cuda_1d(CS *c, const void *pos_d, bool pos_f64, void *const *vals_d, void *const *grads_d,
                  void *const *lapl_d, int num, bool vgl, const char *fn) {
  clear();
  if (!c || !table_ok(c->gb300) || c->gb300->dims != 1) {
    fail(EINSPLINE_GB300_EINVAL, "%s: not a 1D handle made by this library", fn);
    return;
  }
  if (num <= 0) return;
  if (!pos_d || !vals_d || (vgl && (!grads_d || !lapl_d))) { fail(EINSPLINE_GB300_EINVAL, "%s: NULL buffer", fn); return; }
  Table *t = c->gb300;
  EvalArgs a;
  memset(&a, 0, sizeof(a));
  fill_eval_geometry(t, a);
  a.pos = pos_d;
  a.pos_f64 = pos_f64;
  a.rule = 1;
  a.layout = 0;
  a.out = vgl ? 2 : 0;
  a.unscaled = 1;
  a.npts = num;
  a.vals_pp = vals_d; a.grads_pp = grads_d; a.hess_pp = lapl_d;
  if (launch_ld(t, a, cudaStreamLegacy)) return;
  cudaError_t e = cudaStreamSynchronize(cudaStreamLegacy);
  if (e != cudaSuccess) cuda_check(e, fn);
}

}  // namespace

extern "C" {

#define EG_LD_ENTRIES(T, V)                                                                                   \
  void eval_multi_UBspline_1d_##T(multi_UBspline_1d_##T *s, double x, V *vals) {                              \
    eval_point_ld(s, 1, x, 0.0, vals, (V *)nullptr, (V *)nullptr, 0, "eval_multi_UBspline_1d_" #T);           \
  }                                                                                                           \
  void eval_multi_UBspline_1d_##T##_vg(multi_UBspline_1d_##T *s, double x, V *vals, V *grads) {               \
    eval_point_ld(s, 1, x, 0.0, vals, grads, (V *)nullptr, 1, "eval_multi_UBspline_1d_" #T "_vg");            \
  }                                                                                                           \
  void eval_multi_UBspline_1d_##T##_vgl(multi_UBspline_1d_##T *s, double x, V *vals, V *grads, V *lapl) {     \
    eval_point_ld(s, 1, x, 0.0, vals, grads, lapl, 2, "eval_multi_UBspline_1d_" #T "_vgl");                   \
  }                                                                                                           \
  void eval_multi_UBspline_1d_##T##_vgh(multi_UBspline_1d_##T *s, double x, V *vals, V *grads, V *hess) {     \
    eval_point_ld(s, 1, x, 0.0, vals, grads, hess, 3, "eval_multi_UBspline_1d_" #T "_vgh");                   \
  }                                                                                                           \
  void eval_multi_UBspline_2d_##T(multi_UBspline_2d_##T *s, double x, double y, V *vals) {                    \
    eval_point_ld(s, 2, x, y, vals, (V *)nullptr, (V *)nullptr, 0, "eval_multi_UBspline_2d_" #T);             \
  }                                                                                                           \
  void eval_multi_UBspline_2d_##T##_vg(multi_UBspline_2d_##T *s, double x, double y, V *vals, V *grads) {     \
    eval_point_ld(s, 2, x, y, vals, grads, (V *)nullptr, 1, "eval_multi_UBspline_2d_" #T "_vg");              \
  }                                                                                                           \
  void eval_multi_UBspline_2d_##T##_vgl(multi_UBspline_2d_##T *s, double x, double y, V *vals, V *grads,      \
                                        V *lapl) {                                                            \
    eval_point_ld(s, 2, x, y, vals, grads, lapl, 2, "eval_multi_UBspline_2d_" #T "_vgl");                     \
  }                                                                                                           \
  void eval_multi_UBspline_2d_##T##_vgh(multi_UBspline_2d_##T *s, double x, double y, V *vals, V *grads,      \
                                        V *hess) {                                                            \
    eval_point_ld(s, 2, x, y, vals, grads, hess, 3, "eval_multi_UBspline_2d_" #T "_vgh");                     \
  }

EG_LD_ENTRIES(s, float)
EG_LD_ENTRIES(d, double)
EG_LD_ENTRIES(c, complex_float)
EG_LD_ENTRIES(z, complex_double)
#undef EG_LD_ENTRIES

void eval_multi_multi_UBspline_1d_s_cuda(multi_UBspline_1d_s_cuda *c, float *pos_d, float *vals_d[], int num) {
  eval_cuda_1d(c, pos_d, false, (void *const *)vals_d, nullptr, nullptr, num, false,
               "eval_multi_multi_UBspline_1d_s_cuda");
}
void eval_multi_multi_UBspline_1d_s_vgl_cuda(multi_UBspline_1d_s_cuda *c, float *pos_d, float *vals_d[],
                                             float *grads_d[], float *lapl_d[], int num) {
  eval_cuda_1d(c, pos_d, false, (void *const *)vals_d, (void *const *)grads_d, (void *const *)lapl_d, num, true,
               "eval_multi_multi_UBspline_1d_s_vgl_cuda");
}
void eval_multi_multi_UBspline_1d_d_cuda(multi_UBspline_1d_d_cuda *c, double *pos_d, double *vals_d[], int num) {
  eval_cuda_1d(c, pos_d, true, (void *const *)vals_d, nullptr, nullptr, num, false,
               "eval_multi_multi_UBspline_1d_d_cuda");
}
void eval_multi_multi_UBspline_1d_d_vgl_cuda(multi_UBspline_1d_d_cuda *c, double *pos_d, double *vals_d[],
                                             double *grads_d[], double *lapl_d[], int num) {
  eval_cuda_1d(c, pos_d, true, (void *const *)vals_d, (void *const *)grads_d, (void *const *)lapl_d, num, true,
               "eval_multi_multi_UBspline_1d_d_vgl_cuda");
}
void eval_multi_multi_UBspline_1d_c_cuda(multi_UBspline_1d_c_cuda *c, float *pos_d, complex_float *vals_d[],
                                         int num) {
  eval_cuda_1d(c, pos_d, false, (void *const *)vals_d, nullptr, nullptr, num, false,
               "eval_multi_multi_UBspline_1d_c_cuda");
}
void eval_multi_multi_UBspline_1d_c_vgl_cuda(multi_UBspline_1d_c_cuda *c, float *pos_d, complex_float *vals_d[],
                                             complex_float *grads_d[], complex_float *lapl_d[], int num) {
  eval_cuda_1d(c, pos_d, false, (void *const *)vals_d, (void *const *)grads_d, (void *const *)lapl_d, num, true,
               "eval_multi_multi_UBspline_1d_c_vgl_cuda");
}
void eval_multi_multi_UBspline_1d_z_cuda(multi_UBspline_1d_z_cuda *c, double *pos_d, complex_double *vals_d[],
                                         int num) {
  eval_cuda_1d(c, pos_d, true, (void *const *)vals_d, nullptr, nullptr, num, false,
               "eval_multi_multi_UBspline_1d_z_cuda");
}
void eval_multi_multi_UBspline_1d_z_vgl_cuda(multi_UBspline_1d_z_cuda *c, double *pos_d, complex_double *vals_d[],
                                             complex_double *grads_d[], complex_double *lapl_d[], int num) {
  eval_cuda_1d(c, pos_d, true, (void *const *)vals_d, (void *const *)grads_d, (void *const *)lapl_d, num, true,
               "eval_multi_multi_UBspline_1d_z_vgl_cuda");
}

}  // extern "C"
