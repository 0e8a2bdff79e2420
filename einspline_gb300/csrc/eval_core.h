// Device building blocks shared by the evaluation kernels (eval.cu) and the
// fused determinant kernels (det.cu): coefficient storage types, the cubic
// B-spline basis, the two cell rules and the separable 4x4x4 reduction.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <type_traits>

#include "eg_internal.h"

namespace eg {

// ------------------------------------------------------------ double-float
// A value carried as an unevaluated sum h + l of two floats (about 48
// significant bits).  Products use the exact FMA residual of h*h' plus the
// cross terms; sums use Knuth's two-sum (Knuth, TAOCP vol. 2, 4.2.2;
// Dekker 1971) on the high parts and collect every rounding error in l.
// The pair is not renormalised after each step: a stencil sum has at most
// 16 terms per stage, so l stays within a few ulps of h and carries its
// errors with 24 bits to spare; the conversion to double at the end adds
// the two parts.  Only round-to-nearest intrinsics are used, so no
// contraction can change the error terms.  For the FP64 tables on GB300,
// whose FP64 pipe is a small fraction of the FP32 one: 12 FP32 operations
// per multiply-add instead of one DFMA.
struct dfl {
  float h, l;
  __host__ __device__ dfl() {}
  __host__ __device__ constexpr dfl(float x) : h(x), l(0.f) {}
  __host__ __device__ constexpr dfl(float a, float b) : h(a), l(b) {}
};

__device__ __forceinline__ dfl operator*(dfl a, dfl b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return dfl(p, e);
}

// c + a * b
__device__ __forceinline__ dfl fmaT(dfl a, dfl b, dfl c) {
  const dfl p = a * b;
  const float s = __fadd_rn(c.h, p.h);
  const float bb = __fsub_rn(s, c.h);
  const float t = __fadd_rn(__fsub_rn(c.h, __fsub_rn(s, bb)), __fsub_rn(p.h, bb));
  return dfl(s, __fadd_rn(t, __fadd_rn(c.l, p.l)));
}

__device__ __forceinline__ dfl to_dfl(double x) {
  const float h = __double2float_rn(x);
  return dfl(h, __double2float_rn(__dsub_rn(x, (double)h)));
}
__device__ __forceinline__ double to_double(dfl x) { return __dadd_rn((double)x.h, (double)x.l); }

// ------------------------------------------------------------ coefficient types
// Raw is what one thread reads per stencil row (VW stored reals); decode
// turns it into VW accumulator values.
template <int ST> struct CT;
template <> struct CT<ST_F32> {
  using A = float;
  using Raw = float4;
  static constexpr int VW = 4, BYTES = 4;
  __device__ static __forceinline__ void decode(const Raw &x, float (&v)[4]) {
    v[0] = x.x; v[1] = x.y; v[2] = x.z; v[3] = x.w;
  }
};
template <> struct CT<ST_F16> {
  using A = float;
  using Raw = uint2;
  static constexpr int VW = 4, BYTES = 2;
  __device__ static __forceinline__ void decode(const Raw &x, float (&v)[4]) {
    const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&x.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&x.y));
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
};
template <> struct CT<ST_BF16> {
  using A = float;
  using Raw = uint2;
  static constexpr int VW = 4, BYTES = 2;
  __device__ static __forceinline__ void decode(const Raw &x, float (&v)[4]) {
    v[0] = __uint_as_float(x.x << 16); v[1] = __uint_as_float(x.x & 0xFFFF0000u);
    v[2] = __uint_as_float(x.y << 16); v[3] = __uint_as_float(x.y & 0xFFFF0000u);
  }
};
template <> struct CT<ST_I16> {
  using A = float;
  using Raw = uint2;
  static constexpr int VW = 4, BYTES = 2;
  // A biased 16-bit pattern u placed under the exponent of 2^23 is the float
  // 2^23 + u; subtracting 2^23 + bias is exact and leaves the integer.
  __device__ static __forceinline__ void decode(const Raw &x, float (&v)[4]) {
    const float off = 8388608.0f + (float)kI16Bias;
    v[0] = __int_as_float(__byte_perm(x.x, 0x4B000000u, 0x7610)) - off;
    v[1] = __int_as_float(__byte_perm(x.x, 0x4B000000u, 0x7632)) - off;
    v[2] = __int_as_float(__byte_perm(x.y, 0x4B000000u, 0x7610)) - off;
    v[3] = __int_as_float(__byte_perm(x.y, 0x4B000000u, 0x7632)) - off;
  }
};
template <> struct CT<ST_F64> {
  using A = double;
  using Raw = double2;
  static constexpr int VW = 2, BYTES = 8;
  __device__ static __forceinline__ void decode(const Raw &x, double (&v)[2]) { v[0] = x.x; v[1] = x.y; }
};

// The double-float shadow of an FP64 table: (hi, lo) per coefficient, two
// columns per 16-byte load, stored as (hi0, hi1, lo0, lo1) so that the high
// and the low parts of a column pair arrive as register pairs.
template <> struct CT<ST_DF> {
  using A = dfl;
  using Raw = float4;
  static constexpr int VW = 2, BYTES = 8;
  __device__ static __forceinline__ void decode(const Raw &x, dfl (&v)[2]) {
    v[0] = dfl(x.x, x.z);
    v[1] = dfl(x.y, x.w);
  }
};

template <int ST>
__device__ __forceinline__ void load_row(const char *p, typename CT<ST>::A (&v)[CT<ST>::VW]) {
  CT<ST>::decode(__ldg(reinterpret_cast<const typename CT<ST>::Raw *>(p)), v);
}


// 16-byte alignment of a device address.
__device__ __forceinline__ bool al16(const void *p) { return (reinterpret_cast<uintptr_t>(p) & 15) == 0; }

__device__ __forceinline__ float fmaT(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double fmaT(double a, double b, double c) { return fma(a, b, c); }

// Cubic B-spline basis at offset t: w[0..3] values, w[4..7] first and
// w[8..11] second derivatives (the 4x4 power-basis matrices of
// src/bspline_data.c:143-162 in Horner form).  The derivative rows carry the
// axis' delta_inv (d) and delta_inv^2, so the reduction yields derivatives
// in position units directly.
template <typename A>
__device__ __forceinline__ void bspline_weights(A t, A *w, A d) {
  const A s6 = A(1) / A(6), t2 = t * t;
  w[0] = fmaT(fmaT(fmaT(-s6, t, A(0.5)), t, A(-0.5)), t, s6);
  w[1] = fmaT(fmaT(A(0.5), t, A(-1)), t2, A(2) / A(3));
  w[2] = fmaT(fmaT(fmaT(A(-0.5), t, A(0.5)), t, A(0.5)), t, s6);
  w[3] = s6 * t2 * t;
  w[4] = fmaT(fmaT(A(-0.5), t, A(1)), t, A(-0.5));
  w[5] = fmaT(A(1.5), t, A(-2)) * t;
  w[6] = fmaT(fmaT(A(-1.5), t, A(1)), t, A(0.5));
  w[7] = A(0.5) * t2;
  w[8] = A(1) - t;
  w[9] = fmaT(A(3), t, A(-2));
  w[10] = fmaT(A(-3), t, A(1));
  w[11] = t;
  const A d2 = d * d;
#pragma unroll
  for (int i = 0; i < 4; i++) {
    w[4 + i] *= d;
    w[8 + i] *= d2;
  }
}

// Cell index and offset along one axis.
//  rule 0 (CPU entries, src/multi_bspline_eval_std_s_impl.h:746-755):
//    u = (x - start) * delta_inv, rounded to float for FP32 tables;
//    i = trunc(u), t = u - i (modf).  Outside the table the edge cell is
//    extrapolated (the reference reads out of bounds there).
//  rule 1 (GPU entries, src/multi_bspline_cuda_s_impl.h:370-384):
//    u = r * delta_inv (no start offset), i = clamp(floor(u), 0, dim-1),
//    t = u - floor(u).
__device__ __forceinline__ void cell(const EvalArgs &a, int ax, double xd, int &idx, float &t) {
  const int lim = a.lim[ax];
  if (a.rule == 0) {
    const float u = __double2float_rn(__dmul_rn(__dsub_rn(xd, a.start[ax]), a.dinv[ax]));
    const float ip = truncf(u);
    float tt = __fsub_rn(u, ip);
    int i = (int)ip;
    if (i < 0) { tt = __fadd_rn(tt, (float)i); i = 0; }
    if (i > lim) { tt = __fadd_rn(tt, (float)(i - lim)); i = lim; }
    idx = i; t = tt;
  } else {
    const float s = __fmul_rn((float)xd, a.dinvf[ax]);
    const float sf = floorf(s);
    int i = (int)sf;
    i = i < 0 ? 0 : (i > lim ? lim : i);
    idx = i; t = __fsub_rn(s, sf);
  }
}
__device__ __forceinline__ void cell(const EvalArgs &a, int ax, double xd, int &idx, double &t) {
  const int lim = a.lim[ax];
  if (a.rule == 0) {
    const double u = __dmul_rn(__dsub_rn(xd, a.start[ax]), a.dinv[ax]);
    const double ip = trunc(u);
    double tt = __dsub_rn(u, ip);
    int i = (int)ip;
    if (i < 0) { tt = __dadd_rn(tt, (double)i); i = 0; }
    if (i > lim) { tt = __dadd_rn(tt, (double)(i - lim)); i = lim; }
    idx = i; t = tt;
  } else {
    const double s = __dmul_rn(xd, a.dinv[ax]);
    const double sf = floor(s);
    int i = (int)sf;
    i = i < 0 ? 0 : (i > lim ? lim : i);
    idx = i; t = __dsub_rn(s, sf);
  }
}

// ------------------------------------------------------------ packed FP32
// Blackwell's 2-wide FP32 instructions (PTX fma.rn.f32x2 / mul.rn.f32x2):
// each lane is the IEEE round-to-nearest operation of the scalar code, so a
// pair of columns sharing one weight costs one instruction instead of two
// and gives bit-identical results.
typedef unsigned long long f32x2;
__device__ __forceinline__ f32x2 pk2(float a, float b) {
  f32x2 r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void upk2(f32x2 r, float &a, float &b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f32x2 fma2(f32x2 a, f32x2 b, f32x2 c) {
  f32x2 d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
  return d;
}
__device__ __forceinline__ f32x2 mul2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

__device__ __forceinline__ f32x2 add2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 sub2(f32x2 a, f32x2 b) {
  f32x2 d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ f32x2 neg2(f32x2 a) { return a ^ 0x8000000080000000ull; }

// Two double-float values (one per column) in packed form: the same
// operations as dfl's, lane by lane.
struct dfl2 {
  f32x2 h, l;
};
__device__ __forceinline__ dfl2 pk2(dfl a, dfl b) { return dfl2{pk2(a.h, b.h), pk2(a.l, b.l)}; }
__device__ __forceinline__ void upk2(dfl2 x, dfl &a, dfl &b) {
  upk2(x.h, a.h, b.h);
  upk2(x.l, a.l, b.l);
}
__device__ __forceinline__ dfl2 mul2(dfl2 a, dfl2 b) {
  const f32x2 p = mul2(a.h, b.h);
  // the exact product error per lane as two scalar FMAs, whose negated
  // addend costs nothing (a packed negation would be two integer operations)
  float a0, a1, b0, b1, p0, p1;
  upk2(a.h, a0, a1);
  upk2(b.h, b0, b1);
  upk2(p, p0, p1);
  f32x2 e = pk2(fmaf(a0, b0, -p0), fmaf(a1, b1, -p1));
  e = fma2(a.h, b.l, e);
  e = fma2(a.l, b.h, e);
  return dfl2{p, e};
}
__device__ __forceinline__ dfl2 fma2(dfl2 a, dfl2 b, dfl2 c) {
  const dfl2 p = mul2(a, b);
  const f32x2 s = add2(c.h, p.h);
  const f32x2 bb = sub2(s, c.h);
  const f32x2 t = add2(sub2(c.h, sub2(s, bb)), sub2(p.h, bb));
  return dfl2{s, add2(t, add2(c.l, p.l))};
}

// Separable reduction of the 4x4x4 stencil for VW columns.
// w: [0..11] x weights, [12..23] y weights, [24..35] z weights.
// o: v, gx, gy, gz, hxx, hxy, hxz, hyy, hyz, hzz.
// One x-plane i: rows (i, j, k) come from row(j, k, c); z first, then y,
// then this plane's x terms go to o.  Every sum starts with a product (no
// accumulator starts at zero): plane 0 assigns o, later planes add to it.
template <typename A, int VW, bool VGH, typename RowFn>
__device__ __forceinline__ void reduce_plane(int i, const A *w, const A (&wz)[3][4], RowFn row, A (&o)[10][VW]) {
  if constexpr ((std::is_same<A, float>::value && VW % 2 == 0) || (std::is_same<A, dfl>::value && VW == 2)) {
    // the same operations on column pairs, two lanes per instruction
    using P = typename std::conditional<std::is_same<A, float>::value, f32x2, dfl2>::type;
    constexpr int H = VW / 2;
    P wz2[3][4];
#pragma unroll
    for (int d = 0; d < 3; d++)
#pragma unroll
      for (int k = 0; k < 4; k++) wz2[d][k] = pk2(wz[d][k], wz[d][k]);
    P y[6][H];
#pragma unroll
    for (int j = 0; j < 4; j++) {
      A c[4][VW];
#pragma unroll
      for (int k = 0; k < 4; k++) row(j, k, c[k]);
      const P by = pk2(w[12 + j], w[12 + j]), dby = pk2(w[16 + j], w[16 + j]), d2by = pk2(w[20 + j], w[20 + j]);
#pragma unroll
      for (int e = 0; e < H; e++) {
        const P c0 = pk2(c[0][2 * e], c[0][2 * e + 1]), c1 = pk2(c[1][2 * e], c[1][2 * e + 1]);
        const P c2 = pk2(c[2][2 * e], c[2][2 * e + 1]), c3 = pk2(c[3][2 * e], c[3][2 * e + 1]);
        P z0 = mul2(c0, wz2[0][0]);
        z0 = fma2(c1, wz2[0][1], z0);
        z0 = fma2(c2, wz2[0][2], z0);
        z0 = fma2(c3, wz2[0][3], z0);
        y[0][e] = j == 0 ? mul2(by, z0) : fma2(by, z0, y[0][e]);
        if (VGH) {
          P z1 = mul2(c0, wz2[1][0]);
          z1 = fma2(c1, wz2[1][1], z1);
          z1 = fma2(c2, wz2[1][2], z1);
          z1 = fma2(c3, wz2[1][3], z1);
          P z2 = mul2(c0, wz2[2][0]);
          z2 = fma2(c1, wz2[2][1], z2);
          z2 = fma2(c2, wz2[2][2], z2);
          z2 = fma2(c3, wz2[2][3], z2);
          if (j == 0) {
            y[1][e] = mul2(dby, z0);
            y[2][e] = mul2(d2by, z0);
            y[3][e] = mul2(by, z1);
            y[4][e] = mul2(dby, z1);
            y[5][e] = mul2(by, z2);
          } else {
            y[1][e] = fma2(dby, z0, y[1][e]);
            y[2][e] = fma2(d2by, z0, y[2][e]);
            y[3][e] = fma2(by, z1, y[3][e]);
            y[4][e] = fma2(dby, z1, y[4][e]);
            y[5][e] = fma2(by, z2, y[5][e]);
          }
        }
      }
    }
    const P ax = pk2(w[i], w[i]), dax = pk2(w[4 + i], w[4 + i]), d2ax = pk2(w[8 + i], w[8 + i]);
    // o[q] += x weight * y[r] for the ten (q, weight, r) of the scalar path
    constexpr int R[10] = {0, 0, 1, 3, 0, 1, 3, 2, 4, 5};
    constexpr int X[10] = {0, 1, 0, 0, 2, 1, 1, 0, 0, 0};
    if (i == 0) {
#pragma unroll
      for (int e = 0; e < H; e++)
#pragma unroll
        for (int q = 0; q < (VGH ? 10 : 1); q++) {
          const P xw = X[q] == 0 ? ax : (X[q] == 1 ? dax : d2ax);
          upk2(mul2(xw, y[R[q]][e]), o[q][2 * e], o[q][2 * e + 1]);
        }
    } else {
#pragma unroll
      for (int e = 0; e < H; e++)
#pragma unroll
        for (int q = 0; q < (VGH ? 10 : 1); q++) {
          const P xw = X[q] == 0 ? ax : (X[q] == 1 ? dax : d2ax);
          upk2(fma2(xw, y[R[q]][e], pk2(o[q][2 * e], o[q][2 * e + 1])), o[q][2 * e], o[q][2 * e + 1]);
        }
    }
    return;
  }
  A y[6][VW];
#pragma unroll
  for (int j = 0; j < 4; j++) {
    A c[4][VW];
#pragma unroll
    for (int k = 0; k < 4; k++) row(j, k, c[k]);
    const A by = w[12 + j], dby = w[16 + j], d2by = w[20 + j];
#pragma unroll
    for (int e = 0; e < VW; e++) {
      A z0 = c[0][e] * wz[0][0];
      z0 = fmaT(c[1][e], wz[0][1], z0);
      z0 = fmaT(c[2][e], wz[0][2], z0);
      z0 = fmaT(c[3][e], wz[0][3], z0);
      y[0][e] = j == 0 ? by * z0 : fmaT(by, z0, y[0][e]);
      if (VGH) {
        A z1 = c[0][e] * wz[1][0];
        z1 = fmaT(c[1][e], wz[1][1], z1);
        z1 = fmaT(c[2][e], wz[1][2], z1);
        z1 = fmaT(c[3][e], wz[1][3], z1);
        A z2 = c[0][e] * wz[2][0];
        z2 = fmaT(c[1][e], wz[2][1], z2);
        z2 = fmaT(c[2][e], wz[2][2], z2);
        z2 = fmaT(c[3][e], wz[2][3], z2);
        if (j == 0) {
          y[1][e] = dby * z0;
          y[2][e] = d2by * z0;
          y[3][e] = by * z1;
          y[4][e] = dby * z1;
          y[5][e] = by * z2;
        } else {
          y[1][e] = fmaT(dby, z0, y[1][e]);
          y[2][e] = fmaT(d2by, z0, y[2][e]);
          y[3][e] = fmaT(by, z1, y[3][e]);
          y[4][e] = fmaT(dby, z1, y[4][e]);
          y[5][e] = fmaT(by, z2, y[5][e]);
        }
      }
    }
  }
  const A ax = w[i], dax = w[4 + i], d2ax = w[8 + i];
  if (i == 0) {
#pragma unroll
    for (int e = 0; e < VW; e++) {
      o[0][e] = ax * y[0][e];
      if (VGH) {
        o[1][e] = dax * y[0][e];
        o[2][e] = ax * y[1][e];
        o[3][e] = ax * y[3][e];
        o[4][e] = d2ax * y[0][e];
        o[5][e] = dax * y[1][e];
        o[6][e] = dax * y[3][e];
        o[7][e] = ax * y[2][e];
        o[8][e] = ax * y[4][e];
        o[9][e] = ax * y[5][e];
      }
    }
    return;
  }
#pragma unroll
  for (int e = 0; e < VW; e++) {
    o[0][e] = fmaT(ax, y[0][e], o[0][e]);
    if (VGH) {
      o[1][e] = fmaT(dax, y[0][e], o[1][e]);
      o[2][e] = fmaT(ax, y[1][e], o[2][e]);
      o[3][e] = fmaT(ax, y[3][e], o[3][e]);
      o[4][e] = fmaT(d2ax, y[0][e], o[4][e]);
      o[5][e] = fmaT(dax, y[1][e], o[5][e]);
      o[6][e] = fmaT(dax, y[3][e], o[6][e]);
      o[7][e] = fmaT(ax, y[2][e], o[7][e]);
      o[8][e] = fmaT(ax, y[4][e], o[8][e]);
      o[9][e] = fmaT(ax, y[5][e], o[9][e]);
    }
  }
}

template <typename A>
__device__ __forceinline__ void z_weights(const A *w, A (&wz)[3][4]) {
#pragma unroll
  for (int d = 0; d < 3; d++)
#pragma unroll
    for (int k = 0; k < 4; k++) wz[d][k] = w[24 + 4 * d + k];
}

// All four planes, rows read straight from global memory.
template <int ST, bool VGH>
__device__ __forceinline__ void contract(const char *base, int64_t xsb, int64_t ysb, int64_t zsb,
                                         const typename CT<ST>::A *w, typename CT<ST>::A (&o)[10][CT<ST>::VW]) {
  using A = typename CT<ST>::A;
  constexpr int VW = CT<ST>::VW;
  A wz[3][4];
  z_weights<A>(w, wz);
#pragma unroll 1
  for (int i = 0; i < 4; i++) {
    const char *plane = base + i * xsb;
    reduce_plane<A, VW, VGH>(i, w, wz, [&](int j, int k, A(&c)[VW]) { load_row<ST>(plane + j * ysb + k * zsb, c); },
                             o);
  }
}

__host__ __device__ __forceinline__ size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Shared memory: pb * 36 weights, pb * 3 cell indices, pb source indices.
__host__ __device__ __forceinline__ size_t smem_w_bytes(int pb, int accb) { return align_up((size_t)pb * 36 * accb, 16); }
__host__ __device__ __forceinline__ size_t smem_total(int pb, int accb) {
  return smem_w_bytes(pb, accb) + align_up((size_t)pb * 3 * 4, 8) + (size_t)pb * 8;
}

// Point group g of a launch (ntiles blocks each): its first point and the
// number of points it may hold.  Groups hold pb points; with pb_tail > 0 the
// groups from g_tail on hold pb_tail, so the blocks that run in the launch's
// last wave are short and the SMs run out of work nearly together.
__device__ __forceinline__ int64_t group_first(const EvalArgs &a, int64_t g) {
  return (a.pb_tail == 0 || g < a.g_tail) ? g * a.pb : a.g_tail * a.pb + (g - a.g_tail) * a.pb_tail;
}
__device__ __forceinline__ int group_cap(const EvalArgs &a, int64_t g) {
  return (a.pb_tail == 0 || g < a.g_tail) ? a.pb : a.pb_tail;
}

// Points' cells, weights and sources into shared memory (evaluation and
// determinant kernels): at most cap points from p0.
template <typename A>
__device__ __forceinline__ int eval_prologue(const EvalArgs &a, unsigned char *smem, int64_t p0, int cap, int tid,
                                             int nthr) {
  A *sw = reinterpret_cast<A *>(smem);
  int *sidx = reinterpret_cast<int *>(smem + smem_w_bytes(a.pb, sizeof(A)));
  int64_t *ssrc = reinterpret_cast<int64_t *>(smem + smem_w_bytes(a.pb, sizeof(A)) + align_up((size_t)a.pb * 12, 8));
  const int pn = (int)min((int64_t)cap, a.npts - p0);
  for (int q = tid; q < pn * 3; q += nthr) {
    const int pp = q / 3, ax = q - 3 * pp;
    const int64_t src = a.perm ? (int64_t)a.perm[p0 + pp] : p0 + pp;
    double xd;
    if (!a.pos) xd = a.inl[ax];
    else if (a.pos_f64) xd = reinterpret_cast<const double *>(a.pos)[3 * src + ax];
    else xd = (double)reinterpret_cast<const float *>(a.pos)[3 * src + ax];
    int idx;
    if constexpr (sizeof(A) == 8 && !std::is_same<A, double>::value) {
      // double-float: FP64 cell and weights carried as hi + lo
      double t, w[12];
      cell(a, ax, xd, idx, t);
      bspline_weights<double>(t, w, a.dinv[ax]);
#pragma unroll
      for (int m = 0; m < 12; m++) sw[pp * 36 + ax * 12 + m] = to_dfl(w[m]);
    } else {
      A t;
      cell(a, ax, xd, idx, t);
      bspline_weights<A>(t, sw + pp * 36 + ax * 12, sizeof(A) == 4 ? (A)a.dinvf[ax] : (A)a.dinv[ax]);
    }
    sidx[pp * 3 + ax] = idx;
    if (ax == 0) ssrc[pp] = src;
  }
  return pn;
}

// Asynchronous global-to-shared copy of RB = 4, 8 or 16 bytes (both
// addresses RB-aligned); 16-byte copies bypass L1.
template <int RB>
__device__ __forceinline__ void cp_async(unsigned dst, const char *src) {
  static_assert(RB == 4 || RB == 8 || RB == 16, "cp.async copies 4, 8 or 16 bytes");
  if constexpr (RB == 16) asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
  else if constexpr (RB == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

constexpr int kPipeStages = 3;
__host__ __device__ __forceinline__ size_t pipe_bytes(int nthr, int rb, int stages = kPipeStages) {
  return (size_t)stages * 16 * nthr * rb;
}
// Stages of the evaluation copy pipeline per kernel: the double-float
// reduction spends long enough on each stage that one stage in flight hides
// the loads, and the smaller buffers let more warps share an SM; the wide
// 16-bit kernel (one warp a block, 8 blocks an SM by registers) is as well
// served by one stage in flight, and its smaller buffers leave more of the
// SM's memory to L1 (measured 1-2 % faster on GB300).
__host__ __device__ constexpr int pipe_stages(int st, bool wide) { return (wide || st == ST_DF) ? 2 : kPipeStages; }

// ------------------------------------------------------------ tensor-map copies
// Stages of the TMA pipeline and its shared memory: the block's weights and
// indices, 128-byte alignment slack, the stage buffers (16 rows of 16 bytes
// a thread) and one full and one empty mbarrier per stage.
constexpr int kTmaStages = 3;
// The double-float reduction is arithmetic-bound: two stages and more
// resident warps, as in its copy pipeline.
template <int ST>
struct TmaStages { static constexpr int value = kTmaStages; };
template <>
struct TmaStages<ST_DF> { static constexpr int value = 2; };
__host__ __device__ __forceinline__ size_t tma_smem(int pb, int accb, int nthr, int stages) {
  return smem_total(pb, accb) + 128 + (size_t)stages * 16 * 16 * nthr + 2 * stages * 8;
}
// Longest wait on one mbarrier phase before the kernel gives up: a stage's
// copy normally lands within microseconds.
constexpr unsigned long long kWaitNs = 500000000ull;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_arrive(unsigned bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
// Arrives and adds the bytes the phase's copies will deliver.
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
// Waits until the phase of the given parity has completed; false when
// limit_ns of global time passed first.
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity, unsigned long long limit_ns = kWaitNs) {
  unsigned long long t0 = 0;
  for (unsigned n = 1;; n++) {
    unsigned done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if ((n & 63) == 0) {
      const unsigned long long now = global_ns();
      if (n == 64) t0 = now;
      else if (now - t0 > limit_ns) return false;
    }
  }
}
// Brings a tensor map (kernel parameter) into the descriptor cache.
__device__ __forceinline__ void tma_prefetch_map(const CUtensorMap *map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}
// One tiled 4D tensor-map copy into shared memory, completing on mbarrier
// bar; c0 is the innermost (column) coordinate.
__device__ __forceinline__ void tma_load_4d(unsigned dst, const CUtensorMap *map, unsigned bar, int c0, int c1,
                                            int c2, int c3) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5, %6}], [%2];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar), "r"(c0), "r"(c1), "r"(c2), "r"(c3)
      : "memory");
}


// ------------------------------------------------------------ tensor cores
// Shared-memory matrix descriptor of a tcgen05.mma operand: start address,
// leading and stride byte offsets (16-byte units), descriptor version 1 and
// the swizzle mode (0 none, 2 128-byte).  For an MN-major operand in the
// 128-byte swizzle the leading offset steps between 64-element atoms along
// M or N and the stride offset between groups of 8 rows along K; for a
// K-major operand without swizzle, core matrices are 8 rows of 16 bytes,
// the leading offset steps along K and the stride offset along M or N.
__device__ __forceinline__ uint64_t umma_desc(unsigned addr, unsigned lbo, unsigned sbo, unsigned swizzle) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | (uint64_t)((lbo >> 4) & 0x3FFFu) << 16 |
         (uint64_t)((sbo >> 4) & 0x3FFFu) << 32 | (uint64_t)1 << 46 | (uint64_t)(swizzle & 7u) << 61;
}
// Instruction descriptor of a kind::f16 MMA: A and B both f16 (fmt 0) or
// both bf16 (fmt 1), f32 accumulator, A MN-major, B K-major, shape M x N.
__host__ __device__ constexpr uint32_t umma_idesc_16(int M, int N, uint32_t fmt) {
  return (1u << 4) | (fmt << 7) | (fmt << 10) | (1u << 15) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// D[tmem] (+)= A * B for one K = 16 step, issued by one thread.
__device__ __forceinline__ void umma_f16(unsigned tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"((unsigned)acc)
      : "memory");
}
// Arrives once on mbarrier bar when every MMA this thread issued so far is complete.
__device__ __forceinline__ void umma_commit(unsigned bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// Orders this thread's generic shared-memory writes before later reads of
// the same memory by the async proxy (tensor cores, bulk copies).
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// 32 consecutive accumulator columns of this thread's TMEM lane (the warp
// reads lanes 32 * (warp % 4) .. + 31).
__device__ __forceinline__ void tmem_ld32(unsigned taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld16(unsigned taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_ld2(unsigned taddr, uint32_t (&r)[2]) {
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x2.b32 {%0,%1}, [%2];" : "=r"(r[0]), "=r"(r[1]) : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// Tensor-core evaluation (load mode 5, F16 and BF16 tables).  A block owns
// kTcTiles tiles of 128 columns (each the M of one MMA).  Shared memory: the
// points' weights, cells and sources; slack to align the operand area to
// 1024 bytes (the 128-byte swizzle atom); kTcStages stencil buffers,
// each 64 rows x 128 16-bit columns of one tile (16 KB, two 8 KB boxes of 64
// columns); two weight buffers of four 32 x 16 K-major tiles, one per
// x-plane (4 KB: output q's weight parts in columns parts * q + h);
// mbarriers (two per stage, one per weight buffer, two per accumulator);
// the TMEM address, an abort flag and a count.
constexpr int kTcTiles = 2;
constexpr int kTcCols = 128 * kTcTiles;  // columns per block
constexpr int kTcN = 32;                 // 10 outputs x weight parts (<= 3), padded to the MMA's N
constexpr int kTcThreads = 192;          // copy warp, MMA warp, 4 weight/output warps
constexpr int kTcStages = 4;             // stencil stages, one 128-column tile of a point each
// Per table type: an FP32 weight is the sum of two f16 parts (22 bits) or of
// three bf16 parts (exactly: 3 x 8 bits), each part accumulating in its own
// column, summed in the epilogue.
template <int ST> struct TcCfg {
  static constexpr int parts = ST == ST_BF16 ? 3 : 2;
  static constexpr uint32_t fmt = ST == ST_BF16 ? 1u : 0u;
};
__host__ __device__ __forceinline__ size_t tc_smem(int pb) {
  return smem_total(pb, 4) + 1024 + (size_t)kTcStages * 16384 + 2 * 4096 + 16 * kTcStages + 48 + 16;
}

}  // namespace eg
