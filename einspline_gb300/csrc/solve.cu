// Coefficient solve for set_multi_UBspline_3d_*: batched FP64 tridiagonal
// (cyclic for periodic/antiperiodic) solves on the GPU, three sweeps x, y, z
// (src/multi_bspline_create.c:345-372 and :1042-1072), rounded once on store.
//
// Every line along an axis shares the same band matrix (1/6, 2/3, 1/6 plus
// the boundary rows), so its elimination does not depend on the data.  The
// host runs the reference elimination on the band coefficients alone
// (src/bspline_create.c:959-1111) and records each multiplier and divisor;
// the device then pushes every right-hand side through the recorded steps
// in the reference's order with IEEE double operations and no FMA
// contraction, which makes the FP64 tables bit-identical to the reference's
// set_multi_UBspline_3d_d / _z.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <math.h>

#include <cmath>
#include <stdio.h>
#include <string.h>

#include <algorithm>

#include "eg_internal.h"

namespace eg {

// ------------------------------------------------------------------
// Host factorization
// ------------------------------------------------------------------
static void bc_row(int code, double val, double dinv, double row[4]) {
  // src/bspline_create.c:1138-1174: first-derivative rows for DERIV1/FLAT,
  // second-derivative rows for DERIV2/NATURAL; FLAT/NATURAL force val = 0.
  if (code == FLAT || code == NATURAL) val = 0.0;
  if (code == FLAT || code == DERIV1) {
    row[0] = -0.5 * dinv; row[1] = 0.0 * dinv; row[2] = 0.5 * dinv; row[3] = val;
  } else {
    row[0] = 1.0 * dinv * dinv; row[1] = -2.0 * dinv * dinv; row[2] = 1.0 * dinv * dinv; row[3] = val;
  }
}

void build_line_factors(int M, int lcode, int rcode, double dinv, LineFactors &f) {
  f.M = M;
  f.lcode = lcode;
  f.rcode = rcode;
  f.cyclic = (lcode == PERIODIC || lcode == ANTIPERIODIC);
  f.anti = (lcode == ANTIPERIODIC);
  f.P.assign(M + 2, 0.0); f.L.assign(M + 2, 0.0); f.E.assign(M + 2, 0.0);
  f.U.assign(M + 2, 0.0); f.LC.assign(M + 2, 0.0);
  const double basis[3] = {1.0 / 6.0, 2.0 / 3.0, 1.0 / 6.0};
  if (f.cyclic) {
    // Elimination of src/bspline_create.c:1010-1055 / :1064-1111 without the
    // right-hand side column.
    std::vector<double> b(4 * M, 0.0), lastCol(M, 0.0);
    for (int i = 0; i < M; i++) { b[4*i] = basis[0]; b[4*i+1] = basis[1]; b[4*i+2] = basis[2]; }
    if (f.anti) { b[0] *= -1.0; b[4*(M-1)+2] *= -1.0; }
    f.P[0] = b[1];                       // d0 /= P[0]
    b[2] /= b[1];
    b[0] /= b[1];
    b[1] = 1.0;
    b[4*(M-1)+1] -= b[4*(M-1)+2] * b[0];
    f.E[0] = b[4*(M-1)+2];               // dlast -= E[0] * d0
    b[4*(M-1)+2] = -b[4*(M-1)+2] * b[2];
    lastCol[0] = b[0];
    for (int r = 1; r < M - 1; r++) {
      double *row = &b[4*r], *up = &b[4*(r-1)], *last = &b[4*(M-1)];
      row[1] -= row[0] * up[2];
      f.L[r] = row[0];                   // d_r -= L[r] * d_{r-1}
      lastCol[r] = -row[0] * lastCol[r-1];
      row[0] = 0.0;
      row[2] /= row[1];
      f.P[r] = row[1];                   // d_r /= P[r]
      lastCol[r] /= row[1];
      row[1] = 1.0;
      if (r < M - 2) {
        f.E[r] = last[2];                // dlast -= E[r] * d_r
        last[1] -= last[2] * lastCol[r];
        last[2] = -last[2] * row[2];
      }
    }
    b[4*(M-1)+0] += b[4*(M-1)+2];
    b[4*(M-1)+1] -= b[4*(M-1)+0] * (b[4*(M-2)+2] + lastCol[M-2]);
    f.F = b[4*(M-1)+0];                  // dlast -= F * d_{M-2}
    f.Q = b[4*(M-1)+1];                  // dlast /= Q
    for (int r = 0; r <= M - 2; r++) { f.U[r] = b[4*r+2]; f.LC[r] = lastCol[r]; }
  } else {
    // Elimination of src/bspline_create.c:959-1001 without the RHS column.
    std::vector<double> b(4 * (M + 2), 0.0);
    bc_row(lcode, 0.0, dinv, &b[0]);
    bc_row(rcode, 0.0, dinv, &b[4*(M+1)]);
    for (int i = 0; i < M; i++) { b[4*(i+1)] = basis[0]; b[4*(i+1)+1] = basis[1]; b[4*(i+1)+2] = basis[2]; }
    f.P[0] = b[0];                       // d0 = lval / P[0]
    b[1] /= b[0];
    b[2] /= b[0];
    b[0] = 1.0;
    b[4+1] -= b[4+0] * b[1];
    b[4+2] -= b[4+0] * b[2];
    f.L[1] = b[4+0];                     // d1 = data0 - L[1] * d0
    b[0] = 0.0;
    b[4+2] /= b[4+1];
    f.P[1] = b[4+1];                     // d1 /= P[1]
    b[4+1] = 1.0;
    for (int r = 2; r < M + 1; r++) {
      double *row = &b[4*r], *up = &b[4*(r-1)];
      row[1] -= row[0] * up[2];
      f.L[r] = row[0];
      row[2] /= row[1];
      f.P[r] = row[1];
      row[0] = 0.0;
      row[1] = 1.0;
    }
    double *last = &b[4*(M+1)];
    f.R0 = last[0];                      // dM1 -= R0 * d_{M-1}
    last[1] -= last[0] * b[4*(M-1)+2];
    f.R1 = last[1];                      // dM1 -= R1 * d_M
    last[2] -= last[1] * b[4*M+2];
    f.Q = last[2];                       // dM1 /= Q
    for (int r = 1; r <= M; r++) f.U[r] = b[4*r+2];
    f.U0a = b[1];
    f.U0b = b[2];
  }
}

size_t packed_factor_doubles(int M) { return sizeof(PackedFactors) / sizeof(double) + 7 * (size_t)(M + 2); }

// A divisor's reciprocal as hi + lo: hi = RN(1/b), lo = RN((1 - b*hi)/b)
// (1 - b*hi is exact by FMA).  hi = lo = 0 marks a divisor outside
// [2^-64, 2^64] (or zero), which the device divides directly.
static void split_reciprocal(double b, double &hi, double &lo) {
  const double a = std::fabs(b);
  if (!(a >= 0x1p-64 && a <= 0x1p64)) { hi = lo = 0.0; return; }
  hi = 1.0 / b;
  lo = std::fma(-b, hi, 1.0) / b;
}

void pack_line_factors(const LineFactors &f, std::vector<double> &out) {
  const int n = f.M + 2;
  out.assign(packed_factor_doubles(f.M), 0.0);
  PackedFactors h;
  memset(&h, 0, sizeof(h));
  h.M = f.M; h.cyclic = f.cyclic; h.anti = f.anti;
  h.F = f.F; h.Q = f.Q; h.R0 = f.R0; h.R1 = f.R1; h.U0a = f.U0a; h.U0b = f.U0b;
  split_reciprocal(f.Q, h.QH, h.QL);
  memcpy(out.data(), &h, sizeof(h));
  double *p = out.data() + sizeof(PackedFactors) / sizeof(double);
  std::copy(f.P.begin(), f.P.end(), p + 0 * n);
  std::copy(f.L.begin(), f.L.end(), p + 1 * n);
  std::copy(f.E.begin(), f.E.end(), p + 2 * n);
  std::copy(f.U.begin(), f.U.end(), p + 3 * n);
  std::copy(f.LC.begin(), f.LC.end(), p + 4 * n);
  for (size_t i = 0; i < f.P.size(); i++) split_reciprocal(f.P[i], p[5 * n + i], p[6 * n + i]);
}

// ------------------------------------------------------------------
// Right-hand-side solve of one line, shared by host self-test and device.
// ------------------------------------------------------------------
__host__ __device__ __forceinline__ double dmul(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dmul_rn(a, b);
#else
  return a * b;  // host side is compiled with -ffp-contract=off
#endif
}
__host__ __device__ __forceinline__ double dsub(double a, double b) {
#ifdef __CUDA_ARCH__
  return __dsub_rn(a, b);
#else
  return a - b;
#endif
}
// a / b correctly rounded, b a band divisor known in advance with its
// reciprocal split as zh + zl (split_reciprocal).  On the device:
// q0 = a*zh + a*zl is within one ulp of a/b, the remainder r = a - b*q0 is
// exact by FMA, and RN(q0 + r*zh) is the correctly rounded quotient
// (Markstein's correction step: P. Markstein, IBM J. Res. Dev. 34(1), 1990;
// the reciprocal known in advance as in N. Brisebarre, J.-M. Muller and
// S. K. Raina, IEEE Trans. Computers 53(8), 2004): four FP64 operations
// instead of a full division, the same bits.  Numerators outside
// [2^-823, 2^825) in magnitude (zeros, subnormals, near overflow) and
// divisors without a split take the IEEE division, so every intermediate
// stays normal.  The host divides directly.
__host__ __device__ __forceinline__ double ddiv(double a, double b, double zh, double zl) {
#ifdef __CUDA_ARCH__
  const unsigned ea = ((unsigned)__double2hiint(a) >> 20) & 0x7FFu;
  if (ea < 200u || ea > 1847u || __double2hiint(zh) == 0) return __ddiv_rn(a, b);
  const double q0 = __fma_rn(a, zh, __dmul_rn(a, zl));
  const double r = __fma_rn(-q0, b, a);
  return __fma_rn(r, zh, q0);
#else
  (void)zh; (void)zl;
  return a / b;
#endif
}

// in[i*is] for i < M (data), out[i*os] for i < N (coefficients); in and out
// may be the same line (in-place sweeps): every input element is read before
// the output element at the same place is written.
__host__ __device__ inline void solve_line(const double *pk, const double *in, int64_t is,
                                           double *out, int64_t os, double lval, double rval) {
  const PackedFactors &h = *reinterpret_cast<const PackedFactors *>(pk);
  const int M = h.M, n = M + 2;
  const double *P = pk + sizeof(PackedFactors) / sizeof(double);
  const double *L = P + n, *E = P + 2 * n, *U = P + 3 * n, *LC = P + 4 * n, *RH = P + 5 * n, *RL = P + 6 * n;
  if (h.cyclic) {
    double dl = in[(int64_t)(M - 1) * is];
    double nxt = in[1 * is];
    double d = ddiv(in[0], P[0], RH[0], RL[0]);
    dl = dsub(dl, dmul(E[0], d));
    out[1 * os] = d;
    double prev = d;
    for (int r = 1; r < M - 1; r++) {
      double cur = nxt;
      nxt = in[(int64_t)(r + 1) * is];
      d = ddiv(dsub(cur, dmul(L[r], prev)), P[r], RH[r], RL[r]);
      out[(int64_t)(r + 1) * os] = d;
      if (r < M - 2) dl = dsub(dl, dmul(E[r], d));
      prev = d;
    }
    dl = dsub(dl, dmul(h.F, prev));
    dl = ddiv(dl, h.Q, h.QH, h.QL);
    const double cM = dl;
    out[(int64_t)M * os] = cM;
    double cn = cM, c1 = 0.0, c2 = 0.0;
    for (int r = M - 2; r >= 0; r--) {
      double c = dsub(dsub(out[(int64_t)(r + 1) * os], dmul(U[r], cn)), dmul(LC[r], cM));
      out[(int64_t)(r + 1) * os] = c;
      if (r == 1) c2 = c;
      if (r == 0) c1 = c;
      cn = c;
    }
    if (M - 2 < 1) c2 = out[2 * os];
    if (h.anti) {
      out[0] = -cM;
      out[(int64_t)(M + 1) * os] = -c1;
      out[(int64_t)(M + 2) * os] = -c2;
    } else {
      out[0] = cM;
      out[(int64_t)(M + 1) * os] = c1;
      out[(int64_t)(M + 2) * os] = c2;
    }
  } else {
    double nxt = in[0];
    double d0 = ddiv(lval, P[0], RH[0], RL[0]);
    out[0] = d0;
    double prev = d0, prev2 = 0.0;
    for (int r = 1; r <= M; r++) {
      double cur = nxt;
      if (r <= M - 1) nxt = in[(int64_t)r * is];
      double d = (r == 1) ? ddiv(dsub(cur, dmul(L[1], d0)), P[1], RH[1], RL[1])
                          : ddiv(dsub(cur, dmul(L[r], prev)), P[r], RH[r], RL[r]);
      out[(int64_t)r * os] = d;
      prev2 = prev;
      prev = d;
    }
    // prev = d_M, prev2 = d_{M-1}
    double dm1 = dsub(rval, dmul(h.R0, prev2));
    dm1 = dsub(dm1, dmul(h.R1, prev));
    dm1 = ddiv(dm1, h.Q, h.QH, h.QL);
    out[(int64_t)(M + 1) * os] = dm1;
    double cn = dm1;
    for (int r = M; r > 0; r--) {
      double c = dsub(out[(int64_t)r * os], dmul(U[r], cn));
      out[(int64_t)r * os] = c;
      cn = c;
    }
    out[0] = dsub(dsub(out[0], dmul(h.U0a, out[1 * os])), dmul(h.U0b, out[2 * os]));
  }
}

// ------------------------------------------------------------------
// Device kernels
// ------------------------------------------------------------------
// staging [n][P][nc] (input type) -> A [P][n*nc] double, 32x32 tiles.
template <typename Tin, int NC>
__global__ void k_stage_transpose(const Tin *__restrict__ stg, int64_t P, int n, double *__restrict__ A) {
  __shared__ double tile[32][33 * NC];
  const int64_t e0 = (int64_t)blockIdx.x * 32;
  const int s0 = blockIdx.y * 32;
  for (int s = threadIdx.y; s < 32; s += 8) {
    const int slot = s0 + s;
    const int64_t e = e0 + threadIdx.x;
    for (int p = 0; p < NC; p++)
      tile[s][threadIdx.x * NC + p] = (slot < n && e < P) ? (double)stg[((int64_t)slot * P + e) * NC + p] : 0.0;
  }
  __syncthreads();
  const int64_t ncw = (int64_t)n * NC;
  for (int s = threadIdx.y; s < 32; s += 8) {
    const int64_t e = e0 + s;
    const int slot = s0 + threadIdx.x;
    if (e < P && slot < n)
      for (int p = 0; p < NC; p++) A[e * ncw + (int64_t)slot * NC + p] = tile[threadIdx.x][s * NC + p];
  }
}

struct SweepArgs {
  const double *fac;
  const double *in;
  double *out;
  int64_t in_su, in_sv, out_su, out_sv, in_stride, out_stride;
  int nv;
  int64_t nlines;
  int ncw, ncomp;
  double lval[2], rval[2];
};

__global__ void k_sweep(const SweepArgs a) {
  const int cblocks = (a.ncw + blockDim.x - 1) / blockDim.x;
  const int64_t line = blockIdx.x / cblocks;
  const int c = (int)(blockIdx.x % cblocks) * blockDim.x + threadIdx.x;
  if (line >= a.nlines || c >= a.ncw) return;
  const int64_t u = line / a.nv, v = line % a.nv;
  const int p = c % a.ncomp;
  const double *in = a.in + u * a.in_su + v * a.in_sv + c;
  double *out = a.out + u * a.out_su + v * a.out_sv + c;
  solve_line(a.fac, in, a.in_stride, out, a.out_stride, a.lval[p], a.rval[p]);
}

__global__ void k_colmax(const double *__restrict__ W, int64_t ncells, int ncw, unsigned int *colmax) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncw) return;
  float m = 0.f;
  for (int64_t e = blockIdx.y; e < ncells; e += gridDim.y) m = fmaxf(m, (float)fabs(W[e * ncw + c]));
  atomicMax(colmax + c, __float_as_uint(m));
}

// Per-spline factor for 16-bit storage, from the largest |coefficient| m:
//   F16: m * inv just under 65504 (the largest finite half), using the whole
//        half range;
//   I16: m * inv = 32767, so coefficients become integers in [-32767, 32767];
//   BF16: inv = 2^(15-e) with m = f * 2^e, f in [0.5, 1) (the exponent range
//        of bfloat16 needs no scaling; a power of two keeps it exact).
// The stored value is round(c * inv); evaluation multiplies by scale = 1/inv.
__device__ __forceinline__ void choose_scale(int st, float m, float *scale, double *inv) {
  if (!(m > 0.f)) { *scale = 1.0f; *inv = 1.0; return; }
  double iv;
  if (st == ST_F16) iv = (65504.0 * (1.0 - 1.0 / 1048576.0)) / (double)m;
  else if (st == ST_I16) iv = 32767.0 / (double)m;
  else {
    int e = 0;
    frexpf(m, &e);
    iv = ldexp(1.0, 15 - e);
  }
  *inv = iv;
  *scale = __double2float_rn(1.0 / iv);
}

__global__ void k_scales(int st, const unsigned int *colmax, int nslots, int ncomp, const int *slot_spline,
                         float *scale, double *inv_out) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nslots) return;
  float m = 0.f;
  for (int p = 0; p < ncomp; p++) m = fmaxf(m, __uint_as_float(colmax[s * ncomp + p]));
  float sc;
  double iv;
  choose_scale(st, m, &sc, &iv);
  for (int p = 0; p < ncomp; p++) {
    scale[(slot_spline ? slot_spline[s] : s) * ncomp + p] = sc;
    inv_out[s * ncomp + p] = iv;
  }
}

// Rounds one FP64 coefficient to the storage type at table[o].
template <int ST>
__device__ __forceinline__ void store_coef(void *table, int64_t o, double w, double inv) {
  if (ST == ST_F64) ((double *)table)[o] = w;
  else if (ST == ST_F32) ((float *)table)[o] = __double2float_rn(w);
  else if (ST == ST_F16) ((__half *)table)[o] = __double2half(w * inv);
  else if (ST == ST_BF16) ((__nv_bfloat16 *)table)[o] = __double2bfloat16(w * inv);
  else {
    double q = rint(w * inv);
    q = fmin(fmax(q, -32767.0), 32767.0);
    ((unsigned short *)table)[o] = (unsigned short)((int)q + kI16Bias);
  }
}

template <int ST>
__global__ void k_store(const double *__restrict__ W, int64_t ncells, int ncw, int ncomp,
                        const int *__restrict__ slot_spline, const double *__restrict__ inv,
                        void *__restrict__ table, int64_t zs) {
  const int cblocks = (ncw + blockDim.x - 1) / blockDim.x;
  const int64_t cell = blockIdx.x / cblocks;
  const int c = (int)(blockIdx.x % cblocks) * blockDim.x + threadIdx.x;
  if (cell >= ncells || c >= ncw) return;
  const double w = W[cell * ncw + c];
  const int64_t tcol = (int64_t)slot_spline[c / ncomp] * ncomp + (c % ncomp);
  store_coef<ST>(table, cell * zs + tcol, w, is16(ST) ? inv[c] : 1.0);
}

__global__ void k_fill_f32(float *p, int64_t n, float v) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

// ------------------------------------------------------------------
// Table objects
// ------------------------------------------------------------------
static int resolve_storage(char kind, int storage) {
  if (kind == 'd' || kind == 'z') return (storage == ST_NATIVE || storage == ST_F64) ? ST_F64 : -1;
  if (storage == ST_NATIVE) return ST_F32;
  if (storage == ST_F32 || is16(storage)) return storage;
  return -1;
}

static int storage_bytes(int st) { return st == ST_F64 ? 8 : (st == ST_F32 ? 4 : 2); }

static int alloc_storage(Table *t) {
  t->ncol = t->ncomp * t->num_splines;
  const int per_row = 128 / t->elem_bytes;
  t->ncol_pad = (t->ncol + per_row - 1) / per_row * per_row;
  t->zs = t->ncol_pad;
  t->ys = (int64_t)t->Nc[2] * t->zs;
  t->xs = (int64_t)t->Nc[1] * t->ys;
  t->table_bytes = (size_t)t->Nc[0] * (size_t)t->xs * (size_t)t->elem_bytes;
  cudaError_t e = cudaMalloc(&t->coefs, t->table_bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    t->coefs = nullptr;
    return fail(EINSPLINE_GB300_ENOMEM, "cannot allocate %zu bytes of device memory for the coefficient table (%s)",
                t->table_bytes, cudaGetErrorString(e));
  }
  EG_CUDA(cudaMemsetAsync(t->coefs, 0, t->table_bytes, t->stream));
  if (is16(t->storage)) {
    EG_CUDA(cudaMalloc(&t->scale, sizeof(float) * t->ncol_pad));
    k_fill_f32<<<(t->ncol_pad + 255) / 256, 256, 0, t->stream>>>(t->scale, t->ncol_pad, 1.0f);
    count_launch();
    EG_CUDA(cudaGetLastError());
  }
  return 0;
}

Table *table_create(char kind, const GridDesc g[3], int num_splines, int storage, int dims) {
  if (num_splines < 1) { fail(EINSPLINE_GB300_EINVAL, "num_splines must be >= 1 (got %d)", num_splines); return nullptr; }
  if (dims < 1 || dims > 3) { fail(EINSPLINE_GB300_EINVAL, "dims must be 1, 2 or 3"); return nullptr; }
  const int st = resolve_storage(kind, storage);
  if (st < 0) { fail(EINSPLINE_GB300_EINVAL, "storage %d is not available for type %c", storage, kind); return nullptr; }
  for (int a = 0; a < dims; a++) {
    // Only lCode decides between the cyclic and boundary-row systems, as in
    // src/bspline_create.c:1120; rCode matters only for the latter.
    const bool cyc = (g[a].lcode == PERIODIC || g[a].lcode == ANTIPERIODIC);
    if (g[a].lcode < PERIODIC || g[a].lcode > ANTIPERIODIC ||
        (!cyc && (g[a].rcode < PERIODIC || g[a].rcode > ANTIPERIODIC || g[a].rcode == PERIODIC ||
                  g[a].rcode == ANTIPERIODIC))) {
      fail(EINSPLINE_GB300_EINVAL, "axis %d: invalid boundary condition code", a);
      return nullptr;
    }
    if (g[a].num < (cyc ? 4 : 3)) {
      fail(EINSPLINE_GB300_EINVAL, "axis %d: need at least %d grid points (got %d)", a, cyc ? 4 : 3, g[a].num);
      return nullptr;
    }
    if (!(g[a].end > g[a].start)) { fail(EINSPLINE_GB300_EINVAL, "axis %d: end must exceed start", a); return nullptr; }
  }
  Table *t = new Table();
  t->kind = kind;
  t->ncomp = (kind == 'c' || kind == 'z') ? 2 : 1;
  t->storage = st;
  t->elem_bytes = storage_bytes(st);
  t->in_bytes = (kind == 's' || kind == 'c') ? 4 : 8;
  t->num_splines = num_splines;
  t->dims = dims;
  for (int a = dims; a < 3; a++) {
    // an absent axis: one point, one coefficient, never swept or evaluated
    t->M[a] = 1; t->Nc[a] = 1;
    t->start[a] = 0.0; t->end[a] = 1.0; t->delta[a] = 1.0; t->dinv[a] = 1.0;
    t->lcode[a] = t->rcode[a] = -1;
    for (int p = 0; p < 2; p++) t->lval[a][p] = t->rval[a][p] = 0.0;
  }
  for (int a = 0; a < dims; a++) {
    t->M[a] = g[a].num;
    const bool cyc = (g[a].lcode == PERIODIC || g[a].lcode == ANTIPERIODIC);
    t->Nc[a] = cyc ? g[a].num + 3 : g[a].num + 2;
    t->start[a] = g[a].start;
    t->end[a] = g[a].end;
    // src/multi_bspline_create.c:273-275
    t->delta[a] = (g[a].end - g[a].start) / (double)(t->Nc[a] - 3);
    t->dinv[a] = 1.0 / t->delta[a];
    t->lcode[a] = g[a].lcode;
    t->rcode[a] = g[a].rcode;
    for (int p = 0; p < 2; p++) { t->lval[a][p] = g[a].lval[p]; t->rval[a][p] = g[a].rval[p]; }
  }
  if (cudaStreamCreate(&t->stream) != cudaSuccess) {
    cudaGetLastError();
    fail(EINSPLINE_GB300_ECUDA, "cudaStreamCreate failed");
    delete t;
    return nullptr;
  }
  if (alloc_storage(t)) { table_destroy(t); return nullptr; }
  if (cudaHostAlloc((void **)&t->wait_err_h, sizeof(int), cudaHostAllocMapped) != cudaSuccess ||
      cudaHostGetDevicePointer((void **)&t->wait_err_d, t->wait_err_h, 0) != cudaSuccess) {
    cudaGetLastError();
    fail(EINSPLINE_GB300_ENOMEM, "cannot allocate the wait-status word");
    table_destroy(t);
    return nullptr;
  }
  *t->wait_err_h = 0;
  // Line factors for the axes, packed into one device buffer.
  std::vector<double> all, one;
  for (int a = 0; a < dims; a++) {
    LineFactors f;
    build_line_factors(t->M[a], t->lcode[a], t->rcode[a], t->dinv[a], f);
    pack_line_factors(f, one);
    t->factor_off[a] = all.size();
    all.insert(all.end(), one.begin(), one.end());
  }
  if (cudaMalloc(&t->factors_d, all.size() * sizeof(double)) != cudaSuccess ||
      cudaMemcpy(t->factors_d, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
    cudaGetLastError();
    fail(EINSPLINE_GB300_ECUDA, "cannot upload line factors");
    table_destroy(t);
    return nullptr;
  }
  // Splines per batched solve: FP64 work space bounded by a budget.
  const double pts = (double)t->M[0] * t->M[1] * t->M[2];
  const double cells = (double)t->Nc[0] * t->Nc[1] * t->Nc[2];
  const double per = t->ncomp * (pts * t->in_bytes + pts * 8.0 + cells * 8.0);
  double budget = 4.0 * 1024 * 1024 * 1024;
  if (const char *env = getenv("EINSPLINE_GB300_SOLVE_BUDGET_MB")) budget = atof(env) * 1024.0 * 1024.0;
  t->cap = (int)std::max(1.0, std::min((double)num_splines, floor(budget / per)));
  if (cudaStreamSynchronize(t->stream) != cudaSuccess) {
    cuda_check(cudaGetLastError(), "table initialisation");
    table_destroy(t);
    return nullptr;
  }
  return t;
}

static void free_work(Table *t) {
  cudaFree(t->staging); cudaFree(t->work_a); cudaFree(t->work_w); cudaFree(t->colmax); cudaFree(t->slot_spline_d);
  t->staging = nullptr; t->work_a = t->work_w = nullptr; t->colmax = nullptr; t->slot_spline_d = nullptr;
}

void table_destroy(Table *t) {
  if (!t) return;
  if (t->stream) cudaStreamSynchronize(t->stream);
  free_work(t);
  if (t->owns) cudaFree(t->coefs);
  cudaFree(t->scale);
  cudaFree(t->df_coefs);
  cudaFree(t->factors_d);
  if (t->pt_host) cudaFreeHost(t->pt_host);  // pt_dev is its device address
  if (t->host_coefs) cudaFreeHost(t->host_coefs);
  if (t->wait_err_h) cudaFreeHost(t->wait_err_h);
  cudaFree(t->pipe_dev);
  cudaFree(t->sort_dev);
  for (int i = 0; i < 2; i++) {
    if (t->pipe_stream[i]) cudaStreamDestroy(t->pipe_stream[i]);
    if (t->pipe_event[i]) cudaEventDestroy(t->pipe_event[i]);
  }
  if (t->stream) cudaStreamDestroy(t->stream);
  t->magic = 0;
  delete t;
  cudaGetLastError();
}

static int ensure_work(Table *t) {
  if (t->staging) return 0;
  const size_t pts = (size_t)t->M[0] * t->M[1] * t->M[2];
  const size_t cells = (size_t)t->Nc[0] * t->Nc[1] * t->Nc[2];
  const size_t ncw = (size_t)t->cap * t->ncomp;
  cudaError_t e1 = cudaMalloc(&t->staging, pts * ncw * t->in_bytes);
  cudaError_t e2 = cudaMalloc(&t->work_a, pts * ncw * sizeof(double));
  cudaError_t e3 = cudaMalloc(&t->work_w, cells * ncw * sizeof(double));
  cudaError_t e4 = cudaMalloc(&t->colmax, ncw * sizeof(double));
  cudaError_t e5 = cudaMalloc(&t->slot_spline_d, t->cap * sizeof(int));
  if (e1 || e2 || e3 || e4 || e5) {
    cudaGetLastError();
    free_work(t);
    return fail(EINSPLINE_GB300_ENOMEM, "cannot allocate the solve work space (%d splines per batch)", t->cap);
  }
  return 0;
}

// x-axis override for one flush (set_multi_UBspline_1d_{d,z}_BC).
struct AxisOverride {
  const double *fac;  // device line factors
  double lval[2], rval[2];
};

static int flush_locked(Table *t, const AxisOverride *ov = nullptr) {
  const int n = (int)t->pend_spline.size();
  if (n == 0) return 0;
  const int nc = t->ncomp;
  const int ncw = n * nc;
  const int64_t P = (int64_t)t->M[0] * t->M[1] * t->M[2];
  const int Mx = t->M[0], My = t->M[1], Mz = t->M[2];
  const int Nx = t->Nc[0], Ny = t->Nc[1], Nz = t->Nc[2];
  cudaStream_t s = t->stream;
  EG_CUDA(cudaMemcpyAsync(t->slot_spline_d, t->pend_spline.data(), n * sizeof(int), cudaMemcpyHostToDevice, s));
  // 1. transpose queued data to spline-fastest FP64
  dim3 tb(32, 8), tg((unsigned)((P + 31) / 32), (unsigned)((n + 31) / 32));
  if (t->in_bytes == 4) {
    if (nc == 1) k_stage_transpose<float, 1><<<tg, tb, 0, s>>>((const float *)t->staging, P, n, t->work_a);
    else k_stage_transpose<float, 2><<<tg, tb, 0, s>>>((const float *)t->staging, P, n, t->work_a);
  } else {
    if (nc == 1) k_stage_transpose<double, 1><<<tg, tb, 0, s>>>((const double *)t->staging, P, n, t->work_a);
    else k_stage_transpose<double, 2><<<tg, tb, 0, s>>>((const double *)t->staging, P, n, t->work_a);
  }
  count_launch();
  EG_CUDA(cudaGetLastError());
  // 2. sweeps: x (A -> W), then y and z in place on W
  const int64_t wz = ncw, wy = (int64_t)Nz * ncw, wx = (int64_t)Ny * Nz * ncw;
  const int64_t az = ncw, ay = (int64_t)Mz * ncw, ax = (int64_t)My * Mz * ncw;
  const int TB = 128;
  const int cblocks = (ncw + TB - 1) / TB;
  for (int axis = 0; axis < t->dims; axis++) {
    SweepArgs a;
    memset(&a, 0, sizeof(a));
    a.fac = t->factors_d + t->factor_off[axis];
    a.ncw = ncw;
    a.ncomp = nc;
    for (int p = 0; p < 2; p++) { a.lval[p] = t->lval[axis][p]; a.rval[p] = t->rval[axis][p]; }
    if (ov && axis == 0) {
      a.fac = ov->fac;
      for (int p = 0; p < 2; p++) { a.lval[p] = ov->lval[p]; a.rval[p] = ov->rval[p]; }
    }
    if (axis == 0) {
      a.in = t->work_a; a.out = t->work_w;
      a.nv = Mz; a.nlines = (int64_t)My * Mz;
      a.in_su = ay; a.in_sv = az; a.out_su = wy; a.out_sv = wz;
      a.in_stride = ax; a.out_stride = wx;
    } else if (axis == 1) {
      a.in = t->work_w; a.out = t->work_w;
      a.nv = Mz; a.nlines = (int64_t)Nx * Mz;
      a.in_su = wx; a.in_sv = wz; a.out_su = wx; a.out_sv = wz;
      a.in_stride = wy; a.out_stride = wy;
    } else {
      a.in = t->work_w; a.out = t->work_w;
      a.nv = Ny; a.nlines = (int64_t)Nx * Ny;
      a.in_su = wx; a.in_sv = wy; a.out_su = wx; a.out_sv = wy;
      a.in_stride = wz; a.out_stride = wz;
    }
    const int64_t blocks = a.nlines * cblocks;
    k_sweep<<<(unsigned)blocks, TB, 0, s>>>(a);
    count_launch();
    EG_CUDA(cudaGetLastError());
  }
  // 3. scales for 16-bit storage, 4. rounded store into the table columns
  const int64_t ncells = (int64_t)Nx * Ny * Nz;
  double *inv = reinterpret_cast<double *>(t->work_a);  // work_a is free again
  if (is16(t->storage)) {
    EG_CUDA(cudaMemsetAsync(t->colmax, 0, ncw * sizeof(unsigned int), s));
    dim3 cg((ncw + TB - 1) / TB, (unsigned)std::min<int64_t>(ncells, 1024));
    k_colmax<<<cg, TB, 0, s>>>(t->work_w, ncells, ncw, (unsigned int *)t->colmax);
    k_scales<<<(n + 127) / 128, 128, 0, s>>>(t->storage, (const unsigned int *)t->colmax, n, nc, t->slot_spline_d,
                                             t->scale, inv);
    count_launch(2);
    EG_CUDA(cudaGetLastError());
  }
  const int64_t sblocks = ncells * cblocks;
  switch (t->storage) {
    case ST_F64: k_store<ST_F64><<<(unsigned)sblocks, TB, 0, s>>>(t->work_w, ncells, ncw, nc, t->slot_spline_d, inv, t->coefs, t->zs); break;
    case ST_F32: k_store<ST_F32><<<(unsigned)sblocks, TB, 0, s>>>(t->work_w, ncells, ncw, nc, t->slot_spline_d, inv, t->coefs, t->zs); break;
    case ST_F16: k_store<ST_F16><<<(unsigned)sblocks, TB, 0, s>>>(t->work_w, ncells, ncw, nc, t->slot_spline_d, inv, t->coefs, t->zs); break;
    case ST_I16: k_store<ST_I16><<<(unsigned)sblocks, TB, 0, s>>>(t->work_w, ncells, ncw, nc, t->slot_spline_d, inv, t->coefs, t->zs); break;
    default: k_store<ST_BF16><<<(unsigned)sblocks, TB, 0, s>>>(t->work_w, ncells, ncw, nc, t->slot_spline_d, inv, t->coefs, t->zs); break;
  }
  count_launch();
  EG_CUDA(cudaGetLastError());
  t->pend_spline.clear();
  t->slot_of.clear();
  (void)Mx;
  return 0;
}

// Each FP64 coefficient as (hi, lo) = (round(c), round(c - hi)), stored per
// pair of adjacent columns as (hi0, hi1, lo0, lo1): one 16-byte load then
// gives the two high parts and the two low parts as the register pairs the
// packed f32x2 arithmetic takes, with no moves to regroup them (n is even:
// rows are padded to 128 bytes).
__global__ void k_to_df(const double *__restrict__ c, float4 *__restrict__ out, int64_t n) {
  const double2 *c2 = reinterpret_cast<const double2 *>(c);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n / 2; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 v = c2[i];
    const float h0 = __double2float_rn(v.x), h1 = __double2float_rn(v.y);
    out[i] = make_float4(h0, h1, __double2float_rn(__dsub_rn(v.x, (double)h0)),
                         __double2float_rn(__dsub_rn(v.y, (double)h1)));
  }
}

static int df_refresh_locked(Table *t) {
  if (t->fp64_mode != 1 || t->storage != ST_F64 || !t->df_stale) return 0;
  if (!t->df_coefs && cudaMalloc(&t->df_coefs, t->table_bytes) != cudaSuccess) {
    cudaGetLastError();
    t->df_coefs = nullptr;
    return fail(EINSPLINE_GB300_ENOMEM, "cannot allocate the double-float copy of the table (%zu bytes)",
                t->table_bytes);
  }
  const int64_t n = (int64_t)(t->table_bytes / sizeof(double));
  k_to_df<<<(unsigned)std::min<int64_t>((n / 2 + 255) / 256, 4096), 256, 0, t->stream>>>((const double *)t->coefs,
                                                                                          (float4 *)t->df_coefs, n);
  count_launch();
  EG_CUDA(cudaGetLastError());
  EG_CUDA(cudaStreamSynchronize(t->stream));
  t->df_stale = false;
  return 0;
}

int table_df_refresh(Table *t) {
  std::lock_guard<std::mutex> g(t->mu);
  return df_refresh_locked(t);
}

int table_flush(Table *t) {
  std::lock_guard<std::mutex> g(t->mu);
  const bool had = !t->pend_spline.empty();
  if (int r = flush_locked(t)) return r;
  // Evaluations may run on any stream: make the solved table visible to all.
  if (had) {
    EG_CUDA(cudaStreamSynchronize(t->stream));
    t->df_stale = true;
  }
  return df_refresh_locked(t);
}

int table_set_bc(Table *t, int spline, const void *data, int lcode, int rcode, const double lval[2],
                 const double rval[2]) {
  if (t->dims != 1) return fail(EINSPLINE_GB300_EINVAL, "a per-spline boundary condition needs a 1D table");
  if (spline < 0 || spline >= t->num_splines)
    return fail(EINSPLINE_GB300_EINVAL, "spline %d outside [0, %d)", spline, t->num_splines);
  if (!data) return fail(EINSPLINE_GB300_EINVAL, "data pointer is NULL");
  const bool cyc = (lcode == PERIODIC || lcode == ANTIPERIODIC);
  const bool tcyc = (t->lcode[0] == PERIODIC || t->lcode[0] == ANTIPERIODIC);
  if (lcode < PERIODIC || lcode > ANTIPERIODIC || cyc != tcyc ||
      (!cyc && (rcode < DERIV1 || rcode > NATURAL)))
    return fail(EINSPLINE_GB300_EINVAL,
                "boundary condition must be valid and periodic exactly when the table's is (the table has %d "
                "coefficients)", t->Nc[0]);
  std::lock_guard<std::mutex> g(t->mu);
  if (int r = ensure_work(t)) return r;
  if (int r = flush_locked(t)) return r;
  LineFactors f;
  build_line_factors(t->M[0], lcode, rcode, t->dinv[0], f);
  std::vector<double> pk;
  pack_line_factors(f, pk);
  double *fac = nullptr;
  if (cudaMalloc(&fac, pk.size() * sizeof(double)) != cudaSuccess) {
    cudaGetLastError();
    return fail(EINSPLINE_GB300_ENOMEM, "line factors");
  }
  AxisOverride ov;
  ov.fac = fac;
  for (int p = 0; p < 2; p++) {
    // FLAT and NATURAL force a zero boundary value (src/bspline_create.c:1137, :1156).
    ov.lval[p] = (lcode == FLAT || lcode == NATURAL) ? 0.0 : lval[p];
    ov.rval[p] = (rcode == FLAT || rcode == NATURAL) ? 0.0 : rval[p];
  }
  const size_t per = (size_t)t->M[0] * t->ncomp * t->in_bytes;
  t->pend_spline.push_back(spline);
  t->slot_of[spline] = 0;
  int r = 0;
  if (cudaMemcpyAsync(fac, pk.data(), pk.size() * sizeof(double), cudaMemcpyHostToDevice, t->stream) != cudaSuccess ||
      cudaMemcpyAsync(t->staging, data, per, cudaMemcpyHostToDevice, t->stream) != cudaSuccess) {
    r = cuda_check(cudaGetLastError(), "set with boundary condition");
    t->pend_spline.clear();
    t->slot_of.clear();
  } else {
    r = flush_locked(t, &ov);
  }
  cudaError_t e = cudaStreamSynchronize(t->stream);
  cudaFree(fac);
  if (!r && e != cudaSuccess) r = cuda_check(e, "set with boundary condition");
  return r;
}

int table_set(Table *t, int first, int count, const void *data, bool from_device) {
  if (first < 0 || count < 1 || first + count > t->num_splines)
    return fail(EINSPLINE_GB300_EINVAL, "spline range [%d, %d) outside [0, %d)", first, first + count, t->num_splines);
  if (!data) return fail(EINSPLINE_GB300_EINVAL, "data pointer is NULL");
  std::lock_guard<std::mutex> g(t->mu);
  if (int r = ensure_work(t)) return r;
  const size_t per = (size_t)t->M[0] * t->M[1] * t->M[2] * t->ncomp * t->in_bytes;
  for (int i = 0; i < count; i++) {
    const int sp = first + i;
    int slot;
    auto it = t->slot_of.find(sp);
    if (it != t->slot_of.end()) {
      slot = it->second;
    } else {
      if ((int)t->pend_spline.size() == t->cap)
        if (int r = flush_locked(t)) return r;
      slot = (int)t->pend_spline.size();
      t->pend_spline.push_back(sp);
      t->slot_of[sp] = slot;
    }
    const char *src = (const char *)data + (size_t)i * per;
    EG_CUDA(cudaMemcpyAsync((char *)t->staging + (size_t)slot * per, src, per,
                            from_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, t->stream));
  }
  return 0;
}

// ------------------------------------------------------------------
// Storage conversion for the *_cuda creators.
// ------------------------------------------------------------------
template <int SS, int DS>
__global__ void k_convert(const void *__restrict__ src, int64_t szs, void *__restrict__ dst, int64_t dzs,
                          int64_t ncells, int ncol, const double *__restrict__ inv) {
  const int cblocks = (ncol + blockDim.x - 1) / blockDim.x;
  const int64_t cell = blockIdx.x / cblocks;
  const int c = (int)(blockIdx.x % cblocks) * blockDim.x + threadIdx.x;
  if (cell >= ncells || c >= ncol) return;
  double w;
  if (SS == ST_F64) w = ((const double *)src)[cell * szs + c];
  else w = (double)((const float *)src)[cell * szs + c];
  store_coef<DS>(dst, cell * dzs + c, w, is16(DS) ? inv[c] : 1.0);
}

__global__ void k_colmax_table(const void *__restrict__ src, int src_f64, int64_t zs, int64_t ncells, int ncol,
                               unsigned int *colmax) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncol) return;
  float m = 0.f;
  for (int64_t e = blockIdx.y; e < ncells; e += gridDim.y) {
    double w = src_f64 ? ((const double *)src)[e * zs + c] : (double)((const float *)src)[e * zs + c];
    m = fmaxf(m, (float)fabs(w));
  }
  atomicMax(colmax + c, __float_as_uint(m));
}

Table *table_clone(Table *src, int storage) {
  if (int r = table_flush(src)) { (void)r; return nullptr; }
  GridDesc g[3];
  for (int a = 0; a < 3; a++) {
    g[a].start = src->start[a]; g[a].end = src->end[a]; g[a].num = src->M[a];
    g[a].lcode = src->lcode[a]; g[a].rcode = src->rcode[a];
    for (int p = 0; p < 2; p++) { g[a].lval[p] = src->lval[a][p]; g[a].rval[p] = src->rval[a][p]; }
  }
  char kind = src->kind;
  if (storage != ST_F64 && storage != ST_NATIVE && (kind == 'd' || kind == 'z')) kind = (kind == 'd') ? 's' : 'c';
  if (storage == ST_NATIVE) storage = src->storage;
  Table *t = table_create(kind, g, src->num_splines, storage, src->dims);
  if (!t) return nullptr;
  // Make the copy on the source's stream order, then on the new stream.
  if (cudaStreamSynchronize(src->stream) != cudaSuccess) { cuda_check(cudaGetLastError(), "clone sync"); table_destroy(t); return nullptr; }
  const int64_t ncells = (int64_t)t->Nc[0] * t->Nc[1] * t->Nc[2];
  if (src->storage == t->storage) {
    if (cudaMemcpyAsync(t->coefs, src->coefs, t->table_bytes, cudaMemcpyDeviceToDevice, t->stream) != cudaSuccess ||
        (t->scale && cudaMemcpyAsync(t->scale, src->scale, sizeof(float) * t->ncol_pad, cudaMemcpyDeviceToDevice, t->stream) != cudaSuccess)) {
      cuda_check(cudaGetLastError(), "table copy");
      table_destroy(t);
      return nullptr;
    }
  } else {
    if (src->storage != ST_F64 && src->storage != ST_F32) {
      fail(EINSPLINE_GB300_EINVAL, "cannot convert from 16-bit storage");
      table_destroy(t);
      return nullptr;
    }
    double *inv = nullptr;
    unsigned int *cm = nullptr;
    if (cudaMalloc(&inv, sizeof(double) * t->ncol_pad) != cudaSuccess ||
        cudaMalloc(&cm, sizeof(unsigned int) * t->ncol_pad) != cudaSuccess) {
      cudaGetLastError();
      cudaFree(inv);
      fail(EINSPLINE_GB300_ENOMEM, "conversion scratch");
      table_destroy(t);
      return nullptr;
    }
    const int TB = 128, ncol = t->ncol;
    if (is16(t->storage)) {
      cudaMemsetAsync(cm, 0, sizeof(unsigned int) * t->ncol_pad, t->stream);
      dim3 cg((ncol + TB - 1) / TB, (unsigned)std::min<int64_t>(ncells, 1024));
      k_colmax_table<<<cg, TB, 0, t->stream>>>(src->coefs, src->storage == ST_F64, src->zs, ncells, ncol, cm);
      k_scales<<<(t->num_splines + 127) / 128, 128, 0, t->stream>>>(t->storage, cm, t->num_splines, t->ncomp,
                                                                    nullptr, t->scale, inv);
      count_launch(2);
    }
    const int64_t blocks = ncells * ((ncol + TB - 1) / TB);
    const bool s64 = src->storage == ST_F64;
#define EG_CONV(SS, DS) k_convert<SS, DS><<<(unsigned)blocks, TB, 0, t->stream>>>(src->coefs, src->zs, t->coefs, t->zs, ncells, ncol, inv)
    if (s64) {
      if (t->storage == ST_F32) EG_CONV(ST_F64, ST_F32);
      else if (t->storage == ST_F16) EG_CONV(ST_F64, ST_F16);
      else if (t->storage == ST_I16) EG_CONV(ST_F64, ST_I16);
      else EG_CONV(ST_F64, ST_BF16);
    } else {
      if (t->storage == ST_F16) EG_CONV(ST_F32, ST_F16);
      else if (t->storage == ST_BF16) EG_CONV(ST_F32, ST_BF16);
      else if (t->storage == ST_I16) EG_CONV(ST_F32, ST_I16);
      else EG_CONV(ST_F32, ST_F64);
    }
#undef EG_CONV
    count_launch();
    cudaError_t e = cudaStreamSynchronize(t->stream);
    cudaFree(inv);
    cudaFree(cm);
    if (e != cudaSuccess) { cuda_check(e, "table conversion"); table_destroy(t); return nullptr; }
  }
  return t;
}

}  // namespace eg

// Host check of the factored line solve against a caller-supplied oracle:
// coefs (N = M+3 or M+2 values) from data (M values), unit strides.
extern "C" int einspline_gb300_solve_line_host(int M, int lcode, int rcode, double delta_inv, double lval,
                                               double rval, const double *data, double *coefs) {
  eg::LineFactors f;
  eg::build_line_factors(M, lcode, rcode, delta_inv, f);
  std::vector<double> pk;
  eg::pack_line_factors(f, pk);
  eg::solve_line(pk.data(), data, 1, coefs, 1, lval, rval);
  return 0;
}
