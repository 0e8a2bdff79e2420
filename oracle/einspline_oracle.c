/*
 * einspline_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A CPU restatement of einspline's uniform 3D multi-spline path: the
 * interpolating coefficient solve behind set_multi_UBspline_3d_{d,z} and the
 * value / value+gradient+Hessian evaluation of eval_multi_UBspline_3d_{s,d,c,z}
 * and of the batched GPU entries eval_multi_multi_UBspline_3d_*_cuda.
 *
 * Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py
 * load this file's library, and only as the checker (or as the timed CPU
 * baseline).  The GPU library never links or calls it.
 *
 * Pinning: tests/test_oracle.py compares this code bit for bit against the
 * reference's own CPU sources (compiled by `make -C oracle ref` when the
 * reference tree is present) and against the committed golden vectors in
 * tests/golden/, which were produced by that compiled reference.
 *
 * Arithmetic order follows the reference on purpose (same sums, same order,
 * built with -ffp-contract=off) so that results are bit-identical to the
 * reference built with the same flags.  Reference citations are
 * src/<file>:<line> within the einspline project.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* Boundary-condition codes, in the order of bc_code (src/bspline_base.h:49). */
enum { ORC_PERIODIC = 0, ORC_DERIV1, ORC_DERIV2, ORC_FLAT, ORC_NATURAL, ORC_ANTIPERIODIC };

typedef struct {
  double start, end, delta, delta_inv;
  int num;       /* M: number of data points along the axis                 */
  int ncoef;     /* N: M+3 for periodic/antiperiodic, M+2 otherwise         */
  int lcode, rcode;
  double lval[2], rval[2]; /* BC values: [0] real part, [1] imaginary part */
} orc_axis;

typedef struct {
  orc_axis ax[3];
  int num_splines;          /* splines (complex splines for c/z)            */
  int64_t xs, ys, zs;       /* table strides in table elements              */
} orc_desc;

/* Cubic B-spline power-basis matrices: row i gives the weight of control
 * point i as a cubic in t, coefficients of [t^3, t^2, t, 1]
 * (src/bspline_data.c:143-162 float, :174-193 double).  Row 0 is (1-t)^3/6,
 * row 3 is t^3/6; dA and d2A are the first and second t-derivatives. */
static const double kA[3][16] = {
  { -1.0/6.0,  3.0/6.0, -3.0/6.0, 1.0/6.0,
     3.0/6.0, -6.0/6.0,  0.0/6.0, 4.0/6.0,
    -3.0/6.0,  3.0/6.0,  3.0/6.0, 1.0/6.0,
     1.0/6.0,  0.0/6.0,  0.0/6.0, 0.0/6.0 },
  {  0.0, -0.5,  1.0, -0.5,
     0.0,  1.5, -2.0,  0.0,
     0.0, -1.5,  1.0,  0.5,
     0.0,  0.5,  0.0,  0.0 },
  {  0.0, 0.0, -1.0,  1.0,
     0.0, 0.0,  3.0, -2.0,
     0.0, 0.0, -3.0,  1.0,
     0.0, 0.0,  1.0,  0.0 } };

/* ------------------------------------------------------------------ */
/* Grid set-up (src/multi_bspline_create.c:269-294, same for d/c/z).   */
/* ------------------------------------------------------------------ */
int orc_axis_init(orc_axis *a, double start, double end, int num, int lcode, int rcode,
                  double lval_r, double lval_i, double rval_r, double rval_i)
{
  memset(a, 0, sizeof(*a));
  a->start = start; a->end = end; a->num = num;
  a->lcode = lcode; a->rcode = rcode;
  a->lval[0] = lval_r; a->lval[1] = lval_i;
  a->rval[0] = rval_r; a->rval[1] = rval_i;
  a->ncoef = (lcode == ORC_PERIODIC || lcode == ORC_ANTIPERIODIC) ? num + 3 : num + 2;
  a->delta = (end - start) / (double)(a->ncoef - 3);
  a->delta_inv = 1.0 / a->delta;
  return a->ncoef;
}

/* ------------------------------------------------------------------ */
/* 1D interpolation solves in double precision.                        */
/* ------------------------------------------------------------------ */

/* Cyclic tridiagonal solve for (anti)periodic data: eliminate down the
 * band while carrying the wrap-around column, then back-substitute and
 * fill the three wrap coefficients (src/bspline_create.c:1010-1055
 * periodic, :1064-1111 antiperiodic).  b holds M rows of 4: sub, diag,
 * super, rhs. */
static void solve_cyclic_d(double *b, double *c, int M, int64_t cs, int anti)
{
  double *lastCol = (double *)malloc(sizeof(double) * (size_t)M);
  if (anti) { b[0] *= -1.0; b[4*(M-1)+2] *= -1.0; }
  b[2] /= b[1];
  b[0] /= b[1];
  b[3] /= b[1];
  b[1] = 1.0;
  b[4*(M-1)+1] -= b[4*(M-1)+2] * b[0];
  b[4*(M-1)+3] -= b[4*(M-1)+2] * b[3];
  b[4*(M-1)+2] = -b[4*(M-1)+2] * b[2];
  lastCol[0] = b[0];
  for (int r = 1; r < M-1; r++) {
    double *row = b + 4*r, *up = b + 4*(r-1), *last = b + 4*(M-1);
    row[1] -= row[0] * up[2];
    row[3] -= row[0] * up[3];
    lastCol[r] = -row[0] * lastCol[r-1];
    row[0] = 0.0;
    row[2] /= row[1];
    row[3] /= row[1];
    lastCol[r] /= row[1];
    row[1] = 1.0;
    if (r < M-2) {
      last[3] -= last[2] * row[3];
      last[1] -= last[2] * lastCol[r];
      last[2] = -last[2] * row[2];
    }
  }
  b[4*(M-1)+0] += b[4*(M-1)+2];
  b[4*(M-1)+1] -= b[4*(M-1)+0] * (b[4*(M-2)+2] + lastCol[M-2]);
  b[4*(M-1)+3] -= b[4*(M-1)+0] * b[4*(M-2)+3];
  b[4*(M-1)+3] /= b[4*(M-1)+1];
  c[M*cs] = b[4*(M-1)+3];
  for (int r = M-2; r >= 0; r--)
    c[(r+1)*cs] = b[4*r+3] - b[4*r+2]*c[(r+2)*cs] - lastCol[r]*c[M*cs];
  double s = anti ? -1.0 : 1.0;
  c[0] = s * c[M*cs];
  c[(M+1)*cs] = s * c[1*cs];
  c[(M+2)*cs] = s * c[2*cs];
  free(lastCol);
}

/* Tridiagonal solve with one boundary-condition row at each end
 * (src/bspline_create.c:959-1001).  b holds M+2 rows of 4. */
static void solve_bc_d(double *b, double *c, int M, int64_t cs)
{
  b[1] /= b[0];
  b[2] /= b[0];
  b[3] /= b[0];
  b[0] = 1.0;
  b[4+1] -= b[4+0]*b[1];
  b[4+2] -= b[4+0]*b[2];
  b[4+3] -= b[4+0]*b[3];
  b[0] = 0.0;
  b[4+2] /= b[4+1];
  b[4+3] /= b[4+1];
  b[4+1] = 1.0;
  for (int r = 2; r < M+1; r++) {
    double *row = b + 4*r, *up = b + 4*(r-1);
    row[1] -= row[0]*up[2];
    row[3] -= row[0]*up[3];
    row[2] /= row[1];
    row[3] /= row[1];
    row[0] = 0.0;
    row[1] = 1.0;
  }
  double *last = b + 4*(M+1);
  last[1] -= last[0]*b[4*(M-1)+2];
  last[3] -= last[0]*b[4*(M-1)+3];
  last[2] -= last[1]*b[4*M+2];
  last[3] -= last[1]*b[4*M+3];
  last[3] /= last[2];
  last[2] = 1.0;
  c[(M+1)*cs] = last[3];
  for (int r = M; r > 0; r--)
    c[r*cs] = b[4*r+3] - b[4*r+2]*c[cs*(r+1)];
  c[0] = b[3] - b[1]*c[1*cs] - b[2]*c[2*cs];
}

/* Boundary row for one end: first-derivative (DERIV1/FLAT) or
 * second-derivative (DERIV2/NATURAL) condition (src/bspline_create.c:1138-1174). */
static void bc_row(int code, double val, double dinv, double row[4])
{
  if (code == ORC_FLAT || code == ORC_NATURAL) val = 0.0;
  if (code == ORC_FLAT || code == ORC_DERIV1) {
    row[0] = -0.5 * dinv; row[1] = 0.0 * dinv; row[2] = 0.5 * dinv; row[3] = val;
  } else {
    row[0] = 1.0 * dinv * dinv; row[1] = -2.0 * dinv * dinv; row[2] = 1.0 * dinv * dinv; row[3] = val;
  }
}

/* One line: data[i*dstride] for i<M in, coefs[i*cstride] for i<N out
 * (src/bspline_create.c:1116-1198).  part selects the real (0) or
 * imaginary (1) boundary values. */
void orc_find_coefs_1d_d(const orc_axis *a, int part, const double *data, int64_t dstride,
                         double *coefs, int64_t cstride)
{
  const int M = a->num;
  const double basis[3] = {1.0/6.0, 2.0/3.0, 1.0/6.0};
  if (a->lcode == ORC_PERIODIC || a->lcode == ORC_ANTIPERIODIC) {
    double *b = (double *)malloc(sizeof(double) * 4 * (size_t)M);
    for (int i = 0; i < M; i++) {
      b[4*i+0] = basis[0]; b[4*i+1] = basis[1]; b[4*i+2] = basis[2];
      b[4*i+3] = data[i*dstride];
    }
    solve_cyclic_d(b, coefs, M, cstride, a->lcode == ORC_ANTIPERIODIC);
    free(b);
  } else {
    double *b = (double *)malloc(sizeof(double) * 4 * (size_t)(M+2));
    bc_row(a->lcode, a->lval[part], a->delta_inv, b);
    bc_row(a->rcode, a->rval[part], a->delta_inv, b + 4*(M+1));
    for (int i = 0; i < M; i++) {
      b[4*(i+1)+0] = basis[0]; b[4*(i+1)+1] = basis[1]; b[4*(i+1)+2] = basis[2];
      b[4*(i+1)+3] = data[i*dstride];
    }
    solve_bc_d(b, coefs, M, cstride);
    free(b);
  }
}

/* Coefficients of one spline column from data[Mx][My][Mz] (ncomp=1) or
 * interleaved complex data (ncomp=2): sweeps along x, then y, then z
 * (src/multi_bspline_create.c:1020-1073 for d, :1392-1478 for z).  The
 * table is double (or double pairs) with strides d->xs,ys,zs in table
 * elements. */
void orc_set_3d_column_d(const orc_desc *d, int ncomp, int spline, double *table, const double *data)
{
  const orc_axis *X = &d->ax[0], *Y = &d->ax[1], *Z = &d->ax[2];
  const int My = Y->num, Mz = Z->num;
  const int Nx = X->ncoef, Ny = Y->ncoef, Nz = Z->ncoef;
  const int64_t xs = ncomp * d->xs, ys = ncomp * d->ys, zs = ncomp * d->zs;
  for (int p = 0; p < ncomp; p++) {
    double *col = table + (int64_t)ncomp * spline + p;
    const double *dat = data + p;
    for (int iy = 0; iy < My; iy++)
      for (int iz = 0; iz < Mz; iz++)
        orc_find_coefs_1d_d(X, p, dat + (int64_t)ncomp * (iy*Mz + iz), (int64_t)ncomp * My * Mz,
                            col + iy*ys + iz*zs, xs);
    for (int ix = 0; ix < Nx; ix++)
      for (int iz = 0; iz < Mz; iz++)
        orc_find_coefs_1d_d(Y, p, col + ix*xs + iz*zs, ys, col + ix*xs + iz*zs, ys);
    for (int ix = 0; ix < Nx; ix++)
      for (int iy = 0; iy < Ny; iy++)
        orc_find_coefs_1d_d(Z, p, col + ix*xs + iy*ys, zs, col + ix*xs + iy*ys, zs);
  }
  (void)Nz;
}

/* The same for 1D and 2D multi-splines (dims = 1 or 2: axes beyond dims
 * have num = ncoef = 1): sweeps along x, then y
 * (src/multi_bspline_create.c:822-828 and :903-940 for d, :1138-1145 and
 * :1257-1300 for z). */
void orc_set_column_d(const orc_desc *d, int dims, int ncomp, int spline, double *table, const double *data)
{
  if (dims == 3) { orc_set_3d_column_d(d, ncomp, spline, table, data); return; }
  const orc_axis *X = &d->ax[0], *Y = &d->ax[1];
  const int My = dims == 2 ? Y->num : 1;
  const int Nx = X->ncoef;
  const int64_t xs = ncomp * d->xs, ys = ncomp * d->ys;
  for (int p = 0; p < ncomp; p++) {
    double *col = table + (int64_t)ncomp * spline + p;
    const double *dat = data + p;
    for (int iy = 0; iy < My; iy++)
      orc_find_coefs_1d_d(X, p, dat + (int64_t)ncomp * iy, (int64_t)ncomp * My, col + iy*ys, xs);
    if (dims == 2)
      for (int ix = 0; ix < Nx; ix++)
        orc_find_coefs_1d_d(Y, p, col + ix*xs, ys, col + ix*xs, ys);
  }
}

/* ------------------------------------------------------------------ */
/* Evaluation.                                                         */
/* ------------------------------------------------------------------ */

/* Cell and fractional offset.
 * sem 0 (CPU entries, src/multi_bspline_eval_std_s_impl.h:746-755):
 *   u = (x - start) * delta_inv (rounded to float for s/c), t = modf(u),
 *   i = (int) integer part.  The reference reads outside the table when i
 *   leaves [0, N-4]; here i is clamped and t extended so the cell polynomial
 *   is extrapolated (the GPU library does the same).
 * sem 1 (GPU entries, src/multi_bspline_cuda_s_impl.h:370-384):
 *   u = r * delta_inv with no start offset (float for s/c), i = clamp(floor(u),
 *   0, dim-1) with dim = N-3, t = u - floor(u) (t is not adjusted). */
static void cell_f(const orc_axis *a, int sem, double x, int *i, float *t)
{
  int lim = a->ncoef - 4;
  if (sem == 0) {
    x -= a->start;
    float u = (float)(x * a->delta_inv);
    float ip;
    float tt = modff(u, &ip);
    int ii = (int)ip;
    if (ii < 0) { tt += (float)ii; ii = 0; }
    if (ii > lim) { tt += (float)(ii - lim); ii = lim; }
    *i = ii; *t = tt;
  } else {
    float r = (float)x, dinv = (float)a->delta_inv;
    float s = r * dinv;
    float sf = floorf(s);
    int ii = (int)sf;
    ii = ii < 0 ? 0 : (ii > lim ? lim : ii);
    *i = ii; *t = s - sf;
  }
}

static void cell_d(const orc_axis *a, int sem, double x, int *i, double *t)
{
  int lim = a->ncoef - 4;
  if (sem == 0) {
    x -= a->start;
    double u = x * a->delta_inv;
    double ip;
    double tt = modf(u, &ip);
    int ii = (int)ip;
    if (ii < 0) { tt += (double)ii; ii = 0; }
    if (ii > lim) { tt += (double)(ii - lim); ii = lim; }
    *i = ii; *t = tt;
  } else {
    double s = x * a->delta_inv;
    double sf = floor(s);
    int ii = (int)sf;
    ii = ii < 0 ? 0 : (ii > lim ? lim : ii);
    *i = ii; *t = s - sf;
  }
}

/* Basis weights w[d][i] (d = 0 value, 1 first, 2 second derivative) in the
 * reference's order: ((A0 t^3 + A1 t^2) + A2 t) + A3. */
static void basis_f(float t, float w[3][4])
{
  float tp[4] = {t*t*t, t*t, t, 1.0f};
  for (int d = 0; d < 3; d++)
    for (int i = 0; i < 4; i++) {
      float s = (float)kA[d][4*i+0] * tp[0];
      s = s + (float)kA[d][4*i+1] * tp[1];
      s = s + (float)kA[d][4*i+2] * tp[2];
      s = s + (float)kA[d][4*i+3] * tp[3];
      w[d][i] = s;
    }
}

static void basis_d(double t, double w[3][4])
{
  double tp[4] = {t*t*t, t*t, t, 1.0};
  for (int d = 0; d < 3; d++)
    for (int i = 0; i < 4; i++) {
      double s = kA[d][4*i+0] * tp[0];
      s = s + kA[d][4*i+1] * tp[1];
      s = s + kA[d][4*i+2] * tp[2];
      s = s + kA[d][4*i+3] * tp[3];
      w[d][i] = s;
    }
}

/* Generic evaluation body: REAL is the arithmetic type, NC the number of
 * real components per spline (1 real, 2 complex).  Accumulation order is
 * i, j, k outer and spline inner, with the ten weights formed as
 * (w_i * w_j) * w_k (src/multi_bspline_eval_std_s_impl.h:814-841).
 * Output layout is the CPU API's: vals[N], grads[N][3], hess[N][3][3],
 * each entry NC reals wide. */
#define ORC_EVAL_BODY(REAL, CELL, BASIS)                                          \
  const int N = d->num_splines;                                                   \
  int ix, iy, iz; REAL tx, ty, tz;                                                \
  CELL(&d->ax[0], sem, x, &ix, &tx);                                              \
  CELL(&d->ax[1], sem, y, &iy, &ty);                                              \
  CELL(&d->ax[2], sem, z, &iz, &tz);                                              \
  REAL wa[3][4], wb[3][4], wc[3][4];                                              \
  BASIS(tx, wa); BASIS(ty, wb); BASIS(tz, wc);                                    \
  const int64_t xs = NC * d->xs, ys = NC * d->ys, zs = NC * d->zs;                \
  for (int n = 0; n < NC * N; n++) vals[n] = 0;                                   \
  if (vgh) for (int n = 0; n < 3 * NC * N; n++) grads[n] = 0;                     \
  if (vgh) for (int n = 0; n < 9 * NC * N; n++) hess[n] = 0;                      \
  for (int i = 0; i < 4; i++)                                                     \
    for (int j = 0; j < 4; j++)                                                   \
      for (int k = 0; k < 4; k++) {                                               \
        const REAL *cf = coefs + (ix+i)*xs + (iy+j)*ys + (iz+k)*zs;               \
        REAL abc = wa[0][i]*wb[0][j]*wc[0][k];                                    \
        if (!vgh) {                                                               \
          for (int n = 0; n < NC * N; n++) vals[n] += abc * cf[n];                \
          continue;                                                               \
        }                                                                         \
        REAL g[3], h[6];                                                          \
        g[0] = wa[1][i]*wb[0][j]*wc[0][k];                                        \
        g[1] = wa[0][i]*wb[1][j]*wc[0][k];                                        \
        g[2] = wa[0][i]*wb[0][j]*wc[1][k];                                        \
        h[0] = wa[2][i]*wb[0][j]*wc[0][k];                                        \
        h[1] = wa[1][i]*wb[1][j]*wc[0][k];                                        \
        h[2] = wa[1][i]*wb[0][j]*wc[1][k];                                        \
        h[3] = wa[0][i]*wb[2][j]*wc[0][k];                                        \
        h[4] = wa[0][i]*wb[1][j]*wc[1][k];                                        \
        h[5] = wa[0][i]*wb[0][j]*wc[2][k];                                        \
        for (int n = 0; n < N; n++)                                               \
          for (int p = 0; p < NC; p++) {                                          \
            REAL cv = cf[NC*n + p];                                               \
            vals[NC*n + p] += abc * cv;                                           \
            grads[NC*(3*n+0) + p] += g[0] * cv;                                   \
            grads[NC*(3*n+1) + p] += g[1] * cv;                                   \
            grads[NC*(3*n+2) + p] += g[2] * cv;                                   \
            hess[NC*(9*n+0) + p] += h[0] * cv;                                    \
            hess[NC*(9*n+1) + p] += h[1] * cv;                                    \
            hess[NC*(9*n+2) + p] += h[2] * cv;                                    \
            hess[NC*(9*n+4) + p] += h[3] * cv;                                    \
            hess[NC*(9*n+5) + p] += h[4] * cv;                                    \
            hess[NC*(9*n+8) + p] += h[5] * cv;                                    \
          }                                                                       \
      }                                                                           \
  if (!vgh) return;                                                               \
  REAL dxi = (REAL)d->ax[0].delta_inv, dyi = (REAL)d->ax[1].delta_inv;            \
  REAL dzi = (REAL)d->ax[2].delta_inv;                                            \
  for (int n = 0; n < N; n++)                                                     \
    for (int p = 0; p < NC; p++) {                                                \
      grads[NC*(3*n+0)+p] *= dxi;                                                 \
      grads[NC*(3*n+1)+p] *= dyi;                                                 \
      grads[NC*(3*n+2)+p] *= dzi;                                                 \
      hess[NC*(9*n+0)+p] *= dxi*dxi;                                              \
      hess[NC*(9*n+4)+p] *= dyi*dyi;                                              \
      hess[NC*(9*n+8)+p] *= dzi*dzi;                                              \
      hess[NC*(9*n+1)+p] *= dxi*dyi;                                              \
      hess[NC*(9*n+2)+p] *= dxi*dzi;                                              \
      hess[NC*(9*n+5)+p] *= dyi*dzi;                                              \
      hess[NC*(9*n+3)+p] = hess[NC*(9*n+1)+p];                                    \
      hess[NC*(9*n+6)+p] = hess[NC*(9*n+2)+p];                                    \
      hess[NC*(9*n+7)+p] = hess[NC*(9*n+5)+p];                                    \
    }

/* s: src/multi_bspline_eval_std_s_impl.h:480-533 (value), :740-863 (vgh). */
void orc_eval_s(const orc_desc *d, int sem, int vgh, const float *coefs, double x, double y, double z,
                float *vals, float *grads, float *hess)
{
  enum { NC = 1 };
  ORC_EVAL_BODY(float, cell_f, basis_f)
}

/* d: src/multi_bspline_eval_std_d_impl.h:482 (value), :742 (vgh). */
void orc_eval_d(const orc_desc *d, int sem, int vgh, const double *coefs, double x, double y, double z,
                double *vals, double *grads, double *hess)
{
  enum { NC = 1 };
  ORC_EVAL_BODY(double, cell_d, basis_d)
}

/* c: src/multi_bspline_eval_std_c_impl.h:477 (value), :738 (vgh); complex
 * entries are (re, im) float pairs and both parts see the same weights. */
void orc_eval_c(const orc_desc *d, int sem, int vgh, const float *coefs, double x, double y, double z,
                float *vals, float *grads, float *hess)
{
  enum { NC = 2 };
  ORC_EVAL_BODY(float, cell_f, basis_f)
}

/* z: src/multi_bspline_eval_std_z_impl.h:481 (value), :742 (vgh). */
void orc_eval_z(const orc_desc *d, int sem, int vgh, const double *coefs, double x, double y, double z,
                double *vals, double *grads, double *hess)
{
  enum { NC = 2 };
  ORC_EVAL_BODY(double, cell_d, basis_d)
}

/* Value, gradient, Hessian and third derivatives ("vghgh"): the reference's
 * eval_multi_UBspline_3d_{s,d,c,z}_vghgh (src/multi_bspline_eval_std_s_impl.h:866-1038,
 * _d_impl.h:868, _c_impl.h:864, _z_impl.h), declared in its backend headers
 * (src/multi_bspline_eval_std_s.h etc.).  gradhess is [N][3][3][3]; the ten
 * distinct entries are accumulated and copied to their symmetric places. */
#define ORC_VGHGH_BODY(REAL, CELL, BASIS)                                         \
  const int N = d->num_splines;                                                   \
  int ix, iy, iz; REAL tx, ty, tz;                                                \
  CELL(&d->ax[0], 0, x, &ix, &tx);                                                \
  CELL(&d->ax[1], 0, y, &iy, &ty);                                                \
  CELL(&d->ax[2], 0, z, &iz, &tz);                                                \
  REAL wa[3][4], wb[3][4], wc[3][4];                                              \
  BASIS(tx, wa); BASIS(ty, wb); BASIS(tz, wc);                                    \
  const REAL d3w[4] = {(REAL)-1.0, (REAL)3.0, (REAL)-3.0, (REAL)1.0};             \
  const int64_t xs = NC * d->xs, ys = NC * d->ys, zs = NC * d->zs;                \
  for (int n = 0; n < NC * N; n++) vals[n] = 0;                                   \
  for (int n = 0; n < 3 * NC * N; n++) grads[n] = 0;                              \
  for (int n = 0; n < 9 * NC * N; n++) hess[n] = 0;                               \
  for (int n = 0; n < 27 * NC * N; n++) gh[n] = 0;                                \
  static const int gpos[10] = {0, 1, 2, 4, 5, 8, 13, 14, 17, 26};                 \
  for (int i = 0; i < 4; i++)                                                     \
    for (int j = 0; j < 4; j++)                                                   \
      for (int k = 0; k < 4; k++) {                                               \
        const REAL *cf = coefs + (ix+i)*xs + (iy+j)*ys + (iz+k)*zs;               \
        REAL w[20];                                                               \
        w[0] = wa[0][i]*wb[0][j]*wc[0][k];                                        \
        w[1] = wa[1][i]*wb[0][j]*wc[0][k];                                        \
        w[2] = wa[0][i]*wb[1][j]*wc[0][k];                                        \
        w[3] = wa[0][i]*wb[0][j]*wc[1][k];                                        \
        w[4] = wa[2][i]*wb[0][j]*wc[0][k];                                        \
        w[5] = wa[1][i]*wb[1][j]*wc[0][k];                                        \
        w[6] = wa[1][i]*wb[0][j]*wc[1][k];                                        \
        w[7] = wa[0][i]*wb[2][j]*wc[0][k];                                        \
        w[8] = wa[0][i]*wb[1][j]*wc[1][k];                                        \
        w[9] = wa[0][i]*wb[0][j]*wc[2][k];                                        \
        w[10] = d3w[i]*wb[0][j]*wc[0][k];                                         \
        w[11] = wa[2][i]*wb[1][j]*wc[0][k];                                       \
        w[12] = wa[2][i]*wb[0][j]*wc[1][k];                                       \
        w[13] = wa[1][i]*wb[2][j]*wc[0][k];                                       \
        w[14] = wa[1][i]*wb[1][j]*wc[1][k];                                       \
        w[15] = wa[1][i]*wb[0][j]*wc[2][k];                                       \
        w[16] = wa[0][i]*d3w[j]*wc[0][k];                                         \
        w[17] = wa[0][i]*wb[2][j]*wc[1][k];                                       \
        w[18] = wa[0][i]*wb[1][j]*wc[2][k];                                       \
        w[19] = wa[0][i]*wb[0][j]*d3w[k];                                         \
        for (int n = 0; n < N; n++)                                               \
          for (int p = 0; p < NC; p++) {                                          \
            REAL cv = cf[NC*n + p];                                               \
            vals[NC*n + p] += w[0] * cv;                                          \
            for (int c = 0; c < 3; c++) grads[NC*(3*n+c) + p] += w[1+c] * cv;     \
            hess[NC*(9*n+0) + p] += w[4] * cv;                                    \
            hess[NC*(9*n+1) + p] += w[5] * cv;                                    \
            hess[NC*(9*n+2) + p] += w[6] * cv;                                    \
            hess[NC*(9*n+4) + p] += w[7] * cv;                                    \
            hess[NC*(9*n+5) + p] += w[8] * cv;                                    \
            hess[NC*(9*n+8) + p] += w[9] * cv;                                    \
            for (int m = 0; m < 10; m++) gh[NC*(27*n+gpos[m]) + p] += w[10+m] * cv; \
          }                                                                       \
      }                                                                           \
  REAL dx = (REAL)d->ax[0].delta_inv, dy = (REAL)d->ax[1].delta_inv;              \
  REAL dz = (REAL)d->ax[2].delta_inv;                                             \
  const REAL f3[10] = {dx*dx*dx, dx*dx*dy, dx*dx*dz, dx*dy*dy, dx*dy*dz,          \
                       dx*dz*dz, dy*dy*dy, dy*dy*dz, dy*dz*dz, dz*dz*dz};         \
  /* symmetric copies: for each distinct entry, the other index orders */        \
  static const int copies[10][6] = {{-1}, {3, 9, -1}, {6, 18, -1}, {10, 12, -1},  \
      {7, 11, 15, 19, 21, -1}, {20, 24, -1}, {-1}, {16, 22, -1}, {23, 25, -1}, {-1}}; \
  for (int n = 0; n < N; n++)                                                     \
    for (int p = 0; p < NC; p++) {                                                \
      grads[NC*(3*n+0)+p] *= dx;                                                  \
      grads[NC*(3*n+1)+p] *= dy;                                                  \
      grads[NC*(3*n+2)+p] *= dz;                                                  \
      hess[NC*(9*n+0)+p] *= dx*dx;                                                \
      hess[NC*(9*n+4)+p] *= dy*dy;                                                \
      hess[NC*(9*n+8)+p] *= dz*dz;                                                \
      hess[NC*(9*n+1)+p] *= dx*dy;                                                \
      hess[NC*(9*n+2)+p] *= dx*dz;                                                \
      hess[NC*(9*n+5)+p] *= dy*dz;                                                \
      hess[NC*(9*n+3)+p] = hess[NC*(9*n+1)+p];                                    \
      hess[NC*(9*n+6)+p] = hess[NC*(9*n+2)+p];                                    \
      hess[NC*(9*n+7)+p] = hess[NC*(9*n+5)+p];                                    \
      for (int m = 0; m < 10; m++) {                                              \
        REAL *g0 = &gh[NC*(27*n+gpos[m])+p];                                      \
        *g0 *= f3[m];                                                             \
        for (int c = 0; c < 6 && copies[m][c] >= 0; c++) gh[NC*(27*n+copies[m][c])+p] = *g0; \
      }                                                                           \
    }

void orc_eval_s_vghgh(const orc_desc *d, const float *coefs, double x, double y, double z,
                      float *vals, float *grads, float *hess, float *gh)
{
  enum { NC = 1 };
  ORC_VGHGH_BODY(float, cell_f, basis_f)
}
void orc_eval_d_vghgh(const orc_desc *d, const double *coefs, double x, double y, double z,
                      double *vals, double *grads, double *hess, double *gh)
{
  enum { NC = 1 };
  ORC_VGHGH_BODY(double, cell_d, basis_d)
}
void orc_eval_c_vghgh(const orc_desc *d, const float *coefs, double x, double y, double z,
                      float *vals, float *grads, float *hess, float *gh)
{
  enum { NC = 2 };
  ORC_VGHGH_BODY(float, cell_f, basis_f)
}
void orc_eval_z_vghgh(const orc_desc *d, const double *coefs, double x, double y, double z,
                      double *vals, double *grads, double *hess, double *gh)
{
  enum { NC = 2 };
  ORC_VGHGH_BODY(double, cell_d, basis_d)
}

/* 1D and 2D multi-splines at one point, CPU-entry cell rule, the CPU API's
 * layouts (src/multi_bspline_eval_std_s_impl.h:38-181 for 1D, :183-480 for
 * 2D; _d, _c, _z impl files alike).  form: 0 value, 1 vg, 2 vgl, 3 vgh.
 *   1D: vals[N], grads[N], lh[N] = second derivative (vgl and vgh alike: the
 *       reference's 1D vgh calls vgl);
 *   2D: vals[N], grads[N][2], lapl[N] (vgl: (xx + yy)), hess[N][2][2] (vgh).
 * Products and sums in the reference's order: ab = a_i * b_j formed once
 * per (i, j), accumulated over i then j, scaled by delta_inv afterwards.
 * l2 is scratch of 2*N entries for the 2D vgl (the reference's lapl2). */
#define ORC_LD_BODY(REAL, CELL, BASIS)                                           \
  const int N = d->num_splines;                                                  \
  int ix, iy = 0; REAL tx, ty = 0;                                               \
  CELL(&d->ax[0], 0, x, &ix, &tx);                                               \
  REAL wa[3][4], wb[3][4];                                                       \
  BASIS(tx, wa);                                                                 \
  if (dims == 2) { CELL(&d->ax[1], 0, y, &iy, &ty); BASIS(ty, wb); }            \
  const int64_t xs = NC * d->xs, ys = NC * d->ys;                                \
  const int ng = dims;                                                           \
  for (int n = 0; n < NC * N; n++) vals[n] = 0;                                  \
  if (form >= 1) for (int n = 0; n < ng * NC * N; n++) grads[n] = 0;            \
  if (dims == 1 && form >= 2) for (int n = 0; n < NC * N; n++) lh[n] = 0;       \
  if (dims == 2 && form == 2) for (int n = 0; n < 2 * NC * N; n++) l2[n] = 0;   \
  if (dims == 2 && form == 3) for (int n = 0; n < 4 * NC * N; n++) lh[n] = 0;   \
  if (dims == 1) {                                                               \
    for (int i = 0; i < 4; i++) {                                                \
      const REAL *cf = coefs + (ix+i)*xs;                                        \
      for (int n = 0; n < NC * N; n++) {                                         \
        vals[n] += wa[0][i] * cf[n];                                             \
        if (form >= 1) grads[n] += wa[1][i] * cf[n];                             \
        if (form >= 2) lh[n] += wa[2][i] * cf[n];                                \
      }                                                                          \
    }                                                                            \
    REAL dx = (REAL)d->ax[0].delta_inv;                                          \
    for (int n = 0; n < NC * N; n++) {                                           \
      if (form >= 1) grads[n] *= dx;                                             \
      if (form >= 2) lh[n] *= dx*dx;                                             \
    }                                                                            \
  } else {                                                                       \
    for (int i = 0; i < 4; i++)                                                  \
      for (int j = 0; j < 4; j++) {                                              \
        REAL ab = wa[0][i]*wb[0][j];                                             \
        REAL dab0 = wa[1][i]*wb[0][j], dab1 = wa[0][i]*wb[1][j];                 \
        REAL e0 = 0, e1 = 0, e2 = 0;                                             \
        if (form == 2) { e0 = wa[2][i]*wb[0][j]; e1 = wa[0][i]*wb[2][j]; }       \
        if (form == 3) { e0 = wa[2][i]*wb[0][j]; e1 = wa[1][i]*wb[1][j];         \
                         e2 = wa[0][i]*wb[2][j]; }                               \
        const REAL *cf = coefs + (ix+i)*xs + (iy+j)*ys;                          \
        for (int n = 0; n < N; n++)                                              \
          for (int p = 0; p < NC; p++) {                                         \
            REAL c = cf[NC*n + p];                                               \
            vals[NC*n + p] += ab * c;                                            \
            if (form >= 1) {                                                     \
              grads[NC*(2*n+0) + p] += dab0 * c;                                 \
              grads[NC*(2*n+1) + p] += dab1 * c;                                 \
            }                                                                    \
            if (form == 2) {                                                     \
              l2[NC*(2*n+0) + p] += e0 * c;                                      \
              l2[NC*(2*n+1) + p] += e1 * c;                                      \
            }                                                                    \
            if (form == 3) {                                                     \
              lh[NC*(4*n+0) + p] += e0 * c;                                      \
              lh[NC*(4*n+1) + p] += e1 * c;                                      \
              lh[NC*(4*n+3) + p] += e2 * c;                                      \
            }                                                                    \
          }                                                                      \
      }                                                                          \
    REAL dx = (REAL)d->ax[0].delta_inv, dy = (REAL)d->ax[1].delta_inv;           \
    for (int n = 0; n < N; n++)                                                  \
      for (int p = 0; p < NC; p++) {                                             \
        if (form >= 1) {                                                         \
          grads[NC*(2*n+0) + p] *= dx;                                           \
          grads[NC*(2*n+1) + p] *= dy;                                           \
        }                                                                        \
        if (form == 2) {                                                         \
          l2[NC*(2*n+0) + p] *= dx*dx;                                           \
          l2[NC*(2*n+1) + p] *= dy*dy;                                           \
          lh[NC*n + p] = l2[NC*(2*n+0) + p] + l2[NC*(2*n+1) + p];                \
        }                                                                        \
        if (form == 3) {                                                         \
          lh[NC*(4*n+0) + p] *= dx*dx;                                           \
          lh[NC*(4*n+1) + p] *= dx*dy;                                           \
          lh[NC*(4*n+3) + p] *= dy*dy;                                           \
          lh[NC*(4*n+2) + p] = lh[NC*(4*n+1) + p];                               \
        }                                                                        \
      }                                                                          \
  }

void orc_eval_ld_s(const orc_desc *d, int dims, int form, const float *coefs, double x, double y,
                   float *vals, float *grads, float *lh, float *l2)
{
  enum { NC = 1 };
  ORC_LD_BODY(float, cell_f, basis_f)
}
void orc_eval_ld_d(const orc_desc *d, int dims, int form, const double *coefs, double x, double y,
                   double *vals, double *grads, double *lh, double *l2)
{
  enum { NC = 1 };
  ORC_LD_BODY(double, cell_d, basis_d)
}
void orc_eval_ld_c(const orc_desc *d, int dims, int form, const float *coefs, double x, double y,
                   float *vals, float *grads, float *lh, float *l2)
{
  enum { NC = 2 };
  ORC_LD_BODY(float, cell_f, basis_f)
}
void orc_eval_ld_z(const orc_desc *d, int dims, int form, const double *coefs, double x, double y,
                   double *vals, double *grads, double *lh, double *l2)
{
  enum { NC = 2 };
  ORC_LD_BODY(double, cell_d, basis_d)
}

/* Many points, OpenMP over points as the reference's timing driver does
 * (src/time_multi_omp.c:61-176).  type is 's','d','c' or 'z'; pos is
 * xyz-interleaved doubles; outputs are point-major in the CPU layout. */
int orc_eval_batch(int type, int sem, int vgh, const orc_desc *d, const void *coefs, int64_t npts,
                   const double *pos, void *vals, void *grads, void *hess, int nthreads)
{
  const int64_t N = d->num_splines;
  const int nc = (type == 'c' || type == 'z') ? 2 : 1;
  const int64_t vstride = nc * N, gstride = 3 * nc * N, hstride = 9 * nc * N;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel for schedule(static) num_threads(nthreads)
#endif
  for (int64_t p = 0; p < npts; p++) {
    const double *r = pos + 3 * p;
    switch (type) {
      case 's': orc_eval_s(d, sem, vgh, (const float *)coefs, r[0], r[1], r[2],
                           (float *)vals + p*vstride, vgh ? (float *)grads + p*gstride : 0,
                           vgh ? (float *)hess + p*hstride : 0); break;
      case 'c': orc_eval_c(d, sem, vgh, (const float *)coefs, r[0], r[1], r[2],
                           (float *)vals + p*vstride, vgh ? (float *)grads + p*gstride : 0,
                           vgh ? (float *)hess + p*hstride : 0); break;
      case 'd': orc_eval_d(d, sem, vgh, (const double *)coefs, r[0], r[1], r[2],
                           (double *)vals + p*vstride, vgh ? (double *)grads + p*gstride : 0,
                           vgh ? (double *)hess + p*hstride : 0); break;
      case 'z': orc_eval_z(d, sem, vgh, (const double *)coefs, r[0], r[1], r[2],
                           (double *)vals + p*vstride, vgh ? (double *)grads + p*gstride : 0,
                           vgh ? (double *)hess + p*hstride : 0); break;
      default: break;
    }
  }
  (void)nthreads;
  return 0;
}

/* 1D/2D multi-splines at many points, OpenMP over points, outputs
 * point-major in the CPU layouts of orc_eval_ld_* (per point: vals NC*N,
 * grads dims*NC*N, lh NC*N or 4*NC*N for the 2D Hessian).  pos holds dims
 * coordinates per point.  Each thread has its own 2D-laplacian scratch. */
int orc_eval_ld_batch(int type, int dims, int form, const orc_desc *d, const void *coefs, int64_t npts,
                      const double *pos, void *vals, void *grads, void *lh, int nthreads)
{
  const int64_t N = d->num_splines;
  const int nc = (type == 'c' || type == 'z') ? 2 : 1;
  const int rb = (type == 's' || type == 'c') ? 4 : 8;
  const int64_t vs = nc * N, gs = dims * nc * N, hs = (dims == 2 && form == 3 ? 4 : 1) * nc * N;
#ifdef _OPENMP
  if (nthreads <= 0) nthreads = omp_get_max_threads();
#pragma omp parallel num_threads(nthreads)
#endif
  {
    char *l2 = (char *)malloc((size_t)(2 * nc * N + nc) * rb);
#ifdef _OPENMP
#pragma omp for schedule(static)
#endif
    for (int64_t p = 0; p < npts; p++) {
      const double x = pos[dims * p], y = dims == 2 ? pos[dims * p + 1] : 0.0;
      char *v = (char *)vals + p * vs * rb;
      char *g = form >= 1 ? (char *)grads + p * gs * rb : NULL;
      char *h = form >= 2 ? (char *)lh + p * hs * rb : NULL;
      switch (type) {
        case 's': orc_eval_ld_s(d, dims, form, (const float *)coefs, x, y, (float *)v, (float *)g, (float *)h,
                                (float *)l2); break;
        case 'c': orc_eval_ld_c(d, dims, form, (const float *)coefs, x, y, (float *)v, (float *)g, (float *)h,
                                (float *)l2); break;
        case 'd': orc_eval_ld_d(d, dims, form, (const double *)coefs, x, y, (double *)v, (double *)g,
                                (double *)h, (double *)l2); break;
        case 'z': orc_eval_ld_z(d, dims, form, (const double *)coefs, x, y, (double *)v, (double *)g,
                                (double *)h, (double *)l2); break;
        default: break;
      }
    }
    free(l2);
  }
  (void)nthreads;
  return 0;
}

/* Number of OpenMP threads the batch entry would use (1 without OpenMP). */
int orc_max_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
