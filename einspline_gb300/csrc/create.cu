// Drop-in create / set / destroy entry points and the *_cuda creators.
#include <stdlib.h>
#include <string.h>

#include <cuda_fp16.h>

#include "eg_internal.h"

using namespace eg;

namespace {

template <typename BC>
void bc_vals(const BC &bc, double lv[2], double rv[2]);

template <> void bc_vals<BCtype_s>(const BCtype_s &bc, double lv[2], double rv[2]) {
  lv[0] = bc.lVal; lv[1] = 0.0; rv[0] = bc.rVal; rv[1] = 0.0;
}
template <> void bc_vals<BCtype_d>(const BCtype_d &bc, double lv[2], double rv[2]) {
  lv[0] = bc.lVal; lv[1] = 0.0; rv[0] = bc.rVal; rv[1] = 0.0;
}
template <> void bc_vals<BCtype_c>(const BCtype_c &bc, double lv[2], double rv[2]) {
  lv[0] = bc.lVal_r; lv[1] = bc.lVal_i; rv[0] = bc.rVal_r; rv[1] = bc.rVal_i;
}
template <> void bc_vals<BCtype_z>(const BCtype_z &bc, double lv[2], double rv[2]) {
  lv[0] = bc.lVal_r; lv[1] = bc.lVal_i; rv[0] = bc.rVal_r; rv[1] = bc.rVal_i;
}

template <typename BC>
GridDesc make_axis(const Ugrid &g, const BC &bc) {
  GridDesc d;
  d.start = g.start; d.end = g.end; d.num = g.num;
  d.lcode = bc.lCode; d.rcode = bc.rCode;
  bc_vals(bc, d.lval, d.rval);
  // FLAT and NATURAL force a zero boundary value (src/bspline_create.c:1137, :1156).
  if (d.lcode == FLAT || d.lcode == NATURAL) d.lval[0] = d.lval[1] = 0.0;
  if (d.rcode == FLAT || d.rcode == NATURAL) d.rval[0] = d.rval[1] = 0.0;
  return d;
}

void fill_grid(Ugrid &u, const Table *t, int a) {
  u.start = t->start[a]; u.end = t->end[a]; u.num = t->M[a];
  u.delta = t->delta[a]; u.delta_inv = t->dinv[a];
}

// Creates the host struct S around a new table.
template <typename S, typename BC, typename V>
S *create_host(char kind, type_code tc, Ugrid xg, Ugrid yg, Ugrid zg, BC xb, BC yb, BC zb, int n, int storage) {
  clear();
  GridDesc g[3] = {make_axis(xg, xb), make_axis(yg, yb), make_axis(zg, zb)};
  Table *t = table_create(kind, g, n, storage);
  if (!t) return nullptr;
  S *s = (S *)calloc(1, sizeof(S));
  if (!s) { table_destroy(t); fail(EINSPLINE_GB300_ENOMEM, "out of host memory"); return nullptr; }
  s->spcode = MULTI_U3D;
  s->tcode = tc;
  s->coefs = (V *)t->coefs;
  const int per = t->ncomp;  // stored reals per value element
  s->x_stride = (intptr_t)(t->xs / per);
  s->y_stride = (intptr_t)(t->ys / per);
  s->z_stride = (intptr_t)(t->zs / per);
  fill_grid(s->x_grid, t, 0); fill_grid(s->y_grid, t, 1); fill_grid(s->z_grid, t, 2);
  s->xBC = xb; s->yBC = yb; s->zBC = zb;
  s->num_splines = n;
  s->gb300 = t;
  return s;
}

// 1D and 2D host structs (src/multi_bspline_create.c:88-150, :152-248 and
// the d/c/z counterparts): the first DIMS axes of a table.
template <typename S, int DIMS, typename BC, typename V>
S *create_host_ld(char kind, type_code tc, const Ugrid *ug, const BC *bc, int n) {
  clear();
  GridDesc g[3];
  for (int a = 0; a < DIMS; a++) g[a] = make_axis(ug[a], bc[a]);
  Table *t = table_create(kind, g, n, ST_NATIVE, DIMS);
  if (!t) return nullptr;
  S *s = (S *)calloc(1, sizeof(S));
  if (!s) { table_destroy(t); fail(EINSPLINE_GB300_ENOMEM, "out of host memory"); return nullptr; }
  s->spcode = DIMS == 1 ? MULTI_U1D : MULTI_U2D;
  s->tcode = tc;
  s->coefs = (V *)t->coefs;
  const int per = t->ncomp;
  s->x_stride = (intptr_t)(t->xs / per);
  fill_grid(s->x_grid, t, 0);
  s->xBC = bc[0];
  if constexpr (DIMS == 2) {
    s->y_stride = (intptr_t)(t->ys / per);
    fill_grid(s->y_grid, t, 1);
    s->yBC = bc[1];
  }
  s->num_splines = n;
  s->gb300 = t;
  return s;
}

template <typename S>
Table *table_of(S *s, const char *fn) {
  if (!s || !table_ok(s->gb300)) {
    fail(EINSPLINE_GB300_EINVAL, "%s: not a spline made by this library", fn);
    return nullptr;
  }
  return s->gb300;
}

template <typename S>
void set_host(S *s, int num, const void *data, const char *fn) {
  clear();
  Table *t = table_of(s, fn);
  if (!t) return;
  table_set(t, num, 1, data, false);
}

template <typename CS, typename G>
CS *make_cuda(Table *src, int storage, bool is_double_grid) {
  Table *t = table_clone(src, storage);
  if (!t) return nullptr;
  CS *c = (CS *)calloc(1, sizeof(CS));
  if (!c) { table_destroy(t); fail(EINSPLINE_GB300_ENOMEM, "out of host memory"); return nullptr; }
  c->coefs = (decltype(c->coefs))t->coefs;
  auto u32 = [](int64_t v) -> unsigned { return (v > 0xFFFFFFFFll) ? 0u : (unsigned)v; };
  // Strides in reals (float units for c, double units for z), as the
  // reference leaves them after upload (src/multi_bspline_create_cuda.cu:318-320).
  c->stride.x = u32(t->xs); c->stride.y = u32(t->ys); c->stride.z = u32(t->zs);
  c->gridInv.x = (G)t->dinv[0]; c->gridInv.y = (G)t->dinv[1]; c->gridInv.z = (G)t->dinv[2];
  c->dim.x = t->Nc[0] - 3; c->dim.y = t->Nc[1] - 3; c->dim.z = t->Nc[2] - 3;
  c->num_splines = t->num_splines;
  c->gb300 = t;
  (void)is_double_grid;
  return c;
}

// 1D *_cuda handles (src/multi_bspline_create_cuda.cu:17-125): a private
// device copy; stride in reals, dim = number of cells.
template <typename CS, typename G>
CS *make_cuda_1d(Table *src, int storage) {
  Table *t = table_clone(src, storage);
  if (!t) return nullptr;
  CS *c = (CS *)calloc(1, sizeof(CS));
  if (!c) { table_destroy(t); fail(EINSPLINE_GB300_ENOMEM, "out of host memory"); return nullptr; }
  c->coefs = (decltype(c->coefs))t->coefs;
  c->stride = (t->xs > 0xFFFFFFFFll) ? 0u : (unsigned)t->xs;
  c->gridInv = (G)t->dinv[0];
  c->num_splines = t->num_splines;
  c->dim = t->Nc[0] - 3;
  c->gb300 = t;
  return c;
}

template <typename S>
Table *table_of_dims(S *s, int dims, const char *fn) {
  Table *t = table_of(s, fn);
  if (t && t->dims != dims) {
    fail(EINSPLINE_GB300_EINVAL, "%s: the spline is not %dD", fn, dims);
    return nullptr;
  }
  return t;
}

template <typename CS>
void destroy_cuda(CS *c) {
  if (!c) return;
  if (table_ok(c->gb300)) {
    // A caller following the reference may already have freed ->coefs.
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, c->gb300->coefs) != cudaSuccess || at.type != cudaMemoryTypeDevice)
      c->gb300->owns = false;
    cudaGetLastError();
    table_destroy(c->gb300);
  }
  free(c);
}

}  // namespace

extern "C" {

multi_UBspline_3d_s *create_multi_UBspline_3d_s(Ugrid x, Ugrid y, Ugrid z, BCtype_s xb, BCtype_s yb, BCtype_s zb,
                                                int num_splines) {
  return create_host<multi_UBspline_3d_s, BCtype_s, float>('s', SINGLE_REAL, x, y, z, xb, yb, zb, num_splines,
                                                           ST_NATIVE);
}
multi_UBspline_3d_d *create_multi_UBspline_3d_d(Ugrid x, Ugrid y, Ugrid z, BCtype_d xb, BCtype_d yb, BCtype_d zb,
                                                int num_splines) {
  return create_host<multi_UBspline_3d_d, BCtype_d, double>('d', DOUBLE_REAL, x, y, z, xb, yb, zb, num_splines,
                                                            ST_NATIVE);
}
multi_UBspline_3d_c *create_multi_UBspline_3d_c(Ugrid x, Ugrid y, Ugrid z, BCtype_c xb, BCtype_c yb, BCtype_c zb,
                                                int num_splines) {
  return create_host<multi_UBspline_3d_c, BCtype_c, complex_float>('c', SINGLE_COMPLEX, x, y, z, xb, yb, zb,
                                                                   num_splines, ST_NATIVE);
}
multi_UBspline_3d_z *create_multi_UBspline_3d_z(Ugrid x, Ugrid y, Ugrid z, BCtype_z xb, BCtype_z yb, BCtype_z zb,
                                                int num_splines) {
  return create_host<multi_UBspline_3d_z, BCtype_z, complex_double>('z', DOUBLE_COMPLEX, x, y, z, xb, yb, zb,
                                                                    num_splines, ST_NATIVE);
}

multi_UBspline_3d_s *einspline_gb300_create_3d_s(Ugrid x, Ugrid y, Ugrid z, BCtype_s xb, BCtype_s yb, BCtype_s zb,
                                                 int num_splines, int storage) {
  return create_host<multi_UBspline_3d_s, BCtype_s, float>('s', SINGLE_REAL, x, y, z, xb, yb, zb, num_splines,
                                                           storage);
}
multi_UBspline_3d_c *einspline_gb300_create_3d_c(Ugrid x, Ugrid y, Ugrid z, BCtype_c xb, BCtype_c yb, BCtype_c zb,
                                                 int num_splines, int storage) {
  return create_host<multi_UBspline_3d_c, BCtype_c, complex_float>('c', SINGLE_COMPLEX, x, y, z, xb, yb, zb,
                                                                   num_splines, storage);
}

void set_multi_UBspline_3d_s(multi_UBspline_3d_s *s, int num, float *data) {
  set_host(s, num, data, "set_multi_UBspline_3d_s");
}
void set_multi_UBspline_3d_d(multi_UBspline_3d_d *s, int num, double *data) {
  set_host(s, num, data, "set_multi_UBspline_3d_d");
}
void set_multi_UBspline_3d_c(multi_UBspline_3d_c *s, int num, complex_float *data) {
  set_host(s, num, data, "set_multi_UBspline_3d_c");
}
void set_multi_UBspline_3d_z(multi_UBspline_3d_z *s, int num, complex_double *data) {
  set_host(s, num, data, "set_multi_UBspline_3d_z");
}

void destroy_multi_UBspline(Bspline *spline) {
  if (!spline) return;
  Table *t = nullptr;
  const int tc = spline->t_code;
#define EG_HANDLE(D)                                                             \
  switch (tc) {                                                                  \
    case SINGLE_REAL: t = ((multi_UBspline_##D##_s *)spline)->gb300; break;      \
    case DOUBLE_REAL: t = ((multi_UBspline_##D##_d *)spline)->gb300; break;      \
    case SINGLE_COMPLEX: t = ((multi_UBspline_##D##_c *)spline)->gb300; break;   \
    case DOUBLE_COMPLEX: t = ((multi_UBspline_##D##_z *)spline)->gb300; break;   \
  }
  switch (spline->sp_code) {
    case MULTI_U1D: EG_HANDLE(1d) break;
    case MULTI_U2D: EG_HANDLE(2d) break;
    case MULTI_U3D: EG_HANDLE(3d) break;
    default:
      fail(EINSPLINE_GB300_EINVAL, "destroy_multi_UBspline: only uniform 1D/2D/3D multi-splines are built here");
      return;
  }
#undef EG_HANDLE
  if (table_ok(t)) table_destroy(t);
  free(spline);
}

void destroy_Bspline(void *spline) { destroy_multi_UBspline((Bspline *)spline); }

// ------------------------------------------------------------ *_cuda
multi_UBspline_3d_s_cuda *create_multi_UBspline_3d_s_cuda(multi_UBspline_3d_s *s) {
  clear();
  Table *t = table_of(s, "create_multi_UBspline_3d_s_cuda");
  return t ? make_cuda<multi_UBspline_3d_s_cuda, float>(t, ST_NATIVE, false) : nullptr;
}
multi_UBspline_3d_s_cuda *create_multi_UBspline_3d_s_cuda_conv(multi_UBspline_3d_d *s) {
  clear();
  Table *t = table_of(s, "create_multi_UBspline_3d_s_cuda_conv");
  return t ? make_cuda<multi_UBspline_3d_s_cuda, float>(t, ST_F32, false) : nullptr;
}
multi_UBspline_3d_c_cuda *create_multi_UBspline_3d_c_cuda(multi_UBspline_3d_c *s) {
  clear();
  Table *t = table_of(s, "create_multi_UBspline_3d_c_cuda");
  return t ? make_cuda<multi_UBspline_3d_c_cuda, float>(t, ST_NATIVE, false) : nullptr;
}
multi_UBspline_3d_c_cuda *create_multi_UBspline_3d_c_cuda_conv(multi_UBspline_3d_z *s) {
  clear();
  Table *t = table_of(s, "create_multi_UBspline_3d_c_cuda_conv");
  return t ? make_cuda<multi_UBspline_3d_c_cuda, float>(t, ST_F32, false) : nullptr;
}
multi_UBspline_3d_d_cuda *create_multi_UBspline_3d_d_cuda(multi_UBspline_3d_d *s) {
  clear();
  Table *t = table_of(s, "create_multi_UBspline_3d_d_cuda");
  return t ? make_cuda<multi_UBspline_3d_d_cuda, double>(t, ST_NATIVE, true) : nullptr;
}
multi_UBspline_3d_z_cuda *create_multi_UBspline_3d_z_cuda(multi_UBspline_3d_z *s) {
  clear();
  Table *t = table_of(s, "create_multi_UBspline_3d_z_cuda");
  return t ? make_cuda<multi_UBspline_3d_z_cuda, double>(t, ST_NATIVE, true) : nullptr;
}
multi_UBspline_3d_s_cuda *einspline_gb300_create_3d_s_cuda_from_d(multi_UBspline_3d_d *s, int storage) {
  clear();
  if (storage == ST_NATIVE) storage = ST_F32;
  if (storage != ST_F32 && !is16(storage)) {
    fail(EINSPLINE_GB300_EINVAL, "storage must be F32, F16, BF16 or I16");
    return nullptr;
  }
  Table *t = table_of(s, "einspline_gb300_create_3d_s_cuda_from_d");
  return t ? make_cuda<multi_UBspline_3d_s_cuda, float>(t, storage, false) : nullptr;
}
multi_UBspline_3d_c_cuda *einspline_gb300_create_3d_c_cuda_from_z(multi_UBspline_3d_z *s, int storage) {
  clear();
  if (storage == ST_NATIVE) storage = ST_F32;
  if (storage != ST_F32 && !is16(storage)) {
    fail(EINSPLINE_GB300_EINVAL, "storage must be F32, F16, BF16 or I16");
    return nullptr;
  }
  Table *t = table_of(s, "einspline_gb300_create_3d_c_cuda_from_z");
  return t ? make_cuda<multi_UBspline_3d_c_cuda, float>(t, storage, false) : nullptr;
}

void destroy_multi_UBspline_3d_s_cuda(multi_UBspline_3d_s_cuda *c) { destroy_cuda(c); }
void destroy_multi_UBspline_3d_c_cuda(multi_UBspline_3d_c_cuda *c) { destroy_cuda(c); }
void destroy_multi_UBspline_3d_d_cuda(multi_UBspline_3d_d_cuda *c) { destroy_cuda(c); }
void destroy_multi_UBspline_3d_z_cuda(multi_UBspline_3d_z_cuda *c) { destroy_cuda(c); }

multi_UBspline_1d_s *create_multi_UBspline_1d_s(Ugrid x, BCtype_s xb, int num_splines) {
  return create_host_ld<multi_UBspline_1d_s, 1, BCtype_s, float>('s', SINGLE_REAL, &x, &xb, num_splines);
}
multi_UBspline_2d_s *create_multi_UBspline_2d_s(Ugrid x, Ugrid y, BCtype_s xb, BCtype_s yb, int num_splines) {
  const Ugrid g[2] = {x, y};
  const BCtype_s b[2] = {xb, yb};
  return create_host_ld<multi_UBspline_2d_s, 2, BCtype_s, float>('s', SINGLE_REAL, g, b, num_splines);
}
void set_multi_UBspline_1d_s(multi_UBspline_1d_s *s, int num, float *data) {
  set_host(s, num, data, "set_multi_UBspline_1d_s");
}
void set_multi_UBspline_2d_s(multi_UBspline_2d_s *s, int num, float *data) {
  set_host(s, num, data, "set_multi_UBspline_2d_s");
}
multi_UBspline_1d_d *create_multi_UBspline_1d_d(Ugrid x, BCtype_d xb, int num_splines) {
  return create_host_ld<multi_UBspline_1d_d, 1, BCtype_d, double>('d', DOUBLE_REAL, &x, &xb, num_splines);
}
multi_UBspline_2d_d *create_multi_UBspline_2d_d(Ugrid x, Ugrid y, BCtype_d xb, BCtype_d yb, int num_splines) {
  const Ugrid g[2] = {x, y};
  const BCtype_d b[2] = {xb, yb};
  return create_host_ld<multi_UBspline_2d_d, 2, BCtype_d, double>('d', DOUBLE_REAL, g, b, num_splines);
}
void set_multi_UBspline_1d_d(multi_UBspline_1d_d *s, int num, double *data) {
  set_host(s, num, data, "set_multi_UBspline_1d_d");
}
void set_multi_UBspline_2d_d(multi_UBspline_2d_d *s, int num, double *data) {
  set_host(s, num, data, "set_multi_UBspline_2d_d");
}
multi_UBspline_1d_c *create_multi_UBspline_1d_c(Ugrid x, BCtype_c xb, int num_splines) {
  return create_host_ld<multi_UBspline_1d_c, 1, BCtype_c, complex_float>('c', SINGLE_COMPLEX, &x, &xb, num_splines);
}
multi_UBspline_2d_c *create_multi_UBspline_2d_c(Ugrid x, Ugrid y, BCtype_c xb, BCtype_c yb, int num_splines) {
  const Ugrid g[2] = {x, y};
  const BCtype_c b[2] = {xb, yb};
  return create_host_ld<multi_UBspline_2d_c, 2, BCtype_c, complex_float>('c', SINGLE_COMPLEX, g, b, num_splines);
}
void set_multi_UBspline_1d_c(multi_UBspline_1d_c *s, int num, complex_float *data) {
  set_host(s, num, data, "set_multi_UBspline_1d_c");
}
void set_multi_UBspline_2d_c(multi_UBspline_2d_c *s, int num, complex_float *data) {
  set_host(s, num, data, "set_multi_UBspline_2d_c");
}
multi_UBspline_1d_z *create_multi_UBspline_1d_z(Ugrid x, BCtype_z xb, int num_splines) {
  return create_host_ld<multi_UBspline_1d_z, 1, BCtype_z, complex_double>('z', DOUBLE_COMPLEX, &x, &xb, num_splines);
}
multi_UBspline_2d_z *create_multi_UBspline_2d_z(Ugrid x, Ugrid y, BCtype_z xb, BCtype_z yb, int num_splines) {
  const Ugrid g[2] = {x, y};
  const BCtype_z b[2] = {xb, yb};
  return create_host_ld<multi_UBspline_2d_z, 2, BCtype_z, complex_double>('z', DOUBLE_COMPLEX, g, b, num_splines);
}
void set_multi_UBspline_1d_z(multi_UBspline_1d_z *s, int num, complex_double *data) {
  set_host(s, num, data, "set_multi_UBspline_1d_z");
}
void set_multi_UBspline_2d_z(multi_UBspline_2d_z *s, int num, complex_double *data) {
  set_host(s, num, data, "set_multi_UBspline_2d_z");
}
// src/multi_bspline_create.c:830-836 (d) and the z counterpart: one spline
// solved with its own x boundary condition (codes of the same periodicity as
// the table's).
void set_multi_UBspline_1d_d_BC(multi_UBspline_1d_d *s, int num, double *data, BCtype_d xBC) {
  clear();
  Table *t = table_of_dims(s, 1, "set_multi_UBspline_1d_d_BC");
  if (!t) return;
  const double lv[2] = {xBC.lVal, 0.0}, rv[2] = {xBC.rVal, 0.0};
  table_set_bc(t, num, data, xBC.lCode, xBC.rCode, lv, rv);
}
void set_multi_UBspline_1d_z_BC(multi_UBspline_1d_z *s, int num, complex_double *data, BCtype_z xBC) {
  clear();
  Table *t = table_of_dims(s, 1, "set_multi_UBspline_1d_z_BC");
  if (!t) return;
  const double lv[2] = {xBC.lVal_r, xBC.lVal_i}, rv[2] = {xBC.rVal_r, xBC.rVal_i};
  table_set_bc(t, num, data, xBC.lCode, xBC.rCode, lv, rv);
}

multi_UBspline_1d_s_cuda *create_multi_UBspline_1d_s_cuda(multi_UBspline_1d_s *s) {
  clear();
  Table *t = table_of_dims(s, 1, "create_multi_UBspline_1d_s_cuda");
  return t ? make_cuda_1d<multi_UBspline_1d_s_cuda, float>(t, ST_NATIVE) : nullptr;
}
multi_UBspline_1d_s_cuda *create_multi_UBspline_1d_s_cuda_conv(multi_UBspline_1d_d *s) {
  clear();
  Table *t = table_of_dims(s, 1, "create_multi_UBspline_1d_s_cuda_conv");
  return t ? make_cuda_1d<multi_UBspline_1d_s_cuda, float>(t, ST_F32) : nullptr;
}
multi_UBspline_1d_c_cuda *create_multi_UBspline_1d_c_cuda(multi_UBspline_1d_c *s) {
  clear();
  Table *t = table_of_dims(s, 1, "create_multi_UBspline_1d_c_cuda");
  return t ? make_cuda_1d<multi_UBspline_1d_c_cuda, float>(t, ST_NATIVE) : nullptr;
}
multi_UBspline_1d_c_cuda *create_multi_UBspline_1d_c_cuda_conv(multi_UBspline_1d_z *s) {
  clear();
  Table *t = table_of_dims(s, 1, "create_multi_UBspline_1d_c_cuda_conv");
  return t ? make_cuda_1d<multi_UBspline_1d_c_cuda, float>(t, ST_F32) : nullptr;
}
multi_UBspline_1d_d_cuda *create_multi_UBspline_1d_d_cuda(multi_UBspline_1d_d *s) {
  clear();
  Table *t = table_of_dims(s, 1, "create_multi_UBspline_1d_d_cuda");
  return t ? make_cuda_1d<multi_UBspline_1d_d_cuda, double>(t, ST_NATIVE) : nullptr;
}
multi_UBspline_1d_z_cuda *create_multi_UBspline_1d_z_cuda(multi_UBspline_1d_z *s) {
  clear();
  Table *t = table_of_dims(s, 1, "create_multi_UBspline_1d_z_cuda");
  return t ? make_cuda_1d<multi_UBspline_1d_z_cuda, double>(t, ST_NATIVE) : nullptr;
}
void destroy_multi_UBspline_1d_s_cuda(multi_UBspline_1d_s_cuda *c) { destroy_cuda(c); }
void destroy_multi_UBspline_1d_c_cuda(multi_UBspline_1d_c_cuda *c) { destroy_cuda(c); }
void destroy_multi_UBspline_1d_d_cuda(multi_UBspline_1d_d_cuda *c) { destroy_cuda(c); }
void destroy_multi_UBspline_1d_z_cuda(multi_UBspline_1d_z_cuda *c) { destroy_cuda(c); }

// ------------------------------------------------------------ extensions
int einspline_gb300_set_3d_device(einspline_gb300_table *t, int first, int count, const void *data_d) {
  clear();
  if (!table_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_set_3d_device: bad table handle");
  return table_set(t, first, count, data_d, true);
}

int einspline_gb300_flush(einspline_gb300_table *t) {
  clear();
  if (!table_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_flush: bad table handle");
  return table_flush(t);
}

int einspline_gb300_get_table_info(einspline_gb300_table *t, einspline_gb300_table_info *o) {
  clear();
  if (!table_ok(t) || !o) return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_get_table_info: bad argument");
  o->kind = t->kind;
  o->storage = t->storage;
  o->num_splines = t->num_splines;
  o->ncol = t->ncol;
  o->ncol_pad = t->ncol_pad;
  o->elem_bytes = t->elem_bytes;
  o->nx = t->Nc[0]; o->ny = t->Nc[1]; o->nz = t->Nc[2];
  o->x_stride = t->xs; o->y_stride = t->ys; o->z_stride = t->zs;
  o->table_bytes = t->table_bytes;
  o->coefs = t->coefs;
  o->scale = t->scale;
  return 0;
}

}  // extern "C"

namespace {
// Stored 16-bit reals times their column's factor, into the mirror's floats
// (written through its mapped device address): row r of the table, column c.
__global__ void k_dequant(const unsigned short *__restrict__ tab, const float *__restrict__ scale, int storage,
                          int ncol, int ncol_pad, int64_t rows, float *__restrict__ out) {
  const int64_t n = rows * ncol_pad;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int c = (int)(i % ncol_pad);
    const unsigned short u = tab[i];
    float v;
    if (storage == ST_F16) v = __half2float(__ushort_as_half(u));
    else if (storage == ST_BF16) v = __uint_as_float((unsigned)u << 16);
    else v = (float)((int)u - kI16Bias);
    out[i] = c < ncol ? v * scale[c] : 0.f;
  }
}
}  // namespace

extern "C" {

int einspline_gb300_host_coefs(einspline_gb300_table *t, void **coefs_out) {
  clear();
  if (!table_ok(t) || !coefs_out) return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_host_coefs: bad argument");
  if (int r = table_flush(t)) return r;
  std::lock_guard<std::mutex> g(t->mu);
  const bool narrow = t->storage == ST_F16 || t->storage == ST_BF16 || t->storage == ST_I16;
  const size_t reals = t->table_bytes / t->elem_bytes;
  const size_t bytes = reals * (narrow ? sizeof(float) : (size_t)t->elem_bytes);
  if (!t->host_coefs) {
    if (cudaHostAlloc(&t->host_coefs, bytes, cudaHostAllocMapped) != cudaSuccess) {
      cudaGetLastError();
      t->host_coefs = nullptr;
      return fail(EINSPLINE_GB300_ENOMEM, "einspline_gb300_host_coefs: cannot allocate %zu bytes of host memory",
                  bytes);
    }
    t->host_coefs_bytes = bytes;
  }
  EG_CUDA(cudaStreamSynchronize(t->stream));
  if (narrow) {
    void *dev = nullptr;
    EG_CUDA(cudaHostGetDevicePointer(&dev, t->host_coefs, 0));
    const int64_t rows = (int64_t)(reals / t->ncol_pad);
    k_dequant<<<2048, 256, 0, t->stream>>>((const unsigned short *)t->coefs, t->scale, t->storage, t->ncol,
                                          t->ncol_pad, rows, (float *)dev);
    count_launch();
    EG_CUDA(cudaGetLastError());
    EG_CUDA(cudaStreamSynchronize(t->stream));
  } else {
    EG_CUDA(cudaMemcpy(t->host_coefs, t->coefs, bytes, cudaMemcpyDeviceToHost));
  }
  *coefs_out = t->host_coefs;
  return 0;
}

int einspline_gb300_push_host_coefs(einspline_gb300_table *t) {
  clear();
  if (!table_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_push_host_coefs: bad table handle");
  if (!t->host_coefs)
    return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_push_host_coefs: no host mirror (einspline_gb300_host_coefs)");
  if (t->storage == ST_F16 || t->storage == ST_BF16 || t->storage == ST_I16)
    return fail(EINSPLINE_GB300_EINVAL,
                "einspline_gb300_push_host_coefs: 16-bit tables are built from data by set_* (their mirror is read-only)");
  if (int r = table_flush(t)) return r;
  std::lock_guard<std::mutex> g(t->mu);
  EG_CUDA(cudaStreamSynchronize(t->stream));
  EG_CUDA(cudaMemcpy(t->coefs, t->host_coefs, t->table_bytes, cudaMemcpyHostToDevice));
  t->df_stale = true;  // a double-float copy is rebuilt before its next use
  return 0;
}

int einspline_gb300_release_host_coefs(einspline_gb300_table *t) {
  clear();
  if (!table_ok(t)) return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_release_host_coefs: bad table handle");
  std::lock_guard<std::mutex> g(t->mu);
  if (t->host_coefs) cudaFreeHost(t->host_coefs);
  t->host_coefs = nullptr;
  t->host_coefs_bytes = 0;
  return 0;
}

int einspline_gb300_copy_table(einspline_gb300_table *t, void *host_dst, float *scale_host) {
  clear();
  if (!table_ok(t) || !host_dst) return fail(EINSPLINE_GB300_EINVAL, "einspline_gb300_copy_table: bad argument");
  if (int r = table_flush(t)) return r;
  EG_CUDA(cudaStreamSynchronize(t->stream));
  EG_CUDA(cudaMemcpy(host_dst, t->coefs, t->table_bytes, cudaMemcpyDeviceToHost));
  if (scale_host) {
    if (t->scale) EG_CUDA(cudaMemcpy(scale_host, t->scale, sizeof(float) * t->ncol, cudaMemcpyDeviceToHost));
    else for (int i = 0; i < t->ncol; i++) scale_host[i] = 1.0f;
  }
  return 0;
}

}  // extern "C"
