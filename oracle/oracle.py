"""ctypes wrapper for the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a plain-C restatement of einspline's uniform 3D multi-spline
solve and evaluation (oracle/einspline_oracle.c).  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline leg may import this module,
and only to check or to time the CPU path; the GPU library never uses it.

Also wraps the reference's own CPU library (oracle/_ref/libeinspline_ref.so,
built from the reference sources by ``make -C oracle ref``) when it exists, so
that tests can pin the oracle against it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "build")
REF_LIB = os.path.join(HERE, "_ref", "libeinspline_ref.so")

PERIODIC, DERIV1, DERIV2, FLAT, NATURAL, ANTIPERIODIC = range(6)


class OrcAxis(C.Structure):
    _fields_ = [("start", C.c_double), ("end", C.c_double), ("delta", C.c_double),
                ("delta_inv", C.c_double), ("num", C.c_int), ("ncoef", C.c_int),
                ("lcode", C.c_int), ("rcode", C.c_int),
                ("lval", C.c_double * 2), ("rval", C.c_double * 2)]


class OrcDesc(C.Structure):
    _fields_ = [("ax", OrcAxis * 3), ("num_splines", C.c_int),
                ("xs", C.c_int64), ("ys", C.c_int64), ("zs", C.c_int64)]


def build(fast: bool = True) -> None:
    """Compile the oracle libraries with make (cheap; no-op when up to date)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


_libs: dict = {}


def lib(fast: bool = False) -> C.CDLL:
    name = "liboracle_fast.so" if fast else "liboracle.so"
    if name not in _libs:
        path = os.path.join(BUILD, name)
        if not os.path.exists(path):
            build()
        L = C.CDLL(path)
        L.orc_axis_init.argtypes = [C.POINTER(OrcAxis), C.c_double, C.c_double, C.c_int, C.c_int,
                                    C.c_int, C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_axis_init.restype = C.c_int
        L.orc_find_coefs_1d_d.argtypes = [C.POINTER(OrcAxis), C.c_int, C.c_void_p, C.c_int64,
                                          C.c_void_p, C.c_int64]
        L.orc_set_3d_column_d.argtypes = [C.POINTER(OrcDesc), C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        L.orc_set_column_d.argtypes = [C.POINTER(OrcDesc), C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        for t in "sdcz":
            getattr(L, f"orc_eval_ld_{t}").argtypes = [C.POINTER(OrcDesc), C.c_int, C.c_int, C.c_void_p, C.c_double,
                                                      C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        for t in "sdcz":
            f = getattr(L, "orc_eval_" + t)
            f.argtypes = [C.POINTER(OrcDesc), C.c_int, C.c_int, C.c_void_p, C.c_double, C.c_double,
                          C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
        for t in "sdcz":
            f = getattr(L, f"orc_eval_{t}_vghgh")
            f.argtypes = [C.POINTER(OrcDesc), C.c_void_p, C.c_double, C.c_double, C.c_double, C.c_void_p,
                          C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_eval_batch.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(OrcDesc), C.c_void_p,
                                     C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_eval_batch.restype = C.c_int
        L.orc_eval_ld_batch.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(OrcDesc), C.c_void_p, C.c_int64,
                                        C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_eval_ld_batch.restype = C.c_int
        L.orc_max_threads.restype = C.c_int
        _libs[name] = L
    return _libs[name]


def ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)


class Table:
    """A uniform 3D multi-spline held by the oracle: grid/BC description plus
    a coefficient table coefs[Nx][Ny][Nz][N] (complex types: trailing axis of
    2 for re/im).  ``kind`` is one of 's','d','c','z'."""

    def __init__(self, kind, grids, bcs, num_splines):
        # grids: dims x (start, end, num); bcs: dims x (lcode, rcode, lval_r, lval_i, rval_r, rval_i),
        # dims = 1, 2 or 3 (the 1D/2D/3D multi-splines)
        self.kind = kind
        self.dims = len(grids)
        self.ncomp = 2 if kind in "cz" else 1
        self.dtype = np.float32 if kind in "sc" else np.float64
        self.desc = OrcDesc()
        L = lib()
        shape = []
        for a in range(self.dims):
            st, en, num = grids[a]
            lc, rc, *vals = bcs[a]
            vals = list(vals) + [0.0] * (4 - len(vals))
            n = L.orc_axis_init(C.byref(self.desc.ax[a]), st, en, num, lc, rc, *vals)
            shape.append(n)
        for a in range(self.dims, 3):        # absent axes: one point, one coefficient
            self.desc.ax[a].num = 1
            self.desc.ax[a].ncoef = 1
        ext = list(shape) + [1] * (3 - self.dims)
        self.desc.num_splines = num_splines
        self.N = num_splines
        self.shape = tuple(shape)
        self.desc.zs = num_splines
        self.desc.ys = ext[2] * num_splines
        self.desc.xs = ext[1] * ext[2] * num_splines
        full = tuple(shape) + (num_splines,) + ((2,) if self.ncomp == 2 else ())
        # FP64 solve target; for s/c the table is this rounded to float32.
        self.coefs64 = np.zeros(full, dtype=np.float64)
        self._coefs = None

    @property
    def M(self):
        return tuple(self.desc.ax[a].num for a in range(3))

    def set_spline(self, i: int, data: np.ndarray) -> None:
        """FP64 solve of one spline column (set_multi_UBspline_3d_d/z); data
        has shape (Mx,My,Mz) real or (Mx,My,Mz,2) / complex."""
        d = np.ascontiguousarray(_as_pairs(data, self.ncomp), dtype=np.float64)
        lib().orc_set_column_d(C.byref(self.desc), self.dims, self.ncomp, i, ptr(self.coefs64), ptr(d))
        self._coefs = None

    @property
    def coefs(self) -> np.ndarray:
        """Table in its storage precision (FP64 solve rounded once for s/c)."""
        if self._coefs is None:
            self._coefs = np.ascontiguousarray(self.coefs64.astype(self.dtype))
        return self._coefs

    def eval_ld(self, pos, form: int = 3, coefs: np.ndarray = None):
        """1D/2D tables: eval_multi_UBspline_{1,2}d_* at each position (CPU
        rule).  form 0 value, 1 vg, 2 vgl, 3 vgh.  Returns vals [P][N],
        grads [P][N] (1D) or [P][N][2] (2D), and lh: the second derivative
        [P][N] (1D vgl/vgh), the laplacian [P][N] (2D vgl) or the Hessian
        [P][N][2][2] (2D vgh); complex types add a trailing axis of 2."""
        assert self.dims in (1, 2)
        cf = self.coefs if coefs is None else np.ascontiguousarray(coefs)
        return _eval_ld(lambda v, g, lh, l2, x, y: getattr(lib(), f"orc_eval_ld_{self.kind}")(
            C.byref(self.desc), self.dims, form, ptr(cf), x, y, ptr(v), ptr(g), ptr(lh), ptr(l2)),
            self.dims, form, pos, self.dtype, self.N, self.ncomp)

    def eval_ld_batch(self, pos, form: int = 2, coefs: np.ndarray = None, nthreads: int = 0, fast: bool = False):
        """eval_ld for many points with OpenMP (the timed CPU path): same
        outputs as eval_ld."""
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, self.dims)
        P = pos.shape[0]
        cf = self.coefs if coefs is None else np.ascontiguousarray(coefs)
        ext = (2,) if self.ncomp == 2 else ()
        v = np.zeros((P, self.N) + ext, self.dtype)
        g = np.zeros((P, self.N) + ((2,) if self.dims == 2 else ()) + ext, self.dtype) if form >= 1 else None
        h = None
        if form >= 2:
            h = np.zeros((P, self.N) + ((2, 2) if self.dims == 2 and form == 3 else ()) + ext, self.dtype)
        lib(fast).orc_eval_ld_batch(ord(self.kind), self.dims, form, C.byref(self.desc), ptr(cf), P, ptr(pos),
                                    ptr(v), ptr(g), ptr(h), nthreads)
        return v, g, h

    def eval_vghgh(self, pos: np.ndarray, coefs: np.ndarray = None):
        """Value, gradient, Hessian and third derivatives [P][N][3][3][3]
        (CPU-entry rule), as eval_multi_UBspline_3d_*_vghgh."""
        cf = self.coefs if coefs is None else np.ascontiguousarray(coefs)
        f = getattr(lib(), f"orc_eval_{self.kind}_vghgh")
        return _vghgh(lambda o, c, x, y, z, v, g, h, gh: f(C.byref(o), ptr(c), x, y, z, ptr(v), ptr(g), ptr(h),
                                                           ptr(gh)),
                      self.desc, pos, self.dtype, self.N, self.ncomp, cf)

    def eval(self, pos: np.ndarray, vgh: bool = True, sem: int = 0, coefs: np.ndarray = None,
             nthreads: int = 0, fast: bool = False):
        """Evaluate at pos (npts,3).  sem=0: CPU-entry semantics; sem=1: the
        reference GPU entries' cell rule.  Returns vals, grads, hess in the
        CPU layout ([P][N], [P][N][3], [P][N][3][3], complex as a trailing 2)."""
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        P = pos.shape[0]
        cf = self.coefs if coefs is None else np.ascontiguousarray(coefs)
        assert cf.dtype == self.dtype
        ext = (2,) if self.ncomp == 2 else ()
        v = np.zeros((P, self.N) + ext, self.dtype)
        g = np.zeros((P, self.N, 3) + ext, self.dtype) if vgh else None
        h = np.zeros((P, self.N, 3, 3) + ext, self.dtype) if vgh else None
        lib(fast).orc_eval_batch(ord(self.kind), sem, int(vgh), C.byref(self.desc), ptr(cf), P,
                                 ptr(pos), ptr(v), ptr(g), ptr(h), nthreads)
        return v, g, h


def _vghgh(fn, obj, pos, dtype, N, ncomp, coefs):
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
    P = pos.shape[0]
    ext = (2,) if ncomp == 2 else ()
    v = np.zeros((P, N) + ext, dtype)
    g = np.zeros((P, N, 3) + ext, dtype)
    h = np.zeros((P, N, 3, 3) + ext, dtype)
    gh = np.zeros((P, N, 3, 3, 3) + ext, dtype)
    for p in range(P):
        fn(obj, coefs, *[float(c) for c in pos[p]], v[p], g[p], h[p], gh[p])
    return v, g, h, gh


def _eval_ld(fn, dims, form, pos, dtype, N, ncomp):
    pos = np.asarray(pos, dtype=np.float64).reshape(-1, dims)
    P = pos.shape[0]
    ext = (2,) if ncomp == 2 else ()
    v = np.zeros((P, N) + ext, dtype)
    g = np.zeros((P, N) + ((dims,) if dims == 2 else ()) + ext, dtype)
    if dims == 1:
        lh = np.zeros((P, N) + ext, dtype)
    else:
        lh = np.zeros((P, N) + ((2, 2) if form == 3 else ()) + ext, dtype)
    # one spare entry per buffer: the reference's 2D vg clears grads[2N]
    gbuf = np.zeros(g[0].size + ncomp, dtype)
    l2 = np.zeros(2 * N * ncomp + ncomp, dtype)
    for p in range(P):
        y = float(pos[p, 1]) if dims == 2 else 0.0
        fn(v[p], gbuf, lh[p], l2, float(pos[p, 0]), y)
        g[p] = gbuf[:g[0].size].reshape(g[0].shape)
    out = [v, g if form >= 1 else None, lh if form >= 2 else None]
    return out


def _as_pairs(data, ncomp):
    data = np.asarray(data)
    if ncomp == 2 and np.iscomplexobj(data):
        return np.stack([data.real, data.imag], axis=-1)
    return data


# --------------------------------------------------------------------------
# The reference's own CPU library (optional: present only where the
# reference sources were available to compile).
# --------------------------------------------------------------------------
class RefUgrid(C.Structure):
    _fields_ = [("start", C.c_double), ("end", C.c_double), ("num", C.c_int),
                ("delta", C.c_double), ("delta_inv", C.c_double)]


class RefBC_s(C.Structure):
    _fields_ = [("lCode", C.c_int), ("rCode", C.c_int), ("lVal", C.c_float), ("rVal", C.c_float)]


class RefBC_d(C.Structure):
    _fields_ = [("lCode", C.c_int), ("rCode", C.c_int), ("lVal", C.c_double), ("rVal", C.c_double)]


class RefBC_c(C.Structure):
    _fields_ = [("lCode", C.c_int), ("rCode", C.c_int), ("lVal_r", C.c_float), ("lVal_i", C.c_float),
                ("rVal_r", C.c_float), ("rVal_i", C.c_float)]


class RefBC_z(C.Structure):
    _fields_ = [("lCode", C.c_int), ("rCode", C.c_int), ("lVal_r", C.c_double), ("lVal_i", C.c_double),
                ("rVal_r", C.c_double), ("rVal_i", C.c_double)]


def _ref_struct(bc_t):
    class S(C.Structure):
        _fields_ = [("spcode", C.c_int), ("tcode", C.c_int), ("coefs", C.c_void_p),
                    ("x_stride", C.c_ssize_t), ("y_stride", C.c_ssize_t), ("z_stride", C.c_ssize_t),
                    ("x_grid", RefUgrid), ("y_grid", RefUgrid), ("z_grid", RefUgrid),
                    ("xBC", bc_t), ("yBC", bc_t), ("zBC", bc_t), ("num_splines", C.c_int)]
    return S


REF_BC = {"s": RefBC_s, "d": RefBC_d, "c": RefBC_c, "z": RefBC_z}
REF_STRUCT = {k: _ref_struct(v) for k, v in REF_BC.items()}


def _ref_struct_ld(bc_t, dims):
    """multi_UBspline_{1,2}d_* (src/multi_bspline_structs.h:28-51 and alike);
    the 2D complex structs' trailing lapl2 pointer is not read here."""
    ax = "xy"[:dims]
    fields = [("spcode", C.c_int), ("tcode", C.c_int), ("coefs", C.c_void_p)]
    fields += [(f"{a}_stride", C.c_ssize_t) for a in ax] + [(f"{a}_grid", RefUgrid) for a in ax]
    fields += [(f"{a}BC", bc_t) for a in ax] + [("num_splines", C.c_int)]
    return type(f"RefMulti{dims}D", (C.Structure,), {"_fields_": fields})


REF_STRUCT_LD = {(k, d): _ref_struct_ld(v, d) for k, v in REF_BC.items() for d in (1, 2)}
LD_SUFFIX = ("", "_vg", "_vgl", "_vgh")


def ref_available() -> bool:
    return os.path.exists(REF_LIB)


_ref = None


def ref_lib() -> C.CDLL:
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_LIB)
        for t in "sdcz":
            S = REF_STRUCT[t]
            bc = REF_BC[t]
            f = getattr(_ref, f"create_multi_UBspline_3d_{t}")
            f.argtypes = [RefUgrid] * 3 + [bc] * 3 + [C.c_int]
            f.restype = C.POINTER(S)
            getattr(_ref, f"set_multi_UBspline_3d_{t}").argtypes = [C.POINTER(S), C.c_int, C.c_void_p]
            getattr(_ref, f"eval_multi_UBspline_3d_{t}").argtypes = [C.POINTER(S), C.c_double, C.c_double,
                                                                     C.c_double, C.c_void_p]
            getattr(_ref, f"eval_multi_UBspline_3d_{t}_vgh").argtypes = [
                C.POINTER(S), C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p]
            getattr(_ref, f"eval_multi_UBspline_3d_{t}_vghgh").argtypes = [
                C.POINTER(S), C.c_double, C.c_double, C.c_double, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        for t in "sdcz":
            for dims in (1, 2):
                S = REF_STRUCT_LD[(t, dims)]
                f = getattr(_ref, f"create_multi_UBspline_{dims}d_{t}")
                f.argtypes = [RefUgrid] * dims + [REF_BC[t]] * dims + [C.c_int]
                f.restype = C.POINTER(S)
                getattr(_ref, f"set_multi_UBspline_{dims}d_{t}").argtypes = [C.POINTER(S), C.c_int, C.c_void_p]
                for form, suf in enumerate(LD_SUFFIX):
                    getattr(_ref, f"eval_multi_UBspline_{dims}d_{t}{suf}").argtypes = (
                        [C.POINTER(S)] + [C.c_double] * dims + [C.c_void_p] * (1 + min(form, 2)))
        _ref.destroy_Bspline.argtypes = [C.c_void_p]
    return _ref


class RefSplineLD:
    """A 1D or 2D multi-spline built by the reference's create/set."""

    def __init__(self, kind, grids, bcs, num_splines):
        L = ref_lib()
        self.kind, self.N, self.dims = kind, num_splines, len(grids)
        self.ncomp = 2 if kind in "cz" else 1
        self.dtype = np.float32 if kind in "sc" else np.float64
        ug = [RefUgrid(g[0], g[1], g[2], 0.0, 0.0) for g in grids]
        BC = REF_BC[kind]
        bcs_c = []
        for b in bcs:
            lc, rc, *v = b
            v = list(v) + [0.0] * (4 - len(v))
            bcs_c.append(BC(lc, rc, v[0], v[2]) if kind in "sd" else BC(lc, rc, v[0], v[1], v[2], v[3]))
        self.p = getattr(L, f"create_multi_UBspline_{self.dims}d_{kind}")(*ug, *bcs_c, num_splines)
        s = self.p.contents
        self.shape = tuple(RefSpline._n(g, b) for g, b in zip(grids, bcs))
        self.inner = s.y_stride if self.dims == 2 else s.x_stride

    def set_spline(self, i, data):
        d = np.ascontiguousarray(_as_pairs(data, self.ncomp), dtype=self.dtype)
        getattr(ref_lib(), f"set_multi_UBspline_{self.dims}d_{self.kind}")(self.p, i, ptr(d))

    def _view(self):
        s = self.p.contents
        n = self.shape[0] * s.x_stride * self.ncomp
        buf = (C.c_float if self.dtype == np.float32 else C.c_double) * n
        arr = np.frombuffer(buf.from_address(s.coefs), dtype=self.dtype)
        return arr.reshape(self.shape + (self.inner,) + ((2,) if self.ncomp == 2 else ()))

    def table(self) -> np.ndarray:
        return self._view()[..., :self.N, :].copy() if self.ncomp == 2 else self._view()[..., :self.N].copy()

    def load_table(self, coefs: np.ndarray) -> None:
        v = self._view()
        if self.ncomp == 2:
            v[..., :self.N, :] = coefs.astype(self.dtype)
        else:
            v[..., :self.N] = coefs.astype(self.dtype)

    def eval_ld(self, pos, form=3):
        f = getattr(ref_lib(), f"eval_multi_UBspline_{self.dims}d_{self.kind}{LD_SUFFIX[form]}")

        def call(v, g, lh, l2, x, y):
            xy = (x,) if self.dims == 1 else (x, y)
            bufs = [ptr(v), ptr(g), ptr(lh)][:1 + min(form, 2)]
            f(self.p, *xy, *bufs)
        return _eval_ld(call, self.dims, form, pos, self.dtype, self.N, self.ncomp)

    def __del__(self):
        try:
            ref_lib().destroy_Bspline(C.cast(self.p, C.c_void_p))
        except Exception:
            pass


class RefSpline:
    """A spline built by the reference's own create/set (its native solve:
    float for s/c, double for d/z)."""

    def __init__(self, kind, grids, bcs, num_splines):
        L = ref_lib()
        self.kind, self.N = kind, num_splines
        self.ncomp = 2 if kind in "cz" else 1
        self.dtype = np.float32 if kind in "sc" else np.float64
        ug = [RefUgrid(g[0], g[1], g[2], 0.0, 0.0) for g in grids]
        BC = REF_BC[kind]
        bcs_c = []
        for b in bcs:
            lc, rc, *v = b
            v = list(v) + [0.0] * (4 - len(v))
            if kind in "sd":
                bcs_c.append(BC(lc, rc, v[0], v[2]))
            else:
                bcs_c.append(BC(lc, rc, v[0], v[1], v[2], v[3]))
        self.p = getattr(L, f"create_multi_UBspline_3d_{kind}")(*ug, *bcs_c, num_splines)
        s = self.p.contents
        self.shape = tuple(self._n(g, b) for g, b in zip(grids, bcs))
        self.strides = (s.x_stride, s.y_stride, s.z_stride)

    @staticmethod
    def _n(g, b):
        return g[2] + 3 if b[0] in (PERIODIC, ANTIPERIODIC) else g[2] + 2

    def set_spline(self, i, data):
        d = np.ascontiguousarray(_as_pairs(data, self.ncomp), dtype=self.dtype)
        getattr(ref_lib(), f"set_multi_UBspline_3d_{self.kind}")(self.p, i, ptr(d))

    def table(self) -> np.ndarray:
        s = self.p.contents
        n = self.shape[0] * s.x_stride * self.ncomp
        buf = (C.c_float if self.dtype == np.float32 else C.c_double) * n
        arr = np.frombuffer(buf.from_address(s.coefs), dtype=self.dtype).copy()
        arr = arr.reshape(self.shape + (s.z_stride,) + ((2,) if self.ncomp == 2 else ()))
        return arr[:, :, :, :self.N]

    def load_table(self, coefs: np.ndarray) -> None:
        """Overwrite the reference table with coefs (same layout) so that its
        evaluators run on exactly the table under test."""
        s = self.p.contents
        n = self.shape[0] * s.x_stride * self.ncomp
        buf = (C.c_float if self.dtype == np.float32 else C.c_double) * n
        arr = np.frombuffer(buf.from_address(s.coefs), dtype=self.dtype)
        arr = arr.reshape(self.shape + (s.z_stride,) + ((2,) if self.ncomp == 2 else ()))
        arr[:, :, :, :self.N] = coefs.astype(self.dtype)

    def eval(self, pos, vgh=True):
        pos = np.asarray(pos, dtype=np.float64).reshape(-1, 3)
        P = pos.shape[0]
        ext = (2,) if self.ncomp == 2 else ()
        v = np.zeros((P, self.N) + ext, self.dtype)
        g = np.zeros((P, self.N, 3) + ext, self.dtype)
        h = np.zeros((P, self.N, 3, 3) + ext, self.dtype)
        L = ref_lib()
        fv = getattr(L, f"eval_multi_UBspline_3d_{self.kind}")
        fg = getattr(L, f"eval_multi_UBspline_3d_{self.kind}_vgh")
        for p in range(P):
            x, y, z = (float(c) for c in pos[p])
            if vgh:
                fg(self.p, x, y, z, ptr(v[p]), ptr(g[p]), ptr(h[p]))
            else:
                fv(self.p, x, y, z, ptr(v[p]))
        return (v, g, h) if vgh else (v, None, None)

    def eval_vghgh(self, pos):
        f = getattr(ref_lib(), f"eval_multi_UBspline_3d_{self.kind}_vghgh")
        return _vghgh(lambda o, c, x, y, z, v, g, h, gh: f(o, x, y, z, ptr(v), ptr(g), ptr(h), ptr(gh)),
                      self.p, pos, self.dtype, self.N, self.ncomp, None)

    def __del__(self):
        try:
            ref_lib().destroy_Bspline(C.cast(self.p, C.c_void_p))
        except Exception:
            pass


# ---------------------------------------------------------------- determinant step
# Restatement, in float64 numpy, of the reference QMC prototype's use of the
# orbital row (src/cuda_walker.cu): the ratio of calc_ratios (:171-201),
# ratio = sum_j u_j Ainv[j][k], and the two update kernels
# update_inverse_cuda1/2 (src/determinant_update.h:9-111):
#   x[c]   = sum_j Ainv[j][c] (u_j - A[k][j])          (kernel 1, :39-56)
#   Ainv[j][c] += x[c] * (-1/(1 + x[k])) * Ainv[j][k]   (kernel 2, :86-108)
#   A[k][:] = u                                         (kernel 1, :41-43)
# Ainv is indexed [orbital j][electron c]; A is [electron][orbital].

def det_ratio(vals, grads, hess, ainv, k):
    """Per walker: ratio, (sum_j grad_j Ainv[j][k]) / ratio, (sum_j lapl_j
    Ainv[j][k]) / ratio.  vals [W][N], grads [W][N][3], hess [W][N][3][3]
    (CPU layout, oracle eval), ainv [W][N][N] as Ainv[j][c]."""
    v = np.asarray(vals, np.float64)
    col = np.asarray(ainv, np.float64)[:, :, k]
    r = np.einsum("wj,wj->w", v, col)
    out = [r, None, None]
    if grads is not None:
        g = np.einsum("wjd,wj->wd", np.asarray(grads, np.float64), col)
        h = np.asarray(hess, np.float64)
        lap = h[..., 0, 0] + h[..., 1, 1] + h[..., 2, 2]
        out[1] = g / r[:, None]
        out[2] = np.einsum("wj,wj->w", lap, col) / r
    return out


def det_ratio_bound(vals, grads, hess, ainv, k):
    """sum_j |term_j| of each sum in det_ratio: the scale a rounding error of
    the dot products is measured against."""
    v = np.abs(np.asarray(vals, np.float64))
    col = np.abs(np.asarray(ainv, np.float64)[:, :, k])
    sr = np.einsum("wj,wj->w", v, col)
    if grads is None:
        return sr, None, None
    sg = np.einsum("wjd,wj->wd", np.abs(np.asarray(grads, np.float64)), col)
    h = np.asarray(hess, np.float64)
    sl = np.einsum("wj,wj->w", np.abs(h[..., 0, 0] + h[..., 1, 1] + h[..., 2, 2]), col)
    return sr, sg, sl


REF_DET_LIB = os.path.join(HERE, "_ref", "libdetupdate_ref.so")


def ref_det_update(ainv, delta, k):
    """The reference's host update_inverse (src/determinant_update.cu:171-187,
    float): its array, read as M[i][j] = X[j*N + i], is the inverse of a
    matrix whose column k changes by delta; with X = Ainv[j][e] (orbital j,
    electron e) row-major that is our row-k change of A.  N <= 128 (its
    scratch arrays).  Returns the updated Ainv (float32)."""
    L = C.CDLL(REF_DET_LIB)
    f = getattr(L, "_Z14update_inversePfS_ii")  # C++ linkage: update_inverse(float*, float*, int, int)
    f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
    X = np.ascontiguousarray(ainv, dtype=np.float32).copy()
    d = np.ascontiguousarray(delta, dtype=np.float32)
    N = X.shape[0]
    assert X.shape == (N, N) and N <= 128
    f(ptr(X), ptr(d), N, int(k))
    return X


def sm_update(A, ainv, k, u):
    """Sherman-Morrison row update of one walker in float64: returns (A', Ainv')."""
    A = np.array(A, np.float64)
    Ai = np.array(ainv, np.float64)
    u = np.asarray(u, np.float64)
    x = (u - A[k]) @ Ai
    colk = Ai[:, k].copy()
    Ai += np.outer(colk, x) * (-1.0 / (1.0 + x[k]))
    A[k] = u
    return A, Ai
