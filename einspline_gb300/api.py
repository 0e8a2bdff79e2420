"""Python handles over the C-ABI (used by tests, the benchmark and smoke()).

Mirrors the reference's uniform 3D multi-spline interface:
``MultiUBspline3D`` wraps create/set/eval_multi_UBspline_3d_{s,d,c,z}
(src/multi_bspline_create.c, src/multi_bspline_eval_std_*_impl.h) and
``CudaSpline`` wraps create_multi_UBspline_3d_*_cuda plus
eval_multi_multi_UBspline_3d_*[_vgh]_cuda (src/multi_bspline_create_cuda.cu,
src/multi_bspline_cuda_*_impl.h).  Every call goes through
libeinspline_gb300.so; torch is used only to hold device buffers.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import (ANTIPERIODIC, DERIV1, DERIV2, FLAT, NATURAL, PERIODIC, STORE_BF16, STORE_F16,  # noqa: F401
                   STORE_F32, STORE_F64, STORE_I16, STORE_NATIVE, EinsplineError, check)

_TYPE_CODE = {"s": L.SINGLE_REAL, "d": L.DOUBLE_REAL, "c": L.SINGLE_COMPLEX, "z": L.DOUBLE_COMPLEX}


def _lib():
    return L.load()


def _torch():
    import torch
    return torch


def out_dtype(kind):
    return np.float32 if kind in "sc" else np.float64


def _bc(kind, b):
    lc, rc, *v = b
    v = list(v) + [0.0] * (4 - len(v))
    BC = L.BC_TYPES[kind]
    return BC(lc, rc, v[0], v[2]) if kind in "sd" else BC(lc, rc, v[0], v[1], v[2], v[3])


class MultiUBspline3D:
    """A uniform 3D multi-spline made by this library.

    grids: three (start, end, num) tuples; bcs: three (lCode, rCode[, lVal_r,
    lVal_i, rVal_r, rVal_i]) tuples; storage: one of STORE_* (s/c only)."""

    def __init__(self, kind: str, grids, bcs, num_splines: int, storage: int = STORE_NATIVE):
        lib = _lib()
        self.kind = kind
        self.N = num_splines
        self.ncomp = 2 if kind in "cz" else 1
        self.M = tuple(int(g[2]) for g in grids)
        ug = [L.Ugrid(float(g[0]), float(g[1]), int(g[2]), 0.0, 0.0) for g in grids]
        bc = [_bc(kind, b) for b in bcs]
        if storage == STORE_NATIVE:
            f = getattr(lib, f"create_multi_UBspline_3d_{kind}")
            p = f(*ug, *bc, num_splines)
        else:
            if kind not in "sc":
                raise ValueError("only s and c tables take a storage choice")
            p = getattr(lib, f"einspline_gb300_create_3d_{kind}")(*ug, *bc, num_splines, storage)
        check()
        if not p:
            raise EinsplineError("create failed")
        self.ptr = p
        self.table = C.c_void_p(p.contents.gb300)

    # -- set ------------------------------------------------------------
    def set(self, i: int, data) -> None:
        """set_multi_UBspline_3d_*: data (Mx, My, Mz) real or complex/trailing-2 host array."""
        dt = np.float32 if self.kind in "sc" else np.float64
        d = np.asarray(data)
        if self.ncomp == 2 and np.iscomplexobj(d):
            d = np.stack([d.real, d.imag], axis=-1)
        d = np.ascontiguousarray(d, dtype=dt)
        getattr(_lib(), f"set_multi_UBspline_3d_{self.kind}")(self.ptr, i, d.ctypes.data)
        check()

    def set_device(self, first: int, data) -> None:
        """Bulk set from a torch CUDA tensor [count, Mx, My, Mz(, 2)]."""
        count = int(data.shape[0])
        _lib().einspline_gb300_set_3d_device(self.table, first, count, C.c_void_p(data.data_ptr()))
        check()

    def flush(self) -> None:
        _lib().einspline_gb300_flush(self.table)
        check()

    # -- info / table ----------------------------------------------------
    def info(self) -> L.TableInfo:
        ti = L.TableInfo()
        _lib().einspline_gb300_get_table_info(self.table, C.byref(ti))
        check()
        return ti

    def table_host(self):
        """(table, scales): the stored table as numpy [Nx][Ny][Nz][ncol_pad]
        of the storage type (bfloat16 and biased int16 patterns as uint16)."""
        ti = self.info()
        dt = {1: np.float32, 2: np.float16, 3: np.uint16, 4: np.float64, 5: np.uint16}[ti.storage]
        out = np.empty((ti.nx, ti.ny, ti.nz, ti.ncol_pad), dtype=dt)
        sc = np.empty(ti.ncol, dtype=np.float32)
        _lib().einspline_gb300_copy_table(self.table, out.ctypes.data, sc.ctypes.data)
        check()
        return out, sc

    def host_coefs(self) -> np.ndarray:
        """The coefficients in host memory as the reference keeps them: a
        numpy view [Nx][Ny][Nz][ncol_pad] of the library's pinned mirror, in
        the value's real type (float32 for s/c, float64 for d/z; 16-bit
        tables dequantized).  Edits reach the device table through
        push_host_coefs (FP32 and FP64 tables)."""
        ti = self.info()
        p = C.c_void_p()
        _lib().einspline_gb300_host_coefs(self.table, C.byref(p))
        check()
        dt = np.float64 if self.kind in "dz" else np.float32
        n = ti.nx * ti.ny * ti.nz * ti.ncol_pad
        buf = (C.c_char * (n * np.dtype(dt).itemsize)).from_address(p.value)
        return np.frombuffer(buf, dtype=dt).reshape(ti.nx, ti.ny, ti.nz, ti.ncol_pad)

    def push_host_coefs(self) -> None:
        """Upload the host mirror (after edits) into the device table."""
        _lib().einspline_gb300_push_host_coefs(self.table)
        check()

    def release_host_coefs(self) -> None:
        """Free the host mirror; views from host_coefs become invalid."""
        _lib().einspline_gb300_release_host_coefs(self.table)
        check()

    def table_values(self) -> np.ndarray:
        """Dequantized table as float64 [Nx][Ny][Nz][N] (complex: [..., N, 2])."""
        t, sc = self.table_host()
        ti = self.info()
        if ti.storage == STORE_BF16:
            t = (t.astype(np.uint32) << 16).view(np.float32)
        elif ti.storage == STORE_I16:
            t = t.astype(np.int32) - L.I16_BIAS
        v = t[..., :ti.ncol].astype(np.float64) * sc.astype(np.float64)
        if self.ncomp == 2:
            v = v.reshape(v.shape[:3] + (self.N, 2))
        return v

    # -- tiles -----------------------------------------------------------
    def set_tile(self, tx: int, ty: int, pb: int) -> None:
        _lib().einspline_gb300_set_tile(self.table, tx, ty, pb)
        check()

    def get_tile(self):
        a, b, c = C.c_int(), C.c_int(), C.c_int()
        _lib().einspline_gb300_get_tile(self.table, C.byref(a), C.byref(b), C.byref(c))
        check()
        return a.value, b.value, c.value

    def set_load_mode(self, mode: int) -> None:
        """0 direct loads, 1 L2 bulk prefetch, 2 shared-memory async pipeline,
        3 the same with 8 columns a thread (16-bit tables), 4 shared-memory
        pipeline fed by tensor-map (TMA) copies, 5 tensor-core reduction (F16
        tables; FP32-rounding agreement, not bit-identical), -1 autotuned."""
        _lib().einspline_gb300_set_load_mode(self.table, int(mode))
        check()

    def wait_status(self) -> None:
        """Raises (ETIMEOUT) when a TMA-staged launch on this table gave up a
        bounded barrier wait since the last check; call after synchronising."""
        _lib().einspline_gb300_wait_status(self.table)
        check()

    def launch_shape(self, sorted: bool = False, vgh: bool = True):
        """(tx, ty, pb, load mode) of a random-order or cell-sorted launch."""
        v = [C.c_int() for _ in range(4)]
        _lib().einspline_gb300_get_launch_shape(self.table, int(sorted), int(vgh), *[C.byref(x) for x in v])
        check()
        return tuple(x.value for x in v)

    def get_load_mode(self) -> int:
        r = _lib().einspline_gb300_get_load_mode(self.table)
        check()
        return int(r)

    def autotune(self, npts: int, vgh: bool = True, sorted: bool = False):
        """Time every tile and load mode for batches of npts random points
        (sorted: for cell-sorted launches of such batches) and keep the
        fastest; returns the random-order tile."""
        fn = _lib().einspline_gb300_autotune_sorted if sorted else _lib().einspline_gb300_autotune
        fn(self.table, npts, int(vgh))
        check()
        return self.get_tile()

    # -- evaluation --------------------------------------------------------
    def eval_point(self, x: float, y: float, z: float, vgh: bool = True):
        """eval_multi_UBspline_3d_*[_vgh] at one point, CPU layout."""
        dt = out_dtype(self.kind)
        ext = (2,) if self.ncomp == 2 else ()
        v = np.zeros((self.N,) + ext, dt)
        lib = _lib()
        if vgh:
            g = np.zeros((self.N, 3) + ext, dt)
            h = np.zeros((self.N, 3, 3) + ext, dt)
            getattr(lib, f"eval_multi_UBspline_3d_{self.kind}_vgh")(self.ptr, x, y, z, v.ctypes.data,
                                                                    g.ctypes.data, h.ctypes.data)
            check()
            return v, g, h
        getattr(lib, f"eval_multi_UBspline_3d_{self.kind}")(self.ptr, x, y, z, v.ctypes.data)
        check()
        return v, None, None

    def eval_point_vg(self, x: float, y: float, z: float):
        """eval_multi_UBspline_3d_*_vg: (vals, grads) at one point."""
        dt = out_dtype(self.kind)
        ext = (2,) if self.ncomp == 2 else ()
        v = np.zeros((self.N,) + ext, dt)
        g = np.zeros((self.N, 3) + ext, dt)
        getattr(_lib(), f"eval_multi_UBspline_3d_{self.kind}_vg")(self.ptr, x, y, z, v.ctypes.data, g.ctypes.data)
        check()
        return v, g

    def eval_point_vgl(self, x: float, y: float, z: float):
        """eval_multi_UBspline_3d_*_vgl: (vals, grads, lapl) at one point."""
        dt = out_dtype(self.kind)
        ext = (2,) if self.ncomp == 2 else ()
        v = np.zeros((self.N,) + ext, dt)
        g = np.zeros((self.N, 3) + ext, dt)
        lap = np.zeros((self.N,) + ext, dt)
        getattr(_lib(), f"eval_multi_UBspline_3d_{self.kind}_vgl")(self.ptr, x, y, z, v.ctypes.data, g.ctypes.data,
                                                                   lap.ctypes.data)
        check()
        return v, g, lap

    def eval_point_vghgh(self, x: float, y: float, z: float):
        """eval_multi_UBspline_3d_*_vghgh: (vals, grads, hess[3][3],
        gradhess[3][3][3]) at one point."""
        dt = out_dtype(self.kind)
        ext = (2,) if self.ncomp == 2 else ()
        v = np.zeros((self.N,) + ext, dt)
        g = np.zeros((self.N, 3) + ext, dt)
        h = np.zeros((self.N, 3, 3) + ext, dt)
        gh = np.zeros((self.N, 3, 3, 3) + ext, dt)
        getattr(_lib(), f"eval_multi_UBspline_3d_{self.kind}_vghgh")(self.ptr, x, y, z, v.ctypes.data, g.ctypes.data,
                                                                     h.ctypes.data, gh.ctypes.data)
        check()
        return v, g, h, gh

    def out_shapes(self, P, layout):
        ext = (2,) if self.ncomp == 2 else ()
        if layout == 0:
            if self.ncomp == 2:
                return (P, self.N, 2), (P, self.N, 2, 3), (P, self.N, 2, 6)
            return (P, self.N), (P, self.N, 3), (P, self.N, 6)
        return (P, self.N) + ext, (P, self.N, 3) + ext, (P, self.N, 3, 3) + ext

    def opts(self, vgh=True, pos_f64=True, rule=0, layout=0, sort=False, strides=(0, 0, 0)) -> L.EvalOpts:
        return L.EvalOpts(int(vgh), int(pos_f64), rule, layout, int(sort), *strides)

    def eval(self, pos, vgh=True, rule=0, layout=0, sort=False, out=None, stream=None):
        """einspline_gb300_eval_3d on torch CUDA tensors.  pos: [P, 3]
        float32/float64.  Returns (vals, grads, hess) torch tensors."""
        torch = _torch()
        P = int(pos.shape[0])
        dt = torch.float32 if self.kind in "sc" else torch.float64
        if out is None:
            shp = self.out_shapes(P, layout)
            out = (torch.empty(shp[0], dtype=dt, device=pos.device),
                   torch.empty(shp[1], dtype=dt, device=pos.device) if vgh else None,
                   torch.empty(shp[2], dtype=dt, device=pos.device) if vgh else None)
        o = self.opts(vgh, pos.dtype == torch.float64, rule, layout, sort)
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)  # noqa: E731
        s = C.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        _lib().einspline_gb300_eval_3d(self.table, C.byref(o), P, ptr(pos), ptr(out[0]), ptr(out[1]),
                                       ptr(out[2]), s)
        check()
        return out

    def set_fp64_mode(self, mode: int) -> None:
        """FP64 tables: 0 IEEE FP64 evaluation, 1 double-float arithmetic."""
        _lib().einspline_gb300_set_fp64_mode(self.table, int(mode))
        check()

    def set_host_direct(self, mode: int) -> None:
        _lib().einspline_gb300_set_host_direct(self.table, int(mode))
        check()

    def eval_host(self, pos: np.ndarray, vgh=True, rule=0, layout=0, out=None):
        """einspline_gb300_eval_3d_host: host numpy buffers (pin them for speed)."""
        P = pos.shape[0]
        dt = out_dtype(self.kind)
        if out is None:
            shp = self.out_shapes(P, layout)
            out = (np.empty(shp[0], dt), np.empty(shp[1], dt) if vgh else None,
                   np.empty(shp[2], dt) if vgh else None)
        o = self.opts(vgh, pos.dtype == np.float64, rule, layout)
        ptr = lambda a: C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)  # noqa: E731
        _lib().einspline_gb300_eval_3d_host(self.table, C.byref(o), P, ptr(pos), ptr(out[0]), ptr(out[1]),
                                            ptr(out[2]))
        check()
        return out

    # -- device handle -----------------------------------------------------
    def to_cuda(self, storage=None) -> "CudaSpline":
        lib = _lib()
        if storage is None:
            c = getattr(lib, f"create_multi_UBspline_3d_{self.kind}_cuda")(self.ptr)
            kind = self.kind
        elif storage == "conv":
            assert self.kind in "dz"
            kind = "s" if self.kind == "d" else "c"
            c = getattr(lib, f"create_multi_UBspline_3d_{kind}_cuda_conv")(self.ptr)
        else:
            assert self.kind in "dz"
            kind = "s" if self.kind == "d" else "c"
            fn = "einspline_gb300_create_3d_s_cuda_from_d" if self.kind == "d" else \
                "einspline_gb300_create_3d_c_cuda_from_z"
            c = getattr(lib, fn)(self.ptr, storage)
        check()
        return CudaSpline(kind, c, self.N)

    def destroy(self) -> None:
        if getattr(self, "ptr", None):
            _lib().destroy_Bspline(C.cast(self.ptr, C.c_void_p))
            self.ptr = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class CudaSpline:
    """A device handle from create_multi_UBspline_3d_*_cuda[_conv]."""

    def __init__(self, kind, ptr, N):
        self.kind, self.ptr, self.N = kind, ptr, N
        self.ncomp = 2 if kind in "cz" else 1
        self.table = C.c_void_p(ptr.contents.gb300)

    @property
    def fields(self):
        return self.ptr.contents

    def set_fp64_mode(self, mode: int) -> None:
        """The handle's own table: 0 IEEE FP64, 1 double-float arithmetic."""
        _lib().einspline_gb300_set_fp64_mode(self.table, int(mode))
        check()

    def eval_multi(self, pos, vgh=True, outs=None):
        """eval_multi_multi_UBspline_3d_*[_vgh]_cuda with per-point output
        pointer arrays built over contiguous torch buffers (GPU layout)."""
        torch = _torch()
        P = int(pos.shape[0])
        dt = torch.float32 if self.kind in "sc" else torch.float64
        nr = self.N * self.ncomp
        if outs is None:
            v = torch.zeros((P, nr), dtype=dt, device=pos.device)
            g = torch.zeros((P, 3 * nr), dtype=dt, device=pos.device) if vgh else None
            h = torch.zeros((P, 6 * nr), dtype=dt, device=pos.device) if vgh else None
        else:
            v, g, h = outs
        es = v.element_size()

        def ptrs(t, per):
            base = t.data_ptr()
            return torch.tensor([base + i * per * es for i in range(P)], dtype=torch.int64, device=pos.device)

        vp = ptrs(v, v.shape[1])
        lib = _lib()
        if vgh:
            gp, hp = ptrs(g, g.shape[1]), ptrs(h, h.shape[1])
            getattr(lib, f"eval_multi_multi_UBspline_3d_{self.kind}_vgh_cuda")(
                self.ptr, C.c_void_p(pos.data_ptr()), C.c_void_p(vp.data_ptr()), C.c_void_p(gp.data_ptr()),
                C.c_void_p(hp.data_ptr()), P)
        else:
            getattr(lib, f"eval_multi_multi_UBspline_3d_{self.kind}_cuda")(
                self.ptr, C.c_void_p(pos.data_ptr()), C.c_void_p(vp.data_ptr()), P)
        check()
        return v, g, h

    def eval_multi_sign(self, pos, sign):
        """eval_multi_multi_UBspline_3d_s_sign_cuda: values times sign[i]."""
        torch = _torch()
        P = int(pos.shape[0])
        v = torch.zeros((P, self.N), dtype=torch.float32, device=pos.device)
        vp = torch.tensor([v.data_ptr() + i * self.N * 4 for i in range(P)], dtype=torch.int64, device=pos.device)
        _lib().eval_multi_multi_UBspline_3d_s_sign_cuda(self.ptr, C.c_void_p(pos.data_ptr()),
                                                        C.c_void_p(sign.data_ptr()), C.c_void_p(vp.data_ptr()), P)
        check()
        return v

    def eval_multi_vgl(self, pos, linv, row_stride=None, sign=None):
        """eval_multi_multi_UBspline_3d_*_vgl_cuda (or _s_vgl_sign_cuda): returns
        (vals [P][N*ncomp], grad_lapl [P][4][row_stride*ncomp])."""
        torch = _torch()
        P = int(pos.shape[0])
        dt = torch.float32 if self.kind in "sc" else torch.float64
        nr = self.N * self.ncomp
        rs = row_stride if row_stride is not None else self.N
        v = torch.zeros((P, nr), dtype=dt, device=pos.device)
        gl = torch.full((P, 4, rs * self.ncomp), -7.0, dtype=dt, device=pos.device)
        es = v.element_size()
        vp = torch.tensor([v.data_ptr() + i * nr * es for i in range(P)], dtype=torch.int64, device=pos.device)
        gp = torch.tensor([gl.data_ptr() + i * 4 * rs * self.ncomp * es for i in range(P)], dtype=torch.int64,
                          device=pos.device)
        lib = _lib()
        if sign is not None:
            lib.eval_multi_multi_UBspline_3d_s_vgl_sign_cuda(self.ptr, C.c_void_p(pos.data_ptr()),
                                                             C.c_void_p(sign.data_ptr()), C.c_void_p(linv.data_ptr()),
                                                             C.c_void_p(vp.data_ptr()), C.c_void_p(gp.data_ptr()), P, rs)
        else:
            getattr(lib, f"eval_multi_multi_UBspline_3d_{self.kind}_vgl_cuda")(
                self.ptr, C.c_void_p(pos.data_ptr()), C.c_void_p(linv.data_ptr()), C.c_void_p(vp.data_ptr()),
                C.c_void_p(gp.data_ptr()), P, rs)
        check()
        return v, gl

    def destroy(self):
        if getattr(self, "ptr", None):
            getattr(_lib(), f"destroy_multi_UBspline_3d_{self.kind}_cuda")(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Server:
    """einspline_gb300_server_*: continuous batching of walker requests."""

    def __init__(self, spline: MultiUBspline3D, vgh=True, pos_f64=True, rule=0, use_graphs=True,
                 max_inflight=3, max_batch_points=16384, hbm_budget_bytes=0, sort=False):
        self.spline = spline
        self.pos_f64 = pos_f64
        self.vgh = vgh
        o = L.ServerOpts(int(vgh), int(pos_f64), rule, int(use_graphs), max_inflight, max_batch_points,
                         hbm_budget_bytes, int(sort))
        self.h = _lib().einspline_gb300_server_create(spline.table, C.byref(o))
        check()
        if not self.h:
            raise EinsplineError("server create failed")

    def submit(self, pos: np.ndarray) -> int:
        pos = np.ascontiguousarray(pos, np.float64 if self.pos_f64 else np.float32)
        rid = _lib().einspline_gb300_server_submit(self.h, C.c_void_p(pos.ctypes.data), pos.shape[0])
        check()
        return int(rid)

    def wait(self, rid: int, timeout: float = 60.0) -> None:
        _lib().einspline_gb300_server_wait(self.h, rid, timeout)
        check()

    def latency(self, rid: int) -> float:
        lat = C.c_double()
        _lib().einspline_gb300_server_result(self.h, rid, None, None, None, C.byref(lat))
        check()
        return lat.value

    def result(self, rid: int, npts: int):
        dt = out_dtype(self.spline.kind)
        nr = self.spline.N * self.spline.ncomp
        v = np.empty((npts, nr), dt)
        g = np.empty((npts, 3 * nr), dt) if self.vgh else None
        h = np.empty((npts, 6 * nr), dt) if self.vgh else None
        p = lambda a: C.c_void_p(a.ctypes.data) if a is not None else C.c_void_p(0)  # noqa: E731
        _lib().einspline_gb300_server_copy_result(self.h, rid, p(v), p(g), p(h))
        check()
        return v, g, h

    def release(self, rid: int) -> None:
        _lib().einspline_gb300_server_release(self.h, rid)
        check()

    def stats(self) -> L.ServerStats:
        s = L.ServerStats()
        _lib().einspline_gb300_server_get_stats(self.h, C.byref(s))
        check()
        return s

    def replay(self, arrival_s: np.ndarray, npts: np.ndarray, pos_all: np.ndarray):
        """Open-loop native replay; returns (latencies [s], wall seconds)."""
        n = len(npts)
        arr = np.ascontiguousarray(arrival_s, np.float64)
        cnt = np.ascontiguousarray(npts, np.int32)
        off = np.ascontiguousarray(np.concatenate([[0], np.cumsum(cnt)[:-1]]), np.int64)
        pos = np.ascontiguousarray(pos_all, np.float64 if self.pos_f64 else np.float32)
        lat = np.zeros(n, np.float64)
        wall = C.c_double()
        _lib().einspline_gb300_server_replay(self.h, n, C.c_void_p(arr.ctypes.data), C.c_void_p(cnt.ctypes.data),
                                             C.c_void_p(off.ctypes.data), C.c_void_p(pos.ctypes.data),
                                             C.c_void_p(lat.ctypes.data), C.byref(wall))
        check()
        return lat, wall.value

    def close(self):
        if getattr(self, "h", None):
            _lib().einspline_gb300_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MultiUBsplineLD:
    """A uniform 1D or 2D multi-spline: create/set/eval_multi_UBspline_{1,2}d_*
    (src/multi_bspline_create.c:88-248, src/multi_bspline_eval_std_s_impl.h:38-480).
    grids and bcs hold one or two axes."""

    def __init__(self, kind: str, grids, bcs, num_splines: int):
        lib = _lib()
        self.kind, self.N, self.dims = kind, num_splines, len(grids)
        assert self.dims in (1, 2)
        self.ncomp = 2 if kind in "cz" else 1
        self.M = tuple(int(g[2]) for g in grids)
        ug = [L.Ugrid(float(g[0]), float(g[1]), int(g[2]), 0.0, 0.0) for g in grids]
        bc = [_bc(kind, b) for b in bcs]
        p = getattr(lib, f"create_multi_UBspline_{self.dims}d_{kind}")(*ug, *bc, num_splines)
        check()
        if not p:
            raise EinsplineError("create failed")
        self.ptr = p
        self.table = C.c_void_p(p.contents.gb300)

    def set(self, i: int, data) -> None:
        dt = np.float32 if self.kind in "sc" else np.float64
        d = np.asarray(data)
        if self.ncomp == 2 and np.iscomplexobj(d):
            d = np.stack([d.real, d.imag], axis=-1)
        d = np.ascontiguousarray(d, dtype=dt)
        getattr(_lib(), f"set_multi_UBspline_{self.dims}d_{self.kind}")(self.ptr, i, d.ctypes.data)
        check()

    def set_bc(self, i: int, data, bc) -> None:
        """set_multi_UBspline_1d_{d,z}_BC: spline i solved with its own x BC."""
        d = np.asarray(data)
        if self.ncomp == 2 and np.iscomplexobj(d):
            d = np.stack([d.real, d.imag], axis=-1)
        d = np.ascontiguousarray(d, dtype=np.float64)
        getattr(_lib(), f"set_multi_UBspline_1d_{self.kind}_BC")(self.ptr, i, d.ctypes.data, _bc(self.kind, bc))
        check()

    def flush(self) -> None:
        _lib().einspline_gb300_flush(self.table)
        check()

    def table_values(self) -> np.ndarray:
        """The stored table as float64 [Nx](, Ny) [N] (complex: trailing 2)."""
        ti = L.TableInfo()
        lib = _lib()
        lib.einspline_gb300_get_table_info(self.table, C.byref(ti))
        check()
        dt = np.float32 if ti.storage == STORE_F32 else np.float64
        out = np.empty((ti.nx, ti.ny, ti.nz, ti.ncol_pad), dtype=dt)
        lib.einspline_gb300_copy_table(self.table, out.ctypes.data, None)
        check()
        v = out[..., :ti.ncol].astype(np.float64).reshape((ti.nx, ti.ny)[:self.dims] + (ti.ncol,))
        return v.reshape(v.shape[:-1] + (self.N, 2)) if self.ncomp == 2 else v

    def eval_point(self, x: float, y: float = 0.0, form: int = 3):
        """eval_multi_UBspline_{1,2}d_*[_vg|_vgl|_vgh] (form 0..3): (vals,
        grads, lh) in the CPU layouts; lh is the second derivative (1D), the
        laplacian (2D vgl) or the Hessian [N][2][2] (2D vgh)."""
        dt = out_dtype(self.kind)
        ext = (2,) if self.ncomp == 2 else ()
        v = np.zeros((self.N,) + ext, dt)
        g = np.zeros((self.N,) + ((2,) if self.dims == 2 else ()) + ext, dt)
        lh = np.zeros((self.N,) + ((2, 2) if self.dims == 2 and form == 3 else ()) + ext, dt)
        suf = ("", "_vg", "_vgl", "_vgh")[form]
        f = getattr(_lib(), f"eval_multi_UBspline_{self.dims}d_{self.kind}{suf}")
        xy = (x,) if self.dims == 1 else (x, y)
        bufs = [v.ctypes.data, g.ctypes.data, lh.ctypes.data][:1 + min(form, 2)]
        f(self.ptr, *xy, *bufs)
        check()
        return v, (g if form >= 1 else None), (lh if form >= 2 else None)

    def to_cuda(self, conv: bool = False) -> "CudaSpline1D":
        """create_multi_UBspline_1d_*_cuda (conv: the d->s / z->c _conv forms)."""
        assert self.dims == 1
        lib = _lib()
        if conv:
            kind = {"d": "s", "z": "c"}[self.kind]
            p = getattr(lib, f"create_multi_UBspline_1d_{kind}_cuda_conv")(self.ptr)
        else:
            kind = self.kind
            p = getattr(lib, f"create_multi_UBspline_1d_{kind}_cuda")(self.ptr)
        check()
        return CudaSpline1D(kind, p, self.N)

    def destroy(self) -> None:
        if getattr(self, "ptr", None):
            _lib().destroy_Bspline(C.cast(self.ptr, C.c_void_p))
            self.ptr = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class CudaSpline1D:
    """A device handle from create_multi_UBspline_1d_*_cuda[_conv]."""

    def __init__(self, kind, ptr, N):
        self.kind, self.ptr, self.N = kind, ptr, N
        self.ncomp = 2 if kind in "cz" else 1

    @property
    def fields(self):
        return self.ptr.contents

    def eval_multi(self, pos, vgl=False):
        """eval_multi_multi_UBspline_1d_*[_vgl]_cuda: pos [P] (float for s/c,
        double for d/z) -> vals, grads, lapl [P, N * ncomp] (derivatives with
        respect to the cell coordinate, as the reference's kernels)."""
        torch = _torch()
        P = int(pos.shape[0])
        dt = torch.float32 if self.kind in "sc" else torch.float64
        nr = self.N * self.ncomp
        outs = [torch.zeros((P, nr), dtype=dt, device=pos.device) for _ in range(3 if vgl else 1)]
        ptrs = [torch.arange(P, dtype=torch.int64, device=pos.device) * (nr * o.element_size()) + o.data_ptr()
                for o in outs]
        lib = _lib()
        if vgl:
            getattr(lib, f"eval_multi_multi_UBspline_1d_{self.kind}_vgl_cuda")(
                self.ptr, C.c_void_p(pos.data_ptr()), *[C.c_void_p(q.data_ptr()) for q in ptrs], P)
        else:
            getattr(lib, f"eval_multi_multi_UBspline_1d_{self.kind}_cuda")(
                self.ptr, C.c_void_p(pos.data_ptr()), C.c_void_p(ptrs[0].data_ptr()), P)
        check()
        return tuple(outs) if vgl else (outs[0], None, None)

    def destroy(self):
        if getattr(self, "ptr", None):
            getattr(_lib(), f"destroy_multi_UBspline_1d_{self.kind}_cuda")(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass


class Determinants:
    """A population of walkers' Slater matrices A [W][ld][ld] and inverses
    (torch float32 CUDA tensors, one contiguous block each) for the fused
    determinant step: einspline_gb300_det_ratio / _det_update.  trans=0 keeps
    Ainv[j][e] (orbital j, electron e) as the reference does; trans=1 stores
    its transpose so column k is contiguous."""

    def __init__(self, A, ainv, nelec: int, trans: int = 0):
        torch = _torch()
        self.A, self.ainv = A, ainv
        self.W, self.ld = int(A.shape[0]), int(ainv.shape[-1])
        self.nelec, self.trans = int(nelec), int(trans)
        self._cache = {}
        self.a_ptrs = self._ptrs(A)
        self.ainv_ptrs = self._ptrs(ainv)
        self.work = torch.empty(2 * self.nelec * self.W, dtype=torch.float32, device=A.device)

    _CACHE_MAX = 64

    def _remember(self, key, value):
        if len(self._cache) >= self._CACHE_MAX:
            self._cache.pop(next(iter(self._cache)))  # oldest entry
        self._cache[key] = value
        return value

    def _ptrs(self, t):
        """Device array of per-walker pointers into t [W, ...] (cached)."""
        torch = _torch()
        key = ("p", t.data_ptr(), tuple(t.shape), tuple(t.stride()))
        if key not in self._cache:
            step = t.stride(0) * t.element_size()
            base = torch.arange(t.shape[0], dtype=torch.int64, device=t.device) * step
            return self._remember(key, base + t.data_ptr())
        return self._cache[key]

    def _index(self, accepted):
        torch = _torch()
        if isinstance(accepted, torch.Tensor):
            return accepted.to(device=self.A.device, dtype=torch.int64)
        key = ("i", tuple(int(i) for i in accepted))
        if key not in self._cache:
            return self._remember(key, torch.as_tensor(key[1], dtype=torch.int64, device=self.A.device))
        return self._cache[key]

    def opts(self, k, pos_f64=False, rule=1):
        return L.DetOpts(self.nelec, int(k), self.ld, self.trans, int(pos_f64), int(rule))

    def ratio(self, spline: "MultiUBspline3D", pos, k: int, grad_lapl=True, rows=None, rule=1, stream=None):
        """Ratios (and gradient / Laplacian ratios) of every walker moving
        electron k to pos [W, 3]; rows: optional [W, >= nelec] float32 tensor
        that receives the new orbital rows."""
        torch = _torch()
        W = int(pos.shape[0])
        dev = pos.device
        ratio = torch.empty(W, dtype=torch.float32, device=dev)
        grad = torch.empty(W, 3, dtype=torch.float32, device=dev) if grad_lapl else None
        lapl = torch.empty(W, dtype=torch.float32, device=dev) if grad_lapl else None
        row_ptrs = self._ptrs(rows) if rows is not None else None
        o = self.opts(k, pos.dtype == torch.float64, rule)
        ptr = lambda t: C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p(0)  # noqa: E731
        s = C.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        _lib().einspline_gb300_det_ratio(spline.table, C.byref(o), W, ptr(pos), ptr(self.ainv_ptrs), ptr(ratio),
                                         ptr(grad), ptr(lapl), ptr(row_ptrs), s)
        check()
        return ratio, grad, lapl

    def update(self, k: int, accepted, rows, stream=None):
        """Sherman-Morrison update of the accepted walkers (indices) whose
        row k becomes rows[i] (rows: [W, >= nelec] float32 CUDA tensor)."""
        torch = _torch()
        idx = self._index(accepted)
        n = int(idx.numel())
        if n == 0:
            return
        a = self.a_ptrs[idx].contiguous()
        ai = self.ainv_ptrs[idx].contiguous()
        r = self._ptrs(rows)[idx].contiguous()
        o = self.opts(k)
        s = C.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
        _lib().einspline_gb300_det_update(C.byref(o), n, C.c_void_p(a.data_ptr()), C.c_void_p(ai.data_ptr()),
                                          C.c_void_p(r.data_ptr()), C.c_void_p(self.work.data_ptr()), s)
        check()


def launch_count() -> int:
    return int(_lib().einspline_gb300_launch_count())


def fill_uniform(t, seed: int, lo: float = 0.0, hi: float = 1.0, offset: int = 0, stream=None):
    """Fill a torch CUDA float32/float64 tensor with the splitmix64 uniform stream."""
    torch = _torch()
    s = C.c_void_p(stream.cuda_stream if stream is not None else torch.cuda.current_stream().cuda_stream)
    _lib().einspline_gb300_fill_uniform(C.c_void_p(t.data_ptr()), t.numel(), int(t.dtype == torch.float64),
                                        seed & 0xFFFFFFFFFFFFFFFF, offset, lo, hi, s)
    check()
    return t
