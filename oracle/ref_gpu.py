"""The reference's own GPU evaluation kernel, for timing beside the library.

Test and benchmark infrastructure only (bench.py's reference arm loads it;
the library never does).  `make -C oracle ref` compiles the reference's
src/multi_bspline_create_cuda.cu, where it lies in the reference tree, into
a device-only sm_103a module (oracle/_ref/multi_bspline_cuda_ref.cubin).
Device code carries no host architecture, so the module runs wherever a
GB300 is, without the reference sources.  This file loads it into the
current CUDA context through the driver API and launches
eval_multi_multi_UBspline_3d_s_vgh_kernel
(src/multi_bspline_cuda_s_impl.h:342-470) exactly as the reference's
eval_multi_multi_UBspline_3d_s_vgh_cuda does (:542-557): 64-thread blocks, a
grid of (ceil(N/64), points), positions as float xyz, per-point device
pointers to vals[N], grads[N][3], hess[N][6]; likewise the d and c vgh
kernels (src/multi_bspline_cuda_d_impl.h:85, :254-266;
src/multi_bspline_cuda_c_impl.h:258, :442-455, over 2N re/im columns).

The kernel reads the cubic B-spline basis from the module's constant table
Acuda[48]; create_multi_UBspline_3d_s_cuda fills it
(src/multi_bspline_create_cuda.cu:428-441): rows of power-basis coefficients
(t^3, t^2, t, 1) of the four basis functions, then of their first and
second derivatives.  basis_table() builds the same rows by differentiating
the basis polynomials.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
CUBIN = os.path.join(HERE, "_ref", "multi_bspline_cuda_ref.cubin")
# The vgh kernels' device symbols: their C++ names for the parameter lists
# (T*, T3, T*, T**, T**, T**, uint3, uint3, int) with T = float (s, c) or
# double (d), with internal linkage (declared static) or without.
_SIG = {"s": "Pf6float3S_PS_S1_S1_5uint3S2_i", "c": "Pf6float3S_PS_S1_S1_5uint3S2_i",
        "d": "Pd7double3S_PS_S1_S1_5uint3S2_i"}
VGH_NAMES = {k: tuple(f"{p}41eval_multi_multi_UBspline_3d_{k}_vgh_kernel{sig}".encode() for p in ("_ZL", "_Z"))
             for k, sig in _SIG.items()}
# The s vgl kernel (src/multi_bspline_cuda_s_impl.h:566-734): (float *pos,
# float3 drInv, float *coefs, float Linv[], float *vals[], float *grad_lapl[],
# uint3 dim, uint3 strides, int N, int row_stride).
VGL_NAMES = tuple(f"{p}41eval_multi_multi_UBspline_3d_s_vgl_kernelPf6float3S_S_PS_S1_5uint3S2_ii".encode()
                  for p in ("_ZL", "_Z"))
BLOCK = 64  # SPLINE_BLOCK_SIZE of the reference's CUDA files


class Float3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class Double3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


class UInt3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


def basis_table(dtype=np.float32) -> np.ndarray:
    """48 values: for the cubic B-spline basis b0..b3 (b0 = (1-t)^3/6,
    b1 = (3t^3 - 6t^2 + 4)/6, b2 = (-3t^3 + 3t^2 + 3t + 1)/6, b3 = t^3/6),
    then their first and second derivatives, the coefficients of
    (t^3, t^2, t, 1); float for Acuda, double for the FP64 kernels' Bcuda
    (src/multi_bspline_create_cuda.cu:6-7)."""
    b = [np.poly1d([-1, 3, -3, 1]) / 6, np.poly1d([3, -6, 0, 4]) / 6, np.poly1d([-3, 3, 3, 1]) / 6,
         np.poly1d([1, 0, 0, 0]) / 6]
    rows = []
    for d in range(3):
        for p in b:
            q = p.deriv(d) if d else p
            c = np.zeros(4)
            c[4 - len(q.coeffs):] = q.coeffs
            rows.append(c)
    return np.asarray(rows, dtype=np.float64).astype(dtype).reshape(48)


def _cuda():
    for name in ("libcuda.so.1", "libcuda.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    return None


class RefVgh:
    """The reference's vgh kernels (s, c, d) loaded in the current context
    (create after the context exists, e.g. after torch has touched the GPU)."""

    def __init__(self):
        if not os.path.exists(CUBIN):
            raise RuntimeError("the reference's device module was not built (make -C oracle ref)")
        cu = _cuda()
        if cu is None:
            raise RuntimeError("libcuda not found")
        self.cu = cu
        self._check(cu.cuInit(0), "cuInit")
        ctx = C.c_void_p()
        self._check(cu.cuCtxGetCurrent(C.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        self.mod = C.c_void_p()
        self._check(cu.cuModuleLoad(C.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        self.fn = {}
        for kind, names in VGH_NAMES.items():
            fn = C.c_void_p()
            for name in names:
                if cu.cuModuleGetFunction(C.byref(fn), self.mod, name) == 0:
                    self.fn[kind] = fn
                    break
            else:
                raise RuntimeError(f"the {kind} vgh kernel is not in the reference's device module")
        self.vgl = None
        for name in VGL_NAMES:
            fn = C.c_void_p()
            if cu.cuModuleGetFunction(C.byref(fn), self.mod, name) == 0:
                self.vgl = fn
                break
        for sym, dt in ((b"Acuda", np.float32), (b"Bcuda", np.float64)):
            dptr, nbytes = C.c_uint64(), C.c_size_t()
            self._check(cu.cuModuleGetGlobal_v2(C.byref(dptr), C.byref(nbytes), self.mod, sym), sym.decode())
            tab = basis_table(dt)
            if nbytes.value != tab.nbytes:
                raise RuntimeError(f"unexpected size of {sym.decode()}")
            self._check(cu.cuMemcpyHtoD_v2(dptr, tab.ctypes.data_as(C.c_void_p), C.c_size_t(tab.nbytes)),
                        sym.decode() + " copy")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed (CUresult {rc})")

    def launch(self, pos_d: int, num: int, drinv, coefs_d: int, vals_pp: int, grads_pp: int, hess_pp: int,
               dim, strides, n: int, stream: int, kind: str = "s") -> None:
        """One launch of kind's vgh kernel over num points (device pointers
        as integers; positions xyz in the kind's real type; the pointer
        arrays hold num device pointers each; strides in reals, doubled for
        complex tables as the reference's create does)."""
        if not 0 < num <= 65535:
            raise ValueError("the reference kernel takes 1..65535 points per launch (gridDim.y)")
        a_pos, a_coefs = C.c_uint64(pos_d), C.c_uint64(coefs_d)
        a_v, a_g, a_h = C.c_uint64(vals_pp), C.c_uint64(grads_pp), C.c_uint64(hess_pp)
        a_dr = (Double3 if kind == "d" else Float3)(*[float(x) for x in drinv])
        a_dim, a_st = UInt3(*[int(x) for x in dim]), UInt3(*[int(x) for x in strides])
        a_n = C.c_int(n)
        args = (C.c_void_p * 9)(*[C.cast(C.pointer(x), C.c_void_p) for x in
                                  (a_pos, a_dr, a_coefs, a_v, a_g, a_h, a_dim, a_st, a_n)])
        cols = 2 * n if kind == "c" else n  # the complex kernel runs over re/im columns
        gx = (cols + BLOCK - 1) // BLOCK
        self._check(self.cu.cuLaunchKernel(self.fn[kind], C.c_uint(gx), C.c_uint(num), C.c_uint(1), C.c_uint(BLOCK),
                                           C.c_uint(1), C.c_uint(1), C.c_uint(0), C.c_void_p(stream), args, None),
                    "cuLaunchKernel")

    def launch_vgl(self, pos_d: int, num: int, drinv, coefs_d: int, linv_d: int, vals_pp: int, gl_pp: int, dim,
                   strides, n: int, row_stride: int, stream: int) -> None:
        """One launch of the s vgl kernel as eval_multi_multi_UBspline_3d_s_vgl_cuda
        does (src/multi_bspline_cuda_s_impl.h:736-756): grid (ceil(N/64), num),
        64 threads; grad_lapl[i] holds 4 rows of row_stride floats."""
        if self.vgl is None:
            raise RuntimeError("the s vgl kernel is not in the reference's device module")
        if not 0 < num <= 65535:
            raise ValueError("the reference kernel takes 1..65535 points per launch (gridDim.y)")
        a_pos, a_coefs, a_linv = C.c_uint64(pos_d), C.c_uint64(coefs_d), C.c_uint64(linv_d)
        a_v, a_g = C.c_uint64(vals_pp), C.c_uint64(gl_pp)
        a_dr = Float3(*[float(x) for x in drinv])
        a_dim, a_st = UInt3(*[int(x) for x in dim]), UInt3(*[int(x) for x in strides])
        a_n, a_rs = C.c_int(n), C.c_int(row_stride)
        args = (C.c_void_p * 10)(*[C.cast(C.pointer(x), C.c_void_p) for x in
                                   (a_pos, a_dr, a_coefs, a_linv, a_v, a_g, a_dim, a_st, a_n, a_rs)])
        gx = (n + BLOCK - 1) // BLOCK
        self._check(self.cu.cuLaunchKernel(self.vgl, C.c_uint(gx), C.c_uint(num), C.c_uint(1), C.c_uint(BLOCK),
                                           C.c_uint(1), C.c_uint(1), C.c_uint(0), C.c_void_p(stream), args, None),
                    "cuLaunchKernel")
