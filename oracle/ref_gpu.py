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
pointers to vals[N], grads[N][3], hess[N][6].

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
# the kernel's device symbol: its C++ name for the parameter list
# (float*, float3, float*, float**, float**, float**, uint3, uint3, int),
# with internal linkage (declared static) or without
VGH_NAMES = (b"_ZL41eval_multi_multi_UBspline_3d_s_vgh_kernelPf6float3S_PS_S1_S1_5uint3S2_i",
             b"_Z41eval_multi_multi_UBspline_3d_s_vgh_kernelPf6float3S_PS_S1_S1_5uint3S2_i")
BLOCK = 64  # SPLINE_BLOCK_SIZE of the reference's CUDA files


class Float3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class UInt3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


def basis_table() -> np.ndarray:
    """48 floats: for the cubic B-spline basis b0..b3 (b0 = (1-t)^3/6,
    b1 = (3t^3 - 6t^2 + 4)/6, b2 = (-3t^3 + 3t^2 + 3t + 1)/6, b3 = t^3/6),
    then their first and second derivatives, the coefficients of
    (t^3, t^2, t, 1)."""
    b = [np.poly1d([-1, 3, -3, 1]) / 6, np.poly1d([3, -6, 0, 4]) / 6, np.poly1d([-3, 3, 3, 1]) / 6,
         np.poly1d([1, 0, 0, 0]) / 6]
    rows = []
    for d in range(3):
        for p in b:
            q = p.deriv(d) if d else p
            c = np.zeros(4)
            c[4 - len(q.coeffs):] = q.coeffs
            rows.append(c)
    return np.asarray(rows, dtype=np.float32).reshape(48)


def _cuda():
    for name in ("libcuda.so.1", "libcuda.so"):
        try:
            return C.CDLL(name)
        except OSError:
            continue
    return None


class RefVgh:
    """The reference vgh kernel loaded in the current context (create after
    the context exists, e.g. after torch has touched the GPU)."""

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
        self.fn = C.c_void_p()
        for name in VGH_NAMES:
            if cu.cuModuleGetFunction(C.byref(self.fn), self.mod, name) == 0:
                self.name = name.decode()
                break
        else:
            raise RuntimeError("the vgh kernel is not in the reference's device module")
        dptr, nbytes = C.c_uint64(), C.c_size_t()
        self._check(cu.cuModuleGetGlobal_v2(C.byref(dptr), C.byref(nbytes), self.mod, b"Acuda"), "Acuda")
        tab = basis_table()
        if nbytes.value != tab.nbytes:
            raise RuntimeError("unexpected size of Acuda")
        self._check(cu.cuMemcpyHtoD_v2(dptr, tab.ctypes.data_as(C.c_void_p), C.c_size_t(tab.nbytes)), "Acuda copy")

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed (CUresult {rc})")

    def launch(self, pos_d: int, num: int, drinv, coefs_d: int, vals_pp: int, grads_pp: int, hess_pp: int,
               dim, strides, n: int, stream: int) -> None:
        """One launch over num points (device pointers as integers; pos_d
        float xyz; the pointer arrays hold num device pointers each)."""
        if not 0 < num <= 65535:
            raise ValueError("the reference kernel takes 1..65535 points per launch (gridDim.y)")
        a_pos, a_coefs = C.c_uint64(pos_d), C.c_uint64(coefs_d)
        a_v, a_g, a_h = C.c_uint64(vals_pp), C.c_uint64(grads_pp), C.c_uint64(hess_pp)
        a_dr = Float3(*[float(x) for x in drinv])
        a_dim, a_st = UInt3(*[int(x) for x in dim]), UInt3(*[int(x) for x in strides])
        a_n = C.c_int(n)
        args = (C.c_void_p * 9)(*[C.cast(C.pointer(x), C.c_void_p) for x in
                                  (a_pos, a_dr, a_coefs, a_v, a_g, a_h, a_dim, a_st, a_n)])
        gx = (n + BLOCK - 1) // BLOCK
        self._check(self.cu.cuLaunchKernel(self.fn, C.c_uint(gx), C.c_uint(num), C.c_uint(1), C.c_uint(BLOCK),
                                           C.c_uint(1), C.c_uint(1), C.c_uint(0), C.c_void_p(stream), args, None),
                    "cuLaunchKernel")
