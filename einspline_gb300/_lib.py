"""ctypes binding of the C-ABI library libeinspline_gb300.so.

Structures mirror include/*.h field for field.  Loading fails loudly when the
library has not been built: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

PERIODIC, DERIV1, DERIV2, FLAT, NATURAL, ANTIPERIODIC = range(6)
SINGLE_REAL, DOUBLE_REAL, SINGLE_COMPLEX, DOUBLE_COMPLEX = range(4)
STORE_NATIVE, STORE_F32, STORE_F16, STORE_BF16, STORE_F64, STORE_I16 = range(6)
STORAGE_NAMES = {STORE_NATIVE: "native", STORE_F32: "f32", STORE_F16: "f16", STORE_BF16: "bf16", STORE_F64: "f64",
                 STORE_I16: "i16"}
I16_BIAS = 32768


class Ugrid(C.Structure):
    _fields_ = [("start", C.c_double), ("end", C.c_double), ("num", C.c_int),
                ("delta", C.c_double), ("delta_inv", C.c_double)]


class BCtype_s(C.Structure):
    _fields_ = [("lCode", C.c_int), ("rCode", C.c_int), ("lVal", C.c_float), ("rVal", C.c_float)]


class BCtype_d(C.Structure):
    _fields_ = [("lCode", C.c_int), ("rCode", C.c_int), ("lVal", C.c_double), ("rVal", C.c_double)]


class BCtype_c(C.Structure):
    _fields_ = [("lCode", C.c_int), ("rCode", C.c_int), ("lVal_r", C.c_float), ("lVal_i", C.c_float),
                ("rVal_r", C.c_float), ("rVal_i", C.c_float)]


class BCtype_z(C.Structure):
    _fields_ = [("lCode", C.c_int), ("rCode", C.c_int), ("lVal_r", C.c_double), ("lVal_i", C.c_double),
                ("rVal_r", C.c_double), ("rVal_i", C.c_double)]


BC_TYPES = {"s": BCtype_s, "d": BCtype_d, "c": BCtype_c, "z": BCtype_z}


def _host_struct(kind):
    fields = [("spcode", C.c_int), ("tcode", C.c_int), ("coefs", C.c_void_p),
              ("x_stride", C.c_ssize_t), ("y_stride", C.c_ssize_t), ("z_stride", C.c_ssize_t),
              ("x_grid", Ugrid), ("y_grid", Ugrid), ("z_grid", Ugrid),
              ("xBC", BC_TYPES[kind]), ("yBC", BC_TYPES[kind]), ("zBC", BC_TYPES[kind]),
              ("num_splines", C.c_int)]
    if kind in "cz":
        fields.append(("lapl3", C.c_void_p))
    fields.append(("gb300", C.c_void_p))
    return type(f"multi_UBspline_3d_{kind}", (C.Structure,), {"_fields_": fields})


HOST_STRUCTS = {k: _host_struct(k) for k in "sdcz"}


def _host_struct_ld(kind, dims):
    ax = "xy"[:dims]
    fields = [("spcode", C.c_int), ("tcode", C.c_int), ("coefs", C.c_void_p)]
    fields += [(f"{a}_stride", C.c_ssize_t) for a in ax] + [(f"{a}_grid", Ugrid) for a in ax]
    fields += [(f"{a}BC", BC_TYPES[kind]) for a in ax] + [("num_splines", C.c_int)]
    if dims == 2 and kind in "cz":
        fields.append(("lapl2", C.c_void_p))
    fields.append(("gb300", C.c_void_p))
    return type(f"multi_UBspline_{dims}d_{kind}", (C.Structure,), {"_fields_": fields})


HOST_STRUCTS_LD = {(k, d): _host_struct_ld(k, d) for k in "sdcz" for d in (1, 2)}


class uint3(C.Structure):
    _fields_ = [("x", C.c_uint), ("y", C.c_uint), ("z", C.c_uint)]


class float3(C.Structure):
    _fields_ = [("x", C.c_float), ("y", C.c_float), ("z", C.c_float)]


class double3(C.Structure):
    _fields_ = [("x", C.c_double), ("y", C.c_double), ("z", C.c_double)]


def _cuda_struct(kind):
    g = float3 if kind in "sc" else double3
    fields = [("coefs", C.c_void_p), ("stride", uint3), ("gridInv", g), ("dim", uint3),
              ("num_splines", C.c_int), ("gb300", C.c_void_p)]
    return type(f"multi_UBspline_3d_{kind}_cuda", (C.Structure,), {"_fields_": fields})


CUDA_STRUCTS = {k: _cuda_struct(k) for k in "sdcz"}


def _cuda_struct_1d(kind):
    g = C.c_float if kind in "sc" else C.c_double
    fields = [("coefs", C.c_void_p), ("stride", C.c_uint), ("gridInv", g), ("num_splines", C.c_int),
              ("dim", C.c_int), ("gb300", C.c_void_p)]
    return type(f"multi_UBspline_1d_{kind}_cuda", (C.Structure,), {"_fields_": fields})


CUDA_STRUCTS_1D = {k: _cuda_struct_1d(k) for k in "sdcz"}


class EvalOpts(C.Structure):
    _fields_ = [("vgh", C.c_int), ("pos_f64", C.c_int), ("rule", C.c_int), ("layout", C.c_int),
                ("sort", C.c_int), ("vstride", C.c_int64), ("gstride", C.c_int64), ("hstride", C.c_int64)]


class DetOpts(C.Structure):
    _fields_ = [("nelec", C.c_int), ("k", C.c_int), ("ld", C.c_int), ("ainv_trans", C.c_int),
                ("pos_f64", C.c_int), ("rule", C.c_int)]


class TableInfo(C.Structure):
    _fields_ = [("kind", C.c_int), ("storage", C.c_int), ("num_splines", C.c_int), ("ncol", C.c_int),
                ("ncol_pad", C.c_int), ("elem_bytes", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
                ("nz", C.c_int), ("x_stride", C.c_int64), ("y_stride", C.c_int64), ("z_stride", C.c_int64),
                ("table_bytes", C.c_uint64), ("coefs", C.c_void_p), ("scale", C.c_void_p)]


class ServerOpts(C.Structure):
    _fields_ = [("vgh", C.c_int), ("pos_f64", C.c_int), ("rule", C.c_int), ("use_graphs", C.c_int),
                ("max_inflight", C.c_int), ("max_batch_points", C.c_int), ("hbm_budget_bytes", C.c_uint64),
                ("sort", C.c_int)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("released", C.c_int64),
                ("batches", C.c_int64), ("evals", C.c_int64), ("budget_bytes", C.c_uint64),
                ("peak_bytes_in_use", C.c_uint64), ("peak_inflight", C.c_int), ("busy_seconds", C.c_double)]


# Every symbol the headers in include/ declare, with its ctypes signature.
def _signatures():
    vp, i32, i64, dbl = C.c_void_p, C.c_int, C.c_int64, C.c_double
    sig = {}
    for k in "sdcz":
        H = C.POINTER(HOST_STRUCTS[k])
        D = C.POINTER(CUDA_STRUCTS[k])
        BC = BC_TYPES[k]
        sig[f"create_multi_UBspline_3d_{k}"] = ([Ugrid, Ugrid, Ugrid, BC, BC, BC, i32], H)
        sig[f"set_multi_UBspline_3d_{k}"] = ([H, i32, vp], None)
        sig[f"eval_multi_UBspline_3d_{k}"] = ([H, dbl, dbl, dbl, vp], None)
        sig[f"eval_multi_UBspline_3d_{k}_vgh"] = ([H, dbl, dbl, dbl, vp, vp, vp], None)
        sig[f"eval_multi_UBspline_3d_{k}_vg"] = ([H, dbl, dbl, dbl, vp, vp], None)
        sig[f"eval_multi_UBspline_3d_{k}_vgl"] = ([H, dbl, dbl, dbl, vp, vp, vp], None)
        sig[f"eval_multi_UBspline_3d_{k}_vghgh"] = ([H, dbl, dbl, dbl, vp, vp, vp, vp], None)
        sig[f"eval_multi_multi_UBspline_3d_{k}_vgl_cuda"] = ([D, vp, vp, vp, vp, i32, i32], None)
        sig[f"create_multi_UBspline_3d_{k}_cuda"] = ([H], D)
        sig[f"destroy_multi_UBspline_3d_{k}_cuda"] = ([D], None)
        sig[f"eval_multi_multi_UBspline_3d_{k}_cuda"] = ([D, vp, vp, i32], None)
        sig[f"eval_multi_multi_UBspline_3d_{k}_vgh_cuda"] = ([D, vp, vp, vp, vp, i32], None)
    for k in "sdcz":
        BC = BC_TYPES[k]
        H1 = C.POINTER(HOST_STRUCTS_LD[(k, 1)])
        H2 = C.POINTER(HOST_STRUCTS_LD[(k, 2)])
        D1 = C.POINTER(CUDA_STRUCTS_1D[k])
        sig[f"create_multi_UBspline_1d_{k}"] = ([Ugrid, BC, i32], H1)
        sig[f"create_multi_UBspline_2d_{k}"] = ([Ugrid, Ugrid, BC, BC, i32], H2)
        sig[f"set_multi_UBspline_1d_{k}"] = ([H1, i32, vp], None)
        sig[f"set_multi_UBspline_2d_{k}"] = ([H2, i32, vp], None)
        for nout, suf in ((1, ""), (2, "_vg"), (3, "_vgl"), (3, "_vgh")):
            sig[f"eval_multi_UBspline_1d_{k}{suf}"] = ([H1, dbl] + [vp] * nout, None)
            sig[f"eval_multi_UBspline_2d_{k}{suf}"] = ([H2, dbl, dbl] + [vp] * nout, None)
        sig[f"create_multi_UBspline_1d_{k}_cuda"] = ([H1], D1)
        sig[f"destroy_multi_UBspline_1d_{k}_cuda"] = ([D1], None)
        sig[f"eval_multi_multi_UBspline_1d_{k}_cuda"] = ([D1, vp, vp, i32], None)
        sig[f"eval_multi_multi_UBspline_1d_{k}_vgl_cuda"] = ([D1, vp, vp, vp, vp, i32], None)
    sig["create_multi_UBspline_1d_s_cuda_conv"] = ([C.POINTER(HOST_STRUCTS_LD[("d", 1)])],
                                                   C.POINTER(CUDA_STRUCTS_1D["s"]))
    sig["create_multi_UBspline_1d_c_cuda_conv"] = ([C.POINTER(HOST_STRUCTS_LD[("z", 1)])],
                                                   C.POINTER(CUDA_STRUCTS_1D["c"]))
    sig["set_multi_UBspline_1d_d_BC"] = ([C.POINTER(HOST_STRUCTS_LD[("d", 1)]), i32, vp, BCtype_d], None)
    sig["set_multi_UBspline_1d_z_BC"] = ([C.POINTER(HOST_STRUCTS_LD[("z", 1)]), i32, vp, BCtype_z], None)
    sig["create_multi_UBspline_3d_s_cuda_conv"] = ([C.POINTER(HOST_STRUCTS["d"])], C.POINTER(CUDA_STRUCTS["s"]))
    sig["create_multi_UBspline_3d_c_cuda_conv"] = ([C.POINTER(HOST_STRUCTS["z"])], C.POINTER(CUDA_STRUCTS["c"]))
    sig["eval_multi_multi_UBspline_3d_s_sign_cuda"] = ([C.POINTER(CUDA_STRUCTS["s"]), vp, vp, vp, i32], None)
    sig["eval_multi_multi_UBspline_3d_s_vgl_sign_cuda"] = ([C.POINTER(CUDA_STRUCTS["s"]), vp, vp, vp, vp, vp, i32,
                                                            i32], None)
    sig["destroy_Bspline"] = ([vp], None)
    sig["destroy_multi_UBspline"] = ([vp], None)
    sig["einspline_gb300_create_3d_s"] = ([Ugrid, Ugrid, Ugrid, BCtype_s, BCtype_s, BCtype_s, i32, i32],
                                          C.POINTER(HOST_STRUCTS["s"]))
    sig["einspline_gb300_create_3d_c"] = ([Ugrid, Ugrid, Ugrid, BCtype_c, BCtype_c, BCtype_c, i32, i32],
                                          C.POINTER(HOST_STRUCTS["c"]))
    sig["einspline_gb300_create_3d_s_cuda_from_d"] = ([C.POINTER(HOST_STRUCTS["d"]), i32],
                                                      C.POINTER(CUDA_STRUCTS["s"]))
    sig["einspline_gb300_create_3d_c_cuda_from_z"] = ([C.POINTER(HOST_STRUCTS["z"]), i32],
                                                      C.POINTER(CUDA_STRUCTS["c"]))
    sig["einspline_gb300_last_error"] = ([], i32)
    sig["einspline_gb300_last_error_message"] = ([], C.c_char_p)
    sig["einspline_gb300_clear_error"] = ([], None)
    sig["einspline_gb300_set_abort_on_error"] = ([i32], None)
    sig["einspline_gb300_set_3d_device"] = ([vp, i32, i32, vp], i32)
    sig["einspline_gb300_flush"] = ([vp], i32)
    sig["einspline_gb300_get_table_info"] = ([vp, C.POINTER(TableInfo)], i32)
    sig["einspline_gb300_copy_table"] = ([vp, vp, vp], i32)
    sig["einspline_gb300_host_coefs"] = ([vp, C.POINTER(vp)], i32)
    sig["einspline_gb300_push_host_coefs"] = ([vp], i32)
    sig["einspline_gb300_release_host_coefs"] = ([vp], i32)
    sig["einspline_gb300_eval_3d"] = ([vp, C.POINTER(EvalOpts), i64, vp, vp, vp, vp, vp], i32)
    sig["einspline_gb300_eval_3d_host"] = ([vp, C.POINTER(EvalOpts), i64, vp, vp, vp, vp], i32)
    sig["einspline_gb300_eval_3d_sorted_noalloc"] = ([vp, C.POINTER(EvalOpts), i64, vp, vp, vp, vp, vp], i32)
    sig["einspline_gb300_set_host_direct"] = ([vp, i32], i32)
    sig["einspline_gb300_set_fp64_mode"] = ([vp, i32], i32)
    sig["einspline_gb300_get_fp64_mode"] = ([vp], i32)
    sig["einspline_gb300_set_tile"] = ([vp, i32, i32, i32], i32)
    sig["einspline_gb300_get_tile"] = ([vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)], i32)
    sig["einspline_gb300_autotune"] = ([vp, i64, i32], i32)
    sig["einspline_gb300_autotune_sorted"] = ([vp, i64, i32], i32)
    sig["einspline_gb300_get_launch_shape"] = ([vp, i32, i32] + [C.POINTER(i32)] * 4, i32)
    sig["einspline_gb300_set_load_mode"] = ([vp, i32], i32)
    sig["einspline_gb300_get_load_mode"] = ([vp], i32)
    sig["einspline_gb300_wait_status"] = ([vp], i32)
    sig["einspline_gb300_test_wait_timeout"] = ([vp, i32, dbl], i32)
    sig["einspline_gb300_launch_count"] = ([], i64)
    sig["einspline_gb300_fill_uniform"] = ([vp, i64, i32, C.c_uint64, i64, dbl, dbl, vp], i32)
    sig["einspline_gb300_det_ratio"] = ([vp, C.POINTER(DetOpts), i32, vp, vp, vp, vp, vp, vp, vp], i32)
    sig["einspline_gb300_det_update"] = ([C.POINTER(DetOpts), i32, vp, vp, vp, vp, vp], i32)
    sig["einspline_gb300_server_create"] = ([vp, C.POINTER(ServerOpts)], vp)
    sig["einspline_gb300_server_destroy"] = ([vp], i32)
    sig["einspline_gb300_server_submit"] = ([vp, vp, i32], i64)
    sig["einspline_gb300_server_wait"] = ([vp, i64, dbl], i32)
    sig["einspline_gb300_server_result"] = ([vp, i64, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp),
                                             C.POINTER(dbl)], i32)
    sig["einspline_gb300_server_copy_result"] = ([vp, i64, vp, vp, vp], i32)
    sig["einspline_gb300_server_release"] = ([vp, i64], i32)
    sig["einspline_gb300_server_get_stats"] = ([vp, C.POINTER(ServerStats)], i32)
    sig["einspline_gb300_server_replay"] = ([vp, i32, vp, vp, vp, vp, vp, C.POINTER(dbl)], i32)
    return sig


SIGNATURES = _signatures()
# Library-internal helpers exported for tests (not part of include/).
EXTRA_SIGNATURES = {
    "einspline_gb300_solve_line_host": ([C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                         C.c_void_p, C.c_void_p], C.c_int),
}

_lib = None


def lib_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = False) -> C.CDLL:
    """Load the library (once).  Raises if it is missing: the product has no
    CPU fallback."""
    global _lib
    if _lib is None:
        path = lib_path()
        if not os.path.exists(path):
            if build_if_missing:
                _build.build()
            else:
                raise RuntimeError(f"einspline_gb300: {path} is missing; build it with "
                                   "`python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(path)
        for name, (args, res) in {**SIGNATURES, **EXTRA_SIGNATURES}.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        L.einspline_gb300_set_abort_on_error(0)
        _lib = L
    return _lib


class EinsplineError(RuntimeError):
    pass


def check(ret=None):
    """Raise EinsplineError if the last call left an error status."""
    L = load()
    code = L.einspline_gb300_last_error()
    if code:
        msg = L.einspline_gb300_last_error_message().decode()
        L.einspline_gb300_clear_error()
        raise EinsplineError(f"[{code}] {msg}")
    return ret
