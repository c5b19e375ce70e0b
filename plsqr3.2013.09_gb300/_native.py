"""ctypes binding of libplsqr_gpu.so (the C ABI of include/plsqr_gpu.h).

The library is built in-tree (lib/ next to this file).  Loading it needs no
GPU; every call that computes needs one and returns PLSQR_ERR_NODEV without.
There is no fallback: a missing library raises at load time.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

LIB_DIR = Path(__file__).resolve().parent / "lib"
# PLSQR_LIB: another build of the library (the bounds-checked one)
LIB_PATH = Path(os.environ["PLSQR_LIB"]) if os.environ.get("PLSQR_LIB") else LIB_DIR / "libplsqr_gpu.so"

PLSQR_OK = 0
ERR = {
    -1: "PLSQR_ERR_ARG", -2: "PLSQR_ERR_IO", -3: "PLSQR_ERR_FORMAT", -4: "PLSQR_ERR_NOMEM",
    -5: "PLSQR_ERR_CUDA", -6: "PLSQR_ERR_NODEV", -7: "PLSQR_ERR_STATE", -8: "PLSQR_ERR_TIMEOUT",
    -9: "PLSQR_ERR_INTERNAL", -10: "PLSQR_ERR_NUMERIC",
}
PREC_FP64, PREC_MIXED = 0, 1
ORDER_FAST, ORDER_REFERENCE = 0, 1
NOALLOC_MAX_ROWS = 1048576  # PLSQR_NOALLOC_MAX_ROWS

vp = C.c_void_p
i32, i64, f64, u64 = C.c_int32, C.c_int64, C.c_double, C.c_uint64


class Sparse(C.Structure):
    _fields_ = [("num_row", i32), ("num_col", i32), ("nnz", i64), ("ptr32", vp), ("ptr64", vp),
                ("idx", vp), ("val", vp)]


class Files(C.Structure):
    _fields_ = [("dir", C.c_char_p), ("ker_f", C.c_char_p), ("ker_i", C.c_char_p),
                ("damp_f", C.c_char_p), ("damp_i", C.c_char_p), ("damp_f_bycol", C.c_char_p),
                ("damp_i_bycol", C.c_char_p), ("b_k", C.c_char_p), ("row_k", i32),
                ("row_d", i32), ("col", i32), ("col_perm", C.c_char_p)]


class Opts(C.Structure):
    _fields_ = [("device", i32), ("precision", i32), ("use_graph", i32), ("verbose", i32),
                ("grid", i32 * 3), ("order", i32), ("lean", i32)]


class Info(C.Structure):
    _fields_ = [("m_k", i32), ("m_d", i32), ("n", i32), ("nnz_k", i64), ("nnz_d", i64),
                ("device_bytes", i64), ("sm_count", i32), ("hbm_bytes_aprod1", f64),
                ("hbm_bytes_aprod2", f64), ("hbm_bytes_iteration", f64)]


class LsqrArgs(C.Structure):
    _fields_ = [("damp", f64), ("atol", f64), ("btol", f64), ("conlim", f64), ("itnlim", i32),
                ("lsqr_iteration", i32), ("want_se", i32), ("stop_on_istop", i32),
                ("result_txt", C.c_char_p), ("sweeps", i32), ("inner", i32), ("x0", vp)]


class Result(C.Structure):
    _fields_ = [("istop", i32), ("itn", i32), ("anorm", f64), ("acond", f64), ("rnorm", f64),
                ("arnorm_out", f64), ("xnorm", f64), ("arnorm", f64), ("bnorm", f64),
                ("dxmax", f64), ("maxdx", i32), ("warm", i32), ("seconds", f64),
                ("seconds_total", f64)]


class SynthParams(C.Structure):
    _fields_ = [("nx", i32), ("ny", i32), ("nz", i32), ("n_rays", i32), ("tube_radius", f64),
                ("face_axis", i32), ("n_blobs", i32), ("value_scale", f64), ("blob_sigma", f64),
                ("checker_amp", f64), ("checker_period", i32), ("pad", i32), ("noise_frac", f64),
                ("damp_identity", f64), ("damp_lap", f64), ("damp_cross", f64),
                ("n_params", i32), ("pad2", i32), ("seed", u64)]


class BatchArgs(C.Structure):
    _fields_ = [("k", i32), ("sweeps", i32), ("inner", i32), ("variant_rows", i32),
                ("variant_cols", i32), ("retire_every", i32), ("damp", f64), ("atol", f64),
                ("btol", f64), ("conlim", f64), ("b_k", vp), ("lambda_", vp), ("x_ref", vp),
                ("x0", vp), ("retire_err", f64)]


class BatchInfo(C.Structure):
    _fields_ = [("k", i32), ("kp", i32), ("variant_rows", i32), ("variant_cols", i32),
                ("tuned", i32), ("warm", i32), ("ms_rows", f64), ("ms_cols", f64)]


class ProblemDesc(C.Structure):
    _fields_ = [("k_csc", Sparse), ("d_csr", Sparse), ("d_csc", Sparse), ("b_k", vp),
                ("lsqr_iteration", i32), ("itnlim", i32), ("damp", f64), ("atol", f64),
                ("btol", f64), ("conlim", f64)]


class MultiInfo(C.Structure):
    _fields_ = [("count", i32), ("blocks", i32), ("groups", i32), ("blocks_per_sm", i32),
                ("device_bytes", i64), ("wait_ns", i64), ("seconds", f64)]


ITER_DTYPE = np.dtype([(k, "<f8") for k in ("alpha", "beta", "rnorm", "arnorm", "test1", "test2",
                                             "anorm", "acond", "xnorm", "x0", "err")]
                      + [("istop", "<i4"), ("pad", "<i4")])

# name -> (restype, argtypes); every symbol include/plsqr_gpu.h declares
SIGNATURES = {
    "plsqr_strerror": (C.c_char_p, [C.c_int]),
    "plsqr_abi_version": (C.c_int, []),
    "plsqr_check_flags": (C.c_int, [C.POINTER(i32), C.POINTER(C.c_uint32), i32]),
    "plsqr_default_opts": (None, [C.POINTER(Opts)]),
    "plsqr_default_lsqr_args": (None, [C.POINTER(LsqrArgs)]),
    "plsqr_device_count": (C.c_int, [C.POINTER(i32)]),
    "plsqr_ctx_create": (C.c_int, [C.POINTER(Sparse), C.POINTER(Sparse), C.POINTER(Sparse),
                                   C.POINTER(Opts), C.POINTER(vp)]),
    "plsqr_ctx_create_files": (C.c_int, [C.POINTER(Files), C.POINTER(Opts), C.POINTER(vp)]),
    "plsqr_ctx_destroy": (None, [vp]),
    "plsqr_ctx_info": (C.c_int, [vp, C.POINTER(Info)]),
    "plsqr_ctx_last_error": (C.c_char_p, [vp]),
    "plsqr_set_u": (C.c_int, [vp, vp, vp]),
    "plsqr_get_u": (C.c_int, [vp, vp, vp]),
    "plsqr_set_v": (C.c_int, [vp, vp]),
    "plsqr_get_v": (C.c_int, [vp, vp]),
    "plsqr_get_b": (C.c_int, [vp, vp]),
    "plsqr_aprod": (C.c_int, [vp, C.c_int, C.c_int, C.c_int]),
    "plsqr_aprod_host": (C.c_int, [vp, C.c_int, vp, vp, vp, C.c_int, C.c_int]),
    "plsqr_lsqr": (C.c_int, [vp, C.POINTER(LsqrArgs), vp, vp, vp, vp, vp, C.POINTER(Result)]),
    "plsqr_set_reference_x": (C.c_int, [vp, vp]),
    "plsqr_get_x": (C.c_int, [vp, vp]),
    "plsqr_write_result": (C.c_int, [vp, C.c_char_p]),
    "plsqr_bench_aprod": (C.c_int, [vp, C.c_int, C.c_int, C.POINTER(f64)]),
    "plsqr_bench_iteration": (C.c_int, [vp, C.c_int, C.POINTER(f64)]),
    "plsqr_set_timing": (C.c_int, [vp, C.c_int]),
    "plsqr_write_timing": (C.c_int, [vp, C.c_char_p]),
    "plsqr_aprod1_nrm2_noalloc": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp]),
    "plsqr_default_batch_args": (None, [C.POINTER(BatchArgs)]),
    "plsqr_batch_variant": (C.c_int, [i32, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
    "plsqr_batch_lsqr": (C.c_int, [vp, C.POINTER(BatchArgs), vp, vp, vp, C.POINTER(BatchInfo)]),
    "plsqr_batch_bench_aprod": (C.c_int, [vp, i32, C.c_int, i32, C.c_int, C.POINTER(f64)]),
    "plsqr_set_damping_weight": (C.c_int, [vp, f64]),
    "plsqr_unet_create": (C.c_int, [i32, i32, i32, u64, i32, C.POINTER(vp)]),
    "plsqr_unet_destroy": (None, [vp]),
    "plsqr_unet_last_error": (C.c_char_p, [vp]),
    "plsqr_unet_predict": (C.c_int, [vp, vp, vp]),
    "plsqr_unet_train_step": (C.c_int, [vp, vp, vp, C.c_float, C.POINTER(C.c_float)]),
    "plsqr_unet_predict_device": (C.c_int, [vp, vp, vp, vp]),
    "plsqr_unet_train_step_device": (C.c_int, [vp, vp, vp, C.c_float, C.POINTER(C.c_float), vp]),
    "plsqr_unet_weights": (C.c_int, [vp, vp, C.POINTER(i64), i32]),
    "plsqr_nn_conv3d_check": (C.c_int, [i32, i32, i32, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp]),
    "plsqr_default_problem": (None, [C.POINTER(ProblemDesc)]),
    "plsqr_multi_create": (C.c_int, [C.POINTER(ProblemDesc), i32, C.POINTER(Opts), C.POINTER(vp)]),
    "plsqr_multi_destroy": (None, [vp]),
    "plsqr_multi_last_error": (C.c_char_p, [vp]),
    "plsqr_multi_info_get": (C.c_int, [vp, C.POINTER(MultiInfo)]),
    "plsqr_multi_plan": (C.c_int, [vp, vp, vp]),
    "plsqr_multi_plan_host": (C.c_int, [vp, vp, i32, i32, f64, vp, vp, C.POINTER(i32)]),
    "plsqr_multi_set_wait": (C.c_int, [vp, i64]),
    "plsqr_multi_set_exact": (C.c_int, [vp, i32]),
    "plsqr_multi_set_mixed": (C.c_int, [vp, i32]),
    "plsqr_multi_solve": (C.c_int, [vp, vp, vp, vp]),
    "plsqr_multi_check_wait": (C.c_int, [vp, i64]),
    "plsqr_io_read_kernel_info": (C.c_int, [C.c_char_p, i32, vp, vp, C.POINTER(i64)]),
    "plsqr_io_read_kernel": (C.c_int, [C.c_char_p, C.c_char_p, i32, i32, vp, vp, vp]),
    "plsqr_io_read_int32_counts": (C.c_int, [C.c_char_p, i64, vp, C.POINTER(i64)]),
    "plsqr_io_read_damping": (C.c_int, [C.c_char_p, C.c_int, i32, i32, i64, vp, vp, vp]),
    "plsqr_io_read_rhs": (C.c_int, [C.c_char_p, i32, vp]),
    "plsqr_io_read_col_perm": (C.c_int, [C.c_char_p, i32, vp]),
    "plsqr_permute_columns": (C.c_int, [i32, vp, vp, vp, vp, vp, vp, vp]),
    "plsqr_io_write_kernel": (C.c_int, [C.c_char_p, C.c_char_p, i32, i32, vp, vp, vp]),
    "plsqr_io_write_damping": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, i32,
                                         i32, vp, vp, vp, vp, vp, vp]),
    "plsqr_io_write_rhs": (C.c_int, [C.c_char_p, i32, vp]),
    "plsqr_io_write_x": (C.c_int, [C.c_char_p, i32, vp]),
    "plsqr_synth_default_params": (None, [C.POINTER(SynthParams)]),
    "plsqr_synth_kernel_counts": (C.c_int, [C.POINTER(SynthParams), vp]),
    "plsqr_synth_kernel_fill": (C.c_int, [C.POINTER(SynthParams), vp, vp, vp]),
    "plsqr_synth_damping_size": (C.c_int, [C.POINTER(SynthParams), C.POINTER(i64),
                                           C.POINTER(i64)]),
    "plsqr_synth_damping_fill": (C.c_int, [C.POINTER(SynthParams), vp, vp, vp]),
    "plsqr_synth_xtrue": (C.c_int, [C.POINTER(SynthParams), vp]),
    "plsqr_synth_rhs": (C.c_int, [C.POINTER(SynthParams), vp, vp, vp, vp, vp]),
    "plsqr_synth_noisy": (C.c_int, [C.POINTER(SynthParams), u64, i64, vp, vp]),
    "plsqr_transpose": (C.c_int, [i64, i64, vp, vp, vp, vp, vp, vp]),
}

_lib = None


class PlsqrError(RuntimeError):
    def __init__(self, code: int, where: str, detail: str = ""):
        self.code = code
        msg = f"{where}: {ERR.get(code, code)}"
        if detail:
            msg += f" ({detail})"
        super().__init__(msg)


def lib() -> C.CDLL:
    """The loaded library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(rc: int, where: str, ctx=None) -> None:
    if rc != PLSQR_OK:
        detail = ""
        if ctx:
            detail = (lib().plsqr_ctx_last_error(ctx) or b"").decode()
        raise PlsqrError(rc, where, detail)


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(vp)


def device_count() -> int:
    n = i32(0)
    check(lib().plsqr_device_count(C.byref(n)), "plsqr_device_count")
    return int(n.value)


def check_flags(reset: bool = False) -> tuple[bool, int]:
    """(bounds-checked build?, the checks that failed on the current device)."""
    checked, flags = i32(0), C.c_uint32(0)
    check(lib().plsqr_check_flags(C.byref(checked), C.byref(flags), int(reset)),
          "plsqr_check_flags")
    return bool(checked.value), int(flags.value)


def batch_variant(index: int) -> tuple[int, int, int]:
    """(gather width, lanes per line, nonzeros in flight) of a batched
    product variant; PlsqrError past the last one."""
    vw, lpr, u = i32(0), i32(0), i32(0)
    check(lib().plsqr_batch_variant(index, C.byref(vw), C.byref(lpr), C.byref(u)),
          "plsqr_batch_variant")
    return vw.value, lpr.value, u.value
