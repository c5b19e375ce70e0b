"""ORACLE — test infrastructure, not product code.

ctypes binding of lib/liboracle_plsqr.so, the C restatement of the reference
PLSQR3 CPU path (plsqr_oracle.c).  Only tests/, __graft_entry__.smoke() and
bench.py's CPU baseline use it, and only as the reference that results are
compared with or as the timed CPU baseline.  The library is built by `make -C oracle` (see build()).
"""
from __future__ import annotations

import ctypes as C
import os
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "lib" / "liboracle_plsqr.so"
REF_BIN = HERE / "_ref" / "PLSQR3"
# the reference's source directory, for the recipes that compile the
# reference program itself (make ref / ref_gpu_aprod); overridable like the
# Makefile's REF_SRC
REF_SRC = Path(os.environ.get("PLSQR_REF_SRC", "/root/reference/source"))

vp = C.c_void_p


class Sparse(C.Structure):
    _fields_ = [("num_row", C.c_int), ("num_col", C.c_int), ("nnz", C.c_int64),
                ("ptr", vp), ("idx", vp), ("val", vp)]


class Problem(C.Structure):
    _fields_ = [("k_csc", Sparse), ("d_csr", Sparse), ("d_csc", Sparse),
                ("y_k", vp), ("y_d", vp), ("x", vp)]


ITER_DTYPE = np.dtype([(k, "<f8") for k in ("alpha", "beta", "rnorm", "arnorm", "test1",
                                             "test2", "anorm", "acond", "xnorm", "x0")]
                      + [("istop", "<i4"), ("pad", "<i4")])


class Result(C.Structure):
    _fields_ = [("istop", C.c_int), ("itn", C.c_int), ("anorm", C.c_double),
                ("acond", C.c_double), ("rnorm", C.c_double), ("arnorm_out", C.c_double),
                ("xnorm", C.c_double), ("arnorm", C.c_double), ("bnorm", C.c_double),
                ("dxmax", C.c_double), ("maxdx", C.c_int), ("loop_seconds", C.c_double)]


_lib = None

# int (*)(int mode, int m, int n, oracle_problem *p, void *usr, int is_final, int iteration)
APROD_FN = C.CFUNCTYPE(C.c_int, C.c_int, C.c_int, C.c_int, C.POINTER(Problem), vp, C.c_int,
                       C.c_int)


def build(with_reference: bool = False) -> None:
    """make -C oracle (and `make ref` when the reference tree is mounted)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if with_reference and reference_available():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", "-j8", f"REF_SRC={REF_SRC}"],
                       check=True)


def reference_available() -> bool:
    """The reference sources are present and a C compiler can build them."""
    return (REF_SRC / "lsqr.c").exists() and shutil.which("gcc") is not None


REF_GPU_APROD_BIN = HERE / "_ref" / "PLSQR3_gpu_aprod"


def build_gpu_aprod():
    """The reference program linked with the GPU operator shim (make
    ref_gpu_aprod), where the reference tree is mounted; its path, or None."""
    if not reference_available():
        return None
    subprocess.run(["make", "-s", "-C", str(HERE), "ref_gpu_aprod", "-j8", f"REF_SRC={REF_SRC}"],
                   check=True)
    return REF_GPU_APROD_BIN


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        L = C.CDLL(str(LIB_PATH))
        sp = C.POINTER(Sparse)
        L.oracle_spmv_csc.argtypes = [sp, vp, vp]
        L.oracle_spmv_csr.argtypes = [sp, vp, C.c_int, vp]
        L.oracle_spmvT_csc.argtypes = [sp, vp, C.c_int, vp]
        L.oracle_dnrm2.argtypes = [C.c_int64, vp]
        L.oracle_dnrm2.restype = C.c_double
        L.oracle_d2norm.argtypes = [C.c_double, C.c_double]
        L.oracle_d2norm.restype = C.c_double
        L.oracle_aprod.argtypes = [C.c_int, C.POINTER(Problem)]
        L.oracle_lsqr.argtypes = [C.POINTER(Problem), C.c_double, C.c_double, C.c_double,
                                  C.c_double, C.c_int, C.c_int, vp, vp, vp, vp,
                                  C.POINTER(Result), C.c_char_p]
        L.oracle_lsqr_op.argtypes = [C.POINTER(Problem), APROD_FN, vp, C.c_double, C.c_double,
                                     C.c_double, C.c_double, C.c_int, C.c_int, vp, vp, vp, vp,
                                     C.POINTER(Result), C.c_char_p]
        L.oracle_set_threads.argtypes = [C.c_int]
        L.oracle_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(vp)


def _sparse(lines) -> Sparse:
    s = Sparse()
    s.num_row, s.num_col, s.nnz = lines.num_row, lines.num_col, int(lines.ptr[-1])
    s.ptr, s.idx, s.val = _p(lines.ptr), _p(lines.idx), _p(lines.val)
    return s


class OracleProblem:
    """A single-rank PPDataV3_TRI over the arrays of a synth.Problem."""

    def __init__(self, prob):
        self.prob = prob
        self.y_k = np.zeros(prob.m_k)
        self.y_d = np.zeros(prob.m_d)
        self.x = np.zeros(prob.n)
        self.c = Problem()
        self.c.k_csc = _sparse(prob.k_csc)
        self.c.d_csr = _sparse(prob.d_csr)
        self.c.d_csc = _sparse(prob.d_csc)
        self.c.y_k, self.c.y_d, self.c.x = _p(self.y_k), _p(self.y_d), _p(self.x)

    def aprod(self, mode: int) -> None:
        rc = lib().oracle_aprod(mode, C.byref(self.c))
        if rc:
            raise RuntimeError(f"oracle_aprod failed: {rc}")

    def lsqr(self, iterations: int, b_k=None, damp=0.0, atol=1e-10, btol=1e-10, conlim=100.0,
             itnlim=1000, want_se=False, result_txt=None, op=None) -> dict:
        """The reference's lsqr() (source/lsqr.c:195-917).  op: another
        operator for it to call in place of the oracle's aprod, a Python
        callable op(mode, m, n, is_final, iteration) -> int that updates
        self.y_k / self.y_d (mode 1) or self.x (mode 2) in place."""
        self.y_k[:] = self.prob.b_k if b_k is None else b_k
        self.y_d[:] = 0.0
        n = self.prob.n
        w, x = np.zeros(n), np.zeros(n)
        se = np.zeros(n) if want_se else None
        hist = np.zeros(iterations + 1, ITER_DTYPE)
        r = Result()
        txt = result_txt.encode() if result_txt else None
        if op is None:
            rc = lib().oracle_lsqr(C.byref(self.c), damp, atol, btol, conlim, itnlim, iterations,
                                   _p(w), _p(x), _p(se), _p(hist), C.byref(r), txt)
        else:
            errors = []

            def call(mode, m, nn, _prob, _usr, fin, it):
                try:
                    return int(op(mode, m, nn, fin, it))
                except Exception as e:  # stop the solve, re-raised below
                    errors.append(e)
                    return 1

            cb = APROD_FN(call)
            rc = lib().oracle_lsqr_op(C.byref(self.c), cb, None, damp, atol, btol, conlim, itnlim,
                                      iterations, _p(w), _p(x), _p(se), _p(hist), C.byref(r), txt)
            if errors:
                raise errors[0]
        if rc:
            raise RuntimeError(f"oracle_lsqr failed: {rc}")
        res = {k: getattr(r, k) for k, _ in Result._fields_}
        return dict(x=x, w=w, se=se, hist=hist, result=res)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(n)


def get_threads() -> int:
    return lib().oracle_get_threads()
