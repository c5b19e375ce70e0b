"""Python face of the GB300 solver: the reference's aprod / lsqr interface.

`Context` owns one device context of libplsqr_gpu.so.  Its methods mirror
the reference's operator and driver:

  aprod(mode)          aprod(version, rank, np, mode, m, n, x, y, UsrWrk, ...)
                       on the device-resident vectors (source/aprod.c:24-84)
  aprod_host(mode,...) the same on host vectors, updated in place
  lsqr(...)            lsqr(...) with call_lsqr's constants by default
                       (source/lsqr.c:34-184, 195-917)

Every call goes through the C ABI; there is no CPU path here.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .synth import Problem


def _f64(a, n, name):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if a.shape != (n,):
        raise ValueError(f"{name} must have {n} values, got shape {a.shape}")
    return a


class Context:
    def __init__(self, problem: Problem | None = None, *, files: dict | None = None,
                 precision: str = "fp64", device: int = 0, use_graph: bool = True,
                 verbose: bool = False, grid=None, order: str = "fast", lean: bool = False):
        L = N.lib()
        o = N.Opts()
        L.plsqr_default_opts(C.byref(o))
        o.device = device
        o.precision = N.PREC_MIXED if precision == "mixed" else N.PREC_FP64
        o.use_graph = int(use_graph)
        o.verbose = int(verbose)
        if order not in ("fast", "reference"):
            raise ValueError("order must be 'fast' or 'reference'")
        o.order = N.ORDER_REFERENCE if order == "reference" else N.ORDER_FAST
        o.lean = int(lean)  # release K by row / by column once the unit layouts hold them
        if grid is None and problem is not None:
            grid = problem.meta.get("grid")
        if grid is not None:
            o.grid[0], o.grid[1], o.grid[2] = (int(g) for g in grid)
        h = N.vp()
        if files is not None:
            f = N.Files()
            for k in ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol", "damp_i_bycol",
                      "b_k"):
                setattr(f, k, str(files[k]).encode())
            f.dir = str(files["dir"]).encode()
            f.row_k, f.row_d, f.col = int(files["row_k"]), int(files["row_d"]), int(files["col"])
            f.col_perm = str(files["col_perm"]).encode() if files.get("col_perm") else None
            N.check(L.plsqr_ctx_create_files(C.byref(f), C.byref(o), C.byref(h)),
                    "plsqr_ctx_create_files")
        else:
            if problem is None:
                raise ValueError("a Problem or files is needed")
            k, d, dc = (problem.k_csc.as_native(), problem.d_csr.as_native(),
                        problem.d_csc.as_native())
            N.check(L.plsqr_ctx_create(C.byref(k), C.byref(d), C.byref(dc), C.byref(o),
                                       C.byref(h)), "plsqr_ctx_create")
        self._h = h
        # the right-hand side lsqr() uses when none is given: the problem's
        # b_k, or (files) the one the library loaded
        self._b = None if problem is None else np.ascontiguousarray(problem.b_k, np.float64)
        self.precision = precision
        info = self.info()
        self.m_k, self.m_d, self.n = info["m_k"], info["m_d"], info["n"]

    # -- lifetime -----------------------------------------------------------
    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().plsqr_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, where):
        N.check(rc, where, self._h)

    def info(self) -> dict:
        i = N.Info()
        self._check(N.lib().plsqr_ctx_info(self._h, C.byref(i)), "plsqr_ctx_info")
        return {k: getattr(i, k) for k, _ in N.Info._fields_}

    # -- vectors ------------------------------------------------------------
    def set_u(self, y_k, y_d=None) -> None:
        yk = _f64(y_k, self.m_k, "y_k")
        yd = None if y_d is None else _f64(y_d, self.m_d, "y_d")
        self._check(N.lib().plsqr_set_u(self._h, N.ptr(yk), N.ptr(yd)), "plsqr_set_u")

    def get_u(self):
        yk, yd = np.empty(self.m_k), np.empty(self.m_d)
        self._check(N.lib().plsqr_get_u(self._h, N.ptr(yk), N.ptr(yd)), "plsqr_get_u")
        return yk, yd

    def set_v(self, v) -> None:
        vv = _f64(v, self.n, "v")
        self._check(N.lib().plsqr_set_v(self._h, N.ptr(vv)), "plsqr_set_v")

    def get_v(self):
        v = np.empty(self.n)
        self._check(N.lib().plsqr_get_v(self._h, N.ptr(v)), "plsqr_get_v")
        return v

    def get_b(self):
        b = np.empty(self.m_k)
        self._check(N.lib().plsqr_get_b(self._h, N.ptr(b)), "plsqr_get_b")
        return b

    # -- operator -----------------------------------------------------------
    def aprod(self, mode: int, iteration: int = 1, is_final: int = 0) -> None:
        self._check(N.lib().plsqr_aprod(self._h, mode, iteration, is_final), "plsqr_aprod")

    def aprod_host(self, mode: int, y_k: np.ndarray, y_d: np.ndarray, x: np.ndarray,
                   iteration: int = 1, is_final: int = 0) -> None:
        for a, n, nm in ((y_k, self.m_k, "y_k"), (y_d, self.m_d, "y_d"), (x, self.n, "x")):
            if a.dtype != np.float64 or a.shape != (n,) or not a.flags.c_contiguous:
                raise ValueError(f"{nm} must be a contiguous float64 array of {n} values")
        self._check(N.lib().plsqr_aprod_host(self._h, mode, N.ptr(y_k), N.ptr(y_d), N.ptr(x),
                                             iteration, is_final), "plsqr_aprod_host")

    # -- timing report (the reference's GPTL timer names) --------------------
    def set_timing(self, on: bool = True) -> None:
        """Time the following FP64 solves per region of every iteration
        (no CUDA graph while on); see write_timing."""
        self._check(N.lib().plsqr_set_timing(self._h, int(on)), "plsqr_set_timing")

    def write_timing(self, path: str) -> dict:
        """Write the last timed solve's JSON report and return it parsed."""
        import json
        self._check(N.lib().plsqr_write_timing(self._h, str(path).encode()), "plsqr_write_timing")
        with open(path) as f:
            return json.load(f)

    # -- driver -------------------------------------------------------------
    def set_reference_x(self, x_ref) -> None:
        xr = None if x_ref is None else _f64(x_ref, self.n, "x_ref")
        self._check(N.lib().plsqr_set_reference_x(self._h, N.ptr(xr)), "plsqr_set_reference_x")

    def lsqr(self, b_k=None, *, lsqr_iteration: int = 100, damp: float = 0.0,
             atol: float = 1e-10, btol: float = 1e-10, conlim: float = 100.0,
             itnlim: int = 1000, want_se: bool = False, stop_on_istop: bool = False,
             result_txt: str | None = None, sweeps: int = 4, inner: int = 50,
             want_w: bool = False, x0=None) -> dict:
        """One solve (source/lsqr.c:195-917).  Mixed-precision contexts take
        `sweeps` x `inner` iterations instead of lsqr_iteration, and x0 (n,):
        a starting solution, kept when it lowers the residual
        (result["warm"] == 1), else the solve starts from 0."""
        a = N.LsqrArgs()
        N.lib().plsqr_default_lsqr_args(C.byref(a))
        a.damp, a.atol, a.btol, a.conlim = damp, atol, btol, conlim
        a.itnlim, a.lsqr_iteration = itnlim, lsqr_iteration
        a.want_se, a.stop_on_istop = int(want_se), int(stop_on_istop)
        a.result_txt = result_txt.encode() if result_txt else None
        a.sweeps, a.inner = sweeps, inner
        xs = None if x0 is None else _f64(x0, self.n, "x0")
        a.x0 = N.ptr(xs)
        b = self._b if b_k is None else _f64(b_k, self.m_k, "b_k")
        n_hist = (sweeps * inner if self.precision == "mixed" else lsqr_iteration) + 1
        x = np.empty(self.n)
        w = np.empty(self.n) if want_w else None
        se = np.empty(self.n) if want_se else None
        hist = np.zeros(n_hist, N.ITER_DTYPE)
        r = N.Result()
        self._check(N.lib().plsqr_lsqr(self._h, C.byref(a), N.ptr(b), N.ptr(x), N.ptr(w),
                                       N.ptr(se), N.ptr(hist), C.byref(r)), "plsqr_lsqr")
        res = {k: getattr(r, k) for k, _ in N.Result._fields_ if k != "pad"}
        return dict(x=x, w=w, se=se, hist=hist, result=res)

    # -- several right-hand sides ----------------------------------------------
    def batch_lsqr(self, b_k, *, lam=None, x_ref=None, x0=None, sweeps: int = 4, inner: int = 50,
                   damp: float = 0.0, atol: float = 1e-10, btol: float = 1e-10,
                   conlim: float = 100.0, variant_rows: int = -1,
                   variant_cols: int = -1, retire_every: int = 0,
                   retire_err: float = 0.0) -> dict:
        """k <= 32 solves in lock step, one k-wide product per matrix read.

        b_k: (k, m_k) right-hand sides; lam: (k,) damping-row weights (solve j
        uses [K; lam_j D]); x_ref: (k, n) solutions for the history's err
        field; x0: (k, n) starting solutions (warm start, with the cold start
        as fallback where b - A x0 is not smaller than b; info["warm"] has bit
        j set where x0 was kept).  retire_every = R > 0: every R iterations
        the finished solves (err <= retire_err with x_ref where retire_err >
        0, else LSQR's own stop in the last sweep) retire with their x and
        result as they stand (result "itn": the iteration they retired at)
        and the rest go on in a block no wider than they need.  Returns x (k, n), hist (k,
        sweeps*inner + 1), per-solve results and the product variants used."""
        b = np.ascontiguousarray(b_k, np.float64)
        if b.ndim != 2 or b.shape[1] != self.m_k:
            raise ValueError(f"b_k must have shape (k, {self.m_k}), got {b.shape}")
        k = b.shape[0]
        lm = None if lam is None else np.ascontiguousarray(lam, np.float64)
        if lm is not None and lm.shape != (k,):
            raise ValueError(f"lam must have {k} values")
        xr = None if x_ref is None else np.ascontiguousarray(x_ref, np.float64)
        if xr is not None and xr.shape != (k, self.n):
            raise ValueError(f"x_ref must have shape ({k}, {self.n})")
        xs = None if x0 is None else np.ascontiguousarray(x0, np.float64)
        if xs is not None and xs.shape != (k, self.n):
            raise ValueError(f"x0 must have shape ({k}, {self.n})")
        a = N.BatchArgs()
        N.lib().plsqr_default_batch_args(C.byref(a))
        a.k, a.sweeps, a.inner = k, sweeps, inner
        a.variant_rows, a.variant_cols = variant_rows, variant_cols
        a.retire_every, a.retire_err = retire_every, retire_err
        a.damp, a.atol, a.btol, a.conlim = damp, atol, btol, conlim
        a.b_k, a.lambda_, a.x_ref, a.x0 = N.ptr(b), N.ptr(lm), N.ptr(xr), N.ptr(xs)
        x = np.empty((k, self.n))
        hist = np.zeros((k, sweeps * inner + 1), N.ITER_DTYPE)
        res = (N.Result * k)()
        info = N.BatchInfo()
        self._check(N.lib().plsqr_batch_lsqr(self._h, C.byref(a), N.ptr(x), N.ptr(hist),
                                             C.cast(res, N.vp), C.byref(info)),
                    "plsqr_batch_lsqr")
        results = [{f: getattr(r, f) for f, _ in N.Result._fields_ if f != "pad"} for r in res]
        return dict(x=x, hist=hist, results=results,
                    info={f: getattr(info, f) for f, _ in N.BatchInfo._fields_})

    def batch_bench_aprod(self, k: int, mode: int, variant: int = -1, reps: int = 5) -> float:
        """ms per launch of the k-wide product (mode 1 or 2) of a variant
        (-1: the one picked by timing)."""
        ms = N.f64(0)
        self._check(N.lib().plsqr_batch_bench_aprod(self._h, k, mode, variant, reps,
                                                    C.byref(ms)), "plsqr_batch_bench_aprod")
        return float(ms.value)

    def set_damping_weight(self, lam: float) -> None:
        """Damping rows become lam * D (from the values the context was made with)."""
        self._check(N.lib().plsqr_set_damping_weight(self._h, float(lam)),
                    "plsqr_set_damping_weight")

    # -- measurement ----------------------------------------------------------
    def bench_aprod(self, mode: int, reps: int = 10) -> float:
        """ms per launch of the mode-1/2 product kernel (overwrites u, v)."""
        ms = N.f64(0)
        self._check(N.lib().plsqr_bench_aprod(self._h, mode, reps, C.byref(ms)),
                    "plsqr_bench_aprod")
        return float(ms.value)

    def bench_iteration(self, reps: int = 10) -> float:
        """ms per LSQR iteration replayed from its CUDA graph."""
        ms = N.f64(0)
        self._check(N.lib().plsqr_bench_iteration(self._h, reps, C.byref(ms)),
                    "plsqr_bench_iteration")
        return float(ms.value)

    def get_x(self):
        x = np.empty(self.n)
        self._check(N.lib().plsqr_get_x(self._h, N.ptr(x)), "plsqr_get_x")
        return x

    def write_result(self, path: str) -> None:
        self._check(N.lib().plsqr_write_result(self._h, str(path).encode()), "plsqr_write_result")
