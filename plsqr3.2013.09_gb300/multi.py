"""Independent problems of different sizes in one persistent launch.

`Multi` wraps plsqr_multi_*: every problem is a complete FP64 lsqr() on its
own operator, and one cooperative kernel launch runs them all, each on a
group of thread blocks sized by the host planner (`plan_host`).

`uneven_configs()` is the 24-problem set: model grids from 16^3 to 64^3 cells
and 500 to 20,000 rays, built like the 32x32x32 problem (tube radius 1.5,
8 Gaussian blobs, 1% noise, 100 iterations), paired so that grid size and ray
count do not grow together.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .synth import CONFIGS, Problem


def uneven_configs(count: int = 24) -> list[dict]:
    out = []
    for i in range(count):
        f = i / max(count - 1, 1)
        side = int(round(16 * 4.0 ** f))
        j = (7 * i) % count  # a permutation of 0..count-1 (7 and 24 are coprime)
        rays = int(round(500 * 40.0 ** (j / max(count - 1, 1))))
        out.append(dict(CONFIGS["grid32"], nx=side, ny=side, nz=side, n_rays=rays, seed=100 + i,
                        iterations=100))
    return out


def plan_host(bytes_per_iteration, iterations, blocks: int, bw_block: float):
    """The planner on the host: (group of each problem, blocks of each group)."""
    b = np.ascontiguousarray(bytes_per_iteration, np.float64)
    it = np.ascontiguousarray(iterations, np.int32)
    count = b.size
    group = np.empty(count, np.int32)
    gb = np.zeros(max(count, blocks), np.int32)
    ng = N.i32(0)
    N.check(N.lib().plsqr_multi_plan_host(N.ptr(b), N.ptr(it), count, blocks, bw_block,
                                          N.ptr(group), N.ptr(gb), C.byref(ng)),
            "plsqr_multi_plan_host")
    return group, gb[:ng.value].copy()


class Multi:
    def __init__(self, problems: list[Problem], iterations=None, *, device: int = 0,
                 damp: float = 0.0):
        L = N.lib()
        self.count = len(problems)
        its = [p.iterations if iterations is None else
               (iterations[i] if np.ndim(iterations) else int(iterations))
               for i, p in enumerate(problems)]
        self.iterations = [int(v) for v in its]
        self.n = [p.n for p in problems]
        descs = (N.ProblemDesc * self.count)()
        self._keep = []
        for i, p in enumerate(problems):
            d = descs[i]
            L.plsqr_default_problem(C.byref(d))
            b = np.ascontiguousarray(p.b_k, np.float64)
            self._keep.append(b)
            d.k_csc, d.d_csr, d.d_csc = (p.k_csc.as_native(), p.d_csr.as_native(),
                                         p.d_csc.as_native())
            d.b_k = N.ptr(b)
            d.lsqr_iteration = self.iterations[i]
            d.damp = damp
        o = N.Opts()
        L.plsqr_default_opts(C.byref(o))
        o.device = device
        h = N.vp()
        N.check(L.plsqr_multi_create(descs, self.count, C.byref(o), C.byref(h)),
                "plsqr_multi_create")
        self._keep = None
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().plsqr_multi_destroy(self._h)
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
        if rc != N.PLSQR_OK:
            raise N.PlsqrError(rc, where, (N.lib().plsqr_multi_last_error(self._h) or b"").decode())

    def info(self) -> dict:
        i = N.MultiInfo()
        self._check(N.lib().plsqr_multi_info_get(self._h, C.byref(i)), "plsqr_multi_info_get")
        return {k: getattr(i, k) for k, _ in N.MultiInfo._fields_}

    def plan(self):
        g = np.empty(self.count, np.int32)
        gb = np.empty(self.count, np.int32)
        self._check(N.lib().plsqr_multi_plan(self._h, N.ptr(g), N.ptr(gb)), "plsqr_multi_plan")
        return g, gb

    def set_exact(self, exact: bool) -> None:
        """Products in the reference's rounding (multiply and add apart)."""
        self._check(N.lib().plsqr_multi_set_exact(self._h, int(bool(exact))),
                    "plsqr_multi_set_exact")

    def set_mixed(self, sweeps: int) -> None:
        """sweeps > 0: FP32 inner / FP64 outer, `sweeps` refinement sweeps of
        each problem's iteration count; 0: one FP64 LSQR."""
        self._check(N.lib().plsqr_multi_set_mixed(self._h, int(sweeps)), "plsqr_multi_set_mixed")

    def set_wait(self, wait_ns: int) -> None:
        self._check(N.lib().plsqr_multi_set_wait(self._h, int(wait_ns)), "plsqr_multi_set_wait")

    def check_wait(self, wait_ns: int) -> int:
        """Return code of one bounded device wait on a flag nothing sets."""
        return int(N.lib().plsqr_multi_check_wait(self._h, int(wait_ns)))

    def solve(self) -> dict:
        x = np.empty(sum(self.n))
        hist = np.zeros(sum(i + 1 for i in self.iterations), N.ITER_DTYPE)
        res = (N.Result * self.count)()
        self._check(N.lib().plsqr_multi_solve(self._h, N.ptr(x), N.ptr(hist), C.cast(res, N.vp)),
                    "plsqr_multi_solve")
        xs, hs = [], []
        ox = oh = 0
        for n, it in zip(self.n, self.iterations):
            xs.append(x[ox:ox + n])
            hs.append(hist[oh:oh + it + 1])
            ox += n
            oh += it + 1
        results = [{f: getattr(r, f) for f, _ in N.Result._fields_ if f != "pad"} for r in res]
        return dict(x=xs, hist=hs, results=results, seconds=self.info()["seconds"])
