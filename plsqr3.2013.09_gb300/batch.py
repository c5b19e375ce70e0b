"""Right-hand-side sets for the batched solver (Context.batch_lsqr).

The 32-instance set on one operator: 16 noise realisations of the problem's
own measurements (noise seeds 0-15), the problem's measurements under 8
damping weights lambda log-spaced in [0.1, 10] (solve j uses [K; lambda_j D]),
and 8 checkerboard resolution tests (a +-1 checkerboard of period 4-16 cells
as the model, 1% noise).  K x is formed by the context's FP64 operator
(aprod mode 1), the noise by the native generator (plsqr_synth_noisy), so the
set is the same on every machine up to the rounding of K x.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .synth import Problem, params

NOISE_SEEDS = tuple(range(16))
LAMBDAS = tuple(float(v) for v in np.geomspace(0.1, 10.0, 8))
CHECKER_PERIODS = (4, 5, 6, 8, 10, 12, 14, 16)


@dataclass
class Instance:
    name: str
    b_k: np.ndarray
    lam: float
    x_true: np.ndarray


def kernel_product(ctx, x: np.ndarray) -> np.ndarray:
    """K x with the context's FP64 operator (overwrites its u and v)."""
    ctx.set_v(x)
    ctx.set_u(np.zeros(ctx.m_k), np.zeros(ctx.m_d))
    ctx.aprod(1)
    return ctx.get_u()[0]


def noisy(cfg, noise_seed: int, kx: np.ndarray) -> np.ndarray:
    p = params(cfg)
    b = np.empty_like(kx)
    N.check(N.lib().plsqr_synth_noisy(C.byref(p), int(noise_seed), kx.size, N.ptr(kx),
                                      N.ptr(b)), "plsqr_synth_noisy")
    return b


def checkerboard(cfg, period: int) -> np.ndarray:
    p = params(cfg, n_blobs=0, checker_amp=1.0, checker_period=int(period))
    x = np.empty(p.nx * p.ny * p.nz)
    N.check(N.lib().plsqr_synth_xtrue(C.byref(p), N.ptr(x)), "plsqr_synth_xtrue")
    return x


def instances(ctx, prob: Problem, cfg) -> list[Instance]:
    """The 32 instances on prob's operator (ctx holds prob, FP64 products);
    cfg is the configuration name or dict prob was generated from."""
    kx = kernel_product(ctx, prob.x_true)
    out = [Instance(f"noise{s}", noisy(cfg, s, kx), 1.0, prob.x_true) for s in NOISE_SEEDS]
    out += [Instance(f"lambda{lam:.3g}", prob.b_k.copy(), lam, prob.x_true) for lam in LAMBDAS]
    for per in CHECKER_PERIODS:
        xc = checkerboard(cfg, per)
        out.append(Instance(f"checker{per}", noisy(cfg, 0, kernel_product(ctx, xc)), 1.0, xc))
    return out


def pick(insts: list[Instance], k: int) -> list[Instance]:
    """k instances spread over the three kinds (all 32 for k = 32)."""
    if k >= len(insts):
        return list(insts)
    order = []
    groups = [insts[:16], insts[16:24], insts[24:32]]
    i = 0
    while len(order) < k:
        g = groups[i % 3]
        j = i // 3
        if j < len(g):
            order.append(g[j])
        i += 1
    return order
