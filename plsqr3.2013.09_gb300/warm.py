"""Learned warm start: a 3-D U-Net from the column-norm-scaled
back-projection A^T b to a starting solution x0 (plsqr_unet_*), trained on
(A^T b, x_LSQR) pairs that this library's solvers produce, and handed to the
batched solver as x0 (with the cold start as fallback).

The model class: seeded x_true of 16-128 Gaussian blobs plus a checkerboard of
random period (4-16 cells, amplitude 0-0.2), measured through the problem's
kernel with 1% noise.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .batch import kernel_product, noisy
from .synth import params


class UNet:
    def __init__(self, grid, seed: int = 1, device: int = 0):
        nx, ny, nz = (int(g) for g in grid)
        self.grid = (nx, ny, nz)
        self.n = nx * ny * nz
        h = N.vp()
        N.check(N.lib().plsqr_unet_create(nx, ny, nz, seed, device, C.byref(h)), "plsqr_unet_create")
        self._h = h

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().plsqr_unet_destroy(self._h)
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
            raise N.PlsqrError(rc, where, (N.lib().plsqr_unet_last_error(self._h) or b"").decode())

    def predict(self, z: np.ndarray) -> np.ndarray:
        zi = np.ascontiguousarray(z, np.float32)
        out = np.empty(self.n, np.float32)
        self._check(N.lib().plsqr_unet_predict(self._h, N.ptr(zi), N.ptr(out)), "plsqr_unet_predict")
        return out.astype(np.float64)

    def train_step(self, z: np.ndarray, target: np.ndarray, lr: float) -> float:
        zi = np.ascontiguousarray(z, np.float32)
        ti = np.ascontiguousarray(target, np.float32)
        loss = C.c_float(0.0)
        self._check(N.lib().plsqr_unet_train_step(self._h, N.ptr(zi), N.ptr(ti), float(lr),
                                                  C.byref(loss)), "plsqr_unet_train_step")
        return float(loss.value)

    def weights(self) -> np.ndarray:
        cnt = N.i64(0)
        self._check(N.lib().plsqr_unet_weights(self._h, None, C.byref(cnt), 0), "plsqr_unet_weights")
        buf = np.empty(cnt.value, np.float32)
        self._check(N.lib().plsqr_unet_weights(self._h, N.ptr(buf), C.byref(cnt), 0),
                    "plsqr_unet_weights")
        return buf

    def set_weights(self, buf: np.ndarray) -> None:
        b = np.ascontiguousarray(buf, np.float32)
        cnt = N.i64(b.size)
        self._check(N.lib().plsqr_unet_weights(self._h, N.ptr(b), C.byref(cnt), 1),
                    "plsqr_unet_weights")


def conv3d_check(grid, x, w, b, dy):
    """One convolution + ReLU layer through the network's kernels: (y, dx,
    dw, db) for x [n][cin], w [cout][27*cin], b [cout], dy [n][cout]."""
    nx, ny, nz = grid
    n = nx * ny * nz
    cin, cout = x.shape[1], w.shape[0]
    xs, ws, bs, dys = (np.ascontiguousarray(a, np.float32) for a in (x, w, b, dy))
    y = np.empty((n, cout), np.float32)
    dx = np.empty((n, cin), np.float32)
    dw = np.empty((cout, 27 * cin), np.float32)
    db = np.empty(cout, np.float32)
    N.check(N.lib().plsqr_nn_conv3d_check(nx, ny, nz, cin, cout, N.ptr(xs), N.ptr(ws), N.ptr(bs),
                                          N.ptr(dys), N.ptr(y), N.ptr(dx), N.ptr(dw), N.ptr(db)),
            "plsqr_nn_conv3d_check")
    return y, dx, dw, db


def column_norms2(prob) -> np.ndarray:
    """||A e_c||^2 for every column c (kernel and damping parts)."""
    out = np.zeros(prob.n)
    for L in (prob.k_csc, prob.d_csc):
        if L.nnz == 0:
            continue
        starts = np.minimum(L.ptr[:-1], L.nnz - 1)
        out += np.add.reduceat(L.val * L.val, starts) * (np.diff(L.ptr) > 0)
    return out


def back_projection(ctx, b_k: np.ndarray, colnorm2: np.ndarray) -> np.ndarray:
    """A^T [b; 0] / ||A e_c||^2 with the context's FP64 operator."""
    ctx.set_u(b_k, np.zeros(ctx.m_d))
    ctx.set_v(np.zeros(ctx.n))
    ctx.aprod(2)
    v = ctx.get_v()
    return np.where(colnorm2 > 0, v / np.maximum(colnorm2, 1e-300), 0.0)


def model_instance(cfg, seed: int):
    """x_true of the model class for one seed, and the synthetic parameters."""
    rng = np.random.default_rng(10_000 + seed)
    over = dict(seed=int(seed), n_blobs=int(rng.integers(16, 129)),
                checker_amp=float(rng.uniform(0.0, 0.2)), checker_period=int(rng.integers(4, 17)))
    p = params(cfg, **over)
    x = np.empty(p.nx * p.ny * p.nz)
    N.check(N.lib().plsqr_synth_xtrue(C.byref(p), N.ptr(x)), "plsqr_synth_xtrue")
    return x, over


def measurements(ctx, cfg, seed: int):
    """(x_true, b_k) of one instance: the kernel product of x_true with 1%
    noise drawn from the instance's seed."""
    x, over = model_instance(cfg, seed)
    kx = kernel_product(ctx, x)
    return x, noisy(cfg, seed, kx)
