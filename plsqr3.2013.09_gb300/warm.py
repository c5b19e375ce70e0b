"""Learned warm start: a 3-D U-Net from the column-norm-scaled
back-projection A^T b to a starting solution x0 (plsqr_unet_*), trained on
(A^T b, x_LSQR) pairs that this library's solvers produce, and handed to the
batched solver as x0 (with the cold start as fallback).

The model class (model_instance): seeded x_true of 16-128 Gaussian blobs
plus a checkerboard of random period (4-16 cells, amplitude 0-0.2), measured
through the problem's kernel with 1% noise.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .batch import kernel_product, noisy


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

    @property
    def handle(self) -> int:
        """The plsqr_unet pointer, for the PyTorch custom ops (torch_ops)."""
        return int(self._h.value)

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


_OPS = None


def torch_ops():
    """The network as PyTorch custom ops on CUDA tensors (registered once):
    torch.ops.plsqr.unet_predict(net, z) -> x0 and
    torch.ops.plsqr.unet_train_step(net, z, target, lr) -> loss (a 0-d CPU
    tensor), with net = UNet.handle and float32 volumes of the network's
    grid on its device.  They run the device-array calls
    (plsqr_unet_*_device) ordered on the current CUDA stream."""
    global _OPS
    if _OPS is not None:
        return _OPS
    import torch

    if hasattr(torch.ops.plsqr, "unet_predict"):  # registered by another copy of this module
        _OPS = torch.ops.plsqr
        return _OPS

    def _vol(t, name: str):
        if t.dtype != torch.float32 or not t.is_cuda:
            raise ValueError(f"{name} must be a float32 CUDA tensor")
        return t.contiguous()

    @torch.library.custom_op("plsqr::unet_predict", mutates_args=(),
                             schema="(int net, Tensor z) -> Tensor")
    def unet_predict(net, z):
        z = _vol(z, "z")
        out = torch.empty_like(z)
        stream = torch.cuda.current_stream(z.device).cuda_stream
        N.check(N.lib().plsqr_unet_predict_device(C.c_void_p(net), C.c_void_p(z.data_ptr()),
                                                   C.c_void_p(out.data_ptr()),
                                                   C.c_void_p(stream)),
                "plsqr_unet_predict_device")
        return out

    @unet_predict.register_fake
    def _(net, z):
        return torch.empty_like(z)

    @torch.library.custom_op("plsqr::unet_train_step", mutates_args=(),
                             schema="(int net, Tensor z, Tensor target, float lr) -> Tensor")
    def unet_train_step(net, z, target, lr):
        z, target = _vol(z, "z"), _vol(target, "target")
        loss = C.c_float(0.0)
        stream = torch.cuda.current_stream(z.device).cuda_stream
        N.check(N.lib().plsqr_unet_train_step_device(C.c_void_p(net), C.c_void_p(z.data_ptr()),
                                                      C.c_void_p(target.data_ptr()), float(lr),
                                                      C.byref(loss), C.c_void_p(stream)),
                "plsqr_unet_train_step_device")
        return torch.tensor(loss.value, dtype=torch.float32)

    @unet_train_step.register_fake
    def _(net, z, target, lr):
        return torch.empty((), dtype=torch.float32)

    _OPS = torch.ops.plsqr
    return _OPS


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
        step = 4096  # columns per chunk: no squared copy of the whole matrix
        for c0 in range(0, prob.n, step):
            c1 = min(prob.n, c0 + step)
            a, b = int(L.ptr[c0]), int(L.ptr[c1])
            if b == a:
                continue
            v = L.val[a:b]
            starts = np.minimum(L.ptr[c0:c1] - a, b - a - 1)
            out[c0:c1] += np.add.reduceat(v * v, starts) * (np.diff(L.ptr[c0:c1 + 1]) > 0)
    return out


def back_projection(ctx, b_k: np.ndarray, colnorm2: np.ndarray) -> np.ndarray:
    """A^T [b; 0] / ||A e_c||^2 with the context's FP64 operator."""
    ctx.set_u(b_k, np.zeros(ctx.m_d))
    ctx.set_v(np.zeros(ctx.n))
    ctx.aprod(2)
    v = ctx.get_v()
    return np.where(colnorm2 > 0, v / np.maximum(colnorm2, 1e-300), 0.0)


def model_instance(grid, seed: int) -> np.ndarray:
    """x_true of the model class for one seed (NumPy PCG64 stream of the
    seed): 16-128 Gaussian blobs (sigma 3 cells, N(0,1) amplitudes, cut at 4
    sigma) plus a +-a checkerboard, a in [0, 0.2], of period 4-16 cells."""
    nx, ny, nz = grid
    rng = np.random.default_rng(10_000 + int(seed))
    nb = int(rng.integers(16, 129))
    c = rng.uniform(0.0, 1.0, (nb, 3)) * np.array([nz, ny, nx])
    amp = rng.standard_normal(nb)
    period = int(rng.integers(4, 17))
    a = float(rng.uniform(0.0, 0.2))
    x = np.zeros((nz, ny, nx))
    sig, r = 3.0, 12
    for k in range(nb):
        lo = np.maximum(c[k].astype(int) - r, 0)
        hi = np.minimum(c[k].astype(int) + r + 1, [nz, ny, nx])
        zz, yy, xx = np.ogrid[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]]
        d2 = (zz + 0.5 - c[k, 0]) ** 2 + (yy + 0.5 - c[k, 1]) ** 2 + (xx + 0.5 - c[k, 2]) ** 2
        x[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] += amp[k] * np.exp(-d2 / (2 * sig * sig))
    half = max(period // 2, 1)
    zz, yy, xx = np.ogrid[0:nz, 0:ny, 0:nx]
    x += np.where((zz // half + yy // half + xx // half) % 2 == 0, a, -a)
    return x.reshape(-1)


def measurements(ctx, cfg, grid, seed: int):
    """(x_true, b_k) of one instance: the kernel product of x_true with 1%
    noise drawn from the instance's seed (plsqr_synth_noisy)."""
    x = model_instance(grid, seed)
    return x, noisy(cfg, 50_000 + int(seed), kernel_product(ctx, x))


def solve_batches(ctx, bs: list, inner: int, x0s=None, x_refs=None, k: int = 32):
    """Batched mixed solves (one sweep of `inner` iterations) of the right-hand
    sides bs, k at a time: (x list, history list, seconds per batch)."""
    xs, hs, secs = [], [], []
    for i in range(0, len(bs), k):
        b = np.stack(bs[i:i + k])
        kw = dict(sweeps=1, inner=inner)
        if x0s is not None:
            kw["x0"] = np.stack(x0s[i:i + k])
        if x_refs is not None:
            kw["x_ref"] = np.stack(x_refs[i:i + k])
        out = ctx.batch_lsqr(b, **kw)
        xs += list(out["x"])
        hs += list(out["hist"])
        secs.append(out["results"][0]["seconds"])
    return xs, hs, secs
