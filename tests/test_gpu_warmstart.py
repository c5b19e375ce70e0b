"""The warm-start network's kernels and training step (plsqr_unet_*,
plsqr_nn_conv3d_check).  There is no network in the reference: the
yardsticks are a float64 NumPy convolution on the same BF16-rounded operands
and the behaviour of training."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def bf16(a):
    """Round float32 values to the nearest BF16 (ties to even)."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def im2col(x, grid):
    nx, ny, nz = grid
    n, cin = x.shape
    v = x.reshape(nz, ny, nx, cin)
    pad = np.zeros((nz + 2, ny + 2, nx + 2, cin))
    pad[1:-1, 1:-1, 1:-1] = v
    cols = []
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                cols.append(pad[1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx]
                            .reshape(n, cin))
    return np.concatenate(cols, axis=1)  # [n][t*cin + c], t = (dz+1)*9 + (dy+1)*3 + dx+1


def col2im(dcol, grid, cin):
    nx, ny, nz = grid
    n = nx * ny * nz
    out = np.zeros((nz + 2, ny + 2, nx + 2, cin))
    t = 0
    for dz in (-1, 0, 1):
        for dy in (-1, 0, 1):
            for dx in (-1, 0, 1):
                out[1 + dz:1 + dz + nz, 1 + dy:1 + dy + ny, 1 + dx:1 + dx + nx] += \
                    dcol[:, t * cin:(t + 1) * cin].reshape(nz, ny, nx, cin)
                t += 1
    return out[1:-1, 1:-1, 1:-1].reshape(n, cin)


@pytest.mark.parametrize("cin,cout", [(16, 32), (48, 16), (32, 64), (64, 64), (96, 32)])
def test_conv_layer_matches_numpy(pkg, cin, cout):
    grid = (8, 6, 4)
    n = 8 * 6 * 4
    rng = np.random.default_rng(cin + cout)
    x = bf16(rng.standard_normal((n, cin)))
    w = bf16(0.1 * rng.standard_normal((cout, 27 * cin)))
    b = 0.1 * rng.standard_normal(cout).astype(np.float32)
    dy = rng.standard_normal((n, cout)).astype(np.float32)
    y, dx, dw, db = pkg.warm.conv3d_check(grid, x, w, b, dy)
    col = im2col(x.astype(np.float64), grid)
    y_ref = np.maximum(col @ w.astype(np.float64).T + b, 0.0)
    assert rel(y, y_ref) <= 1e-2  # BF16 output
    dz = bf16(np.where(y > 0, dy, 0.0))
    assert rel(db, dz.sum(axis=0)) <= 1e-5
    assert rel(dw, dz.astype(np.float64).T @ col) <= 1e-4
    dx_ref = col2im(dz.astype(np.float64) @ w.astype(np.float64), grid, cin)
    assert rel(dx, dx_ref) <= 1e-4


def test_training_lowers_the_loss_and_is_repeatable(pkg):
    grid = (16, 16, 8)
    n = 16 * 16 * 8
    rng = np.random.default_rng(3)
    z = rng.standard_normal(n)
    target = 0.5 * z + 0.2 * np.roll(z, 1)  # a local linear map
    losses = []
    with pkg.warm.UNet(grid, seed=4) as net:
        w0 = net.weights()
        p0 = net.predict(z)
        assert np.array_equal(p0, net.predict(z))
        for _ in range(40):
            losses.append(net.train_step(z, target, 2e-3))
        p1 = net.predict(z)
        net.set_weights(w0)
        assert np.array_equal(net.predict(z), p0)
    assert all(np.isfinite(losses))
    assert np.mean(losses[-5:]) < 0.5 * np.mean(losses[:5])
    assert rel(p1, target) < rel(p0, target)


def test_torch_custom_ops_match_the_host_calls(pkg):
    """torch.ops.plsqr.unet_predict / unet_train_step on CUDA tensors give the
    bits of plsqr_unet_predict / plsqr_unet_train_step on host arrays."""
    torch = pytest.importorskip("torch")
    grid = (16, 16, 8)
    n = 16 * 16 * 8
    rng = np.random.default_rng(11)
    z = rng.standard_normal(n).astype(np.float32)
    target = (0.5 * z + 0.2 * np.roll(z, 1)).astype(np.float32)
    ops = pkg.warm.torch_ops()
    zt = torch.tensor(z, device="cuda")
    tt = torch.tensor(target, device="cuda")
    with pkg.warm.UNet(grid, seed=4) as a, pkg.warm.UNet(grid, seed=4) as b:
        p_host = a.predict(z)
        p_dev = ops.unet_predict(b.handle, zt)
        assert np.array_equal(p_host, p_dev.cpu().numpy().astype(np.float64))
        for lr in (2e-3, 1e-3):
            l_host = a.train_step(z, target, lr)
            l_dev = ops.unet_train_step(b.handle, zt, tt, lr)
            assert l_host == float(l_dev)
        assert np.array_equal(a.weights(), b.weights())
        assert np.array_equal(a.predict(z), ops.unet_predict(b.handle, zt).cpu().numpy()
                              .astype(np.float64))
