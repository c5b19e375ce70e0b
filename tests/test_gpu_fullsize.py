"""The 96x96x32 problem at full size (200,000 rays, 1.33e9 kernel nonzeros,
~45 GB on the device), where the oracle would take minutes per iteration:
size-independent properties instead of a comparison with the reference.
The adjoint identity and linearity of the products, residual norms that
never grow over the LSQR iterations, the mixed-precision start-up and first
iterations within FP32 accuracy of the FP64 ones, and exact power-of-two
scaling across a batch of right-hand sides."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grid96(pkg):
    return pkg.generate("grid96")


def test_products_are_adjoint_and_linear(pkg, grid96):
    prob = grid96
    rng = np.random.default_rng(21)
    x1, x2 = rng.standard_normal(prob.n), rng.standard_normal(prob.n)
    yk, yd = rng.standard_normal(prob.m_k), rng.standard_normal(prob.m_d)
    with pkg.Context(prob) as ctx:

        def ax(x):
            k, d = np.zeros(prob.m_k), np.zeros(prob.m_d)
            ctx.aprod_host(1, k, d, x.copy())
            return k, d

        a1k, a1d = ax(x1)
        a2k, a2d = ax(x2)
        a3k, a3d = ax(x1 + 2.0 * x2)
        aty = np.zeros(prob.n)
        ctx.aprod_host(2, yk.copy(), yd.copy(), aty)
    # <A x, y> = <x, A^T y>, to rounding of |A||x||y|
    lhs = a1k @ yk + a1d @ yd
    rhs = x1 @ aty
    assert abs(lhs - rhs) <= 1e-12 * (np.abs(a1k) @ np.abs(yk) + np.abs(a1d) @ np.abs(yd))
    # A (x1 + 2 x2) = A x1 + 2 A x2
    assert rel(a3k, a1k + 2.0 * a2k) <= 1e-12
    assert rel(a3d, a1d + 2.0 * a2d) <= 1e-12


def test_lsqr_residuals_never_grow(pkg, grid96):
    with pkg.Context(grid96) as ctx:
        out = ctx.lsqr(lsqr_iteration=30)
    r = out["hist"]["rnorm"]
    assert np.all(np.isfinite(out["x"]))
    assert np.all(np.diff(r) <= 1e-12 * r[:-1])
    assert r[-1] < r[0]


def test_mixed_start_and_first_iterations_match_fp64(pkg, grid96):
    with pkg.Context(grid96) as c64:
        h64 = c64.lsqr(lsqr_iteration=5)["hist"]
    with pkg.Context(grid96, precision="mixed") as cm:
        hm = cm.lsqr(sweeps=1, inner=5)["hist"]
    for key in ("alpha", "beta"):
        assert np.max(np.abs(hm[key] - h64[key]) / np.abs(h64[key])) <= 1e-5, key


def test_batched_right_hand_sides_scale_exactly(pkg, grid96):
    """k right-hand sides b, b/2 and 2b in one batch: the solutions are x,
    x/2 and 2x bit for bit (scaling by a power of two is exact and the
    right-hand sides do not interact)."""
    b = grid96.b_k
    with pkg.Context(grid96) as ctx:
        out = ctx.batch_lsqr(np.stack([b, 0.5 * b, 2.0 * b]), sweeps=1, inner=10)
    x = out["x"]
    assert np.all(np.isfinite(x[0])) and np.any(x[0] != 0.0)
    assert np.array_equal(x[1], 0.5 * x[0])
    assert np.array_equal(x[2], 2.0 * x[0])
