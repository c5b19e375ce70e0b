"""Host side of the batched solver: the instance set, the noise generator it
uses and the product-variant table (no GPU)."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest


def test_instance_parameters(pkg):
    B = pkg.batch
    assert B.NOISE_SEEDS == tuple(range(16))
    assert len(B.LAMBDAS) == 8 and B.LAMBDAS[0] == pytest.approx(0.1)
    assert B.LAMBDAS[-1] == pytest.approx(10.0)
    assert np.allclose(np.diff(np.log(B.LAMBDAS)), np.log(100.0) / 7)
    assert B.CHECKER_PERIODS[0] == 4 and B.CHECKER_PERIODS[-1] == 16
    assert len(B.CHECKER_PERIODS) == 8


def test_pick_spreads_over_kinds(pkg):
    insts = [pkg.batch.Instance(f"i{j}", None, 1.0, None) for j in range(32)]
    assert [i.name for i in pkg.batch.pick(insts, 4)] == ["i0", "i16", "i24", "i1"]
    assert len(pkg.batch.pick(insts, 32)) == 32
    sel = pkg.batch.pick(insts, 24)
    assert len({i.name for i in sel}) == 24


def test_noise_with_the_problem_seed_gives_its_measurements(pkg):
    """plsqr_synth_noisy(seed = the problem's seed) on K x_true reproduces
    plsqr_synth_rhs bit for bit; another seed gives other noise of the same
    size."""
    N = pkg._native
    prob = pkg.generate("tiny", keep_rows=True)
    K = prob.meta["k_csr"]
    p0 = pkg.synth.params("tiny", noise_frac=0.0)
    kx = np.empty(prob.m_k)
    N.check(N.lib().plsqr_synth_rhs(C.byref(p0), N.ptr(K.ptr), N.ptr(K.idx), N.ptr(K.val),
                                    N.ptr(prob.x_true), N.ptr(kx)), "rhs")
    same = pkg.batch.noisy("tiny", pkg.CONFIGS["tiny"]["seed"], kx)
    assert np.array_equal(same, prob.b_k)
    other = pkg.batch.noisy("tiny", 3, kx)
    assert not np.array_equal(other, prob.b_k)
    n0, n1 = prob.b_k - kx, other - kx
    assert np.linalg.norm(n1) == pytest.approx(np.linalg.norm(n0), rel=0.5)


def test_checkerboard_model(pkg):
    x = pkg.batch.checkerboard("grid32", 8)
    assert set(np.unique(x)) == {-1.0, 1.0}
    cube = x.reshape(32, 32, 32)  # (iz, iy, ix)
    assert np.all(cube[0, 0, :4] == cube[0, 0, 0]) and cube[0, 0, 4] == -cube[0, 0, 0]
    assert cube[0, 4, 0] == -cube[0, 0, 0] and cube[4, 0, 0] == -cube[0, 0, 0]


def test_variant_table(pkg):
    seen = []
    for v in range(64):
        try:
            seen.append(pkg._native.batch_variant(v))
        except pkg._native.PlsqrError as e:
            assert e.code == -1
            break
    assert len(seen) == 14 and len(set(seen)) == 14
    assert all(vw in (2, 4) and lpr in (8, 16, 32) and u in (2, 4) for vw, lpr, u in seen[:12])
    assert seen[12] == (4, 0, 0)  # the slab form
    assert seen[13] == (4, -1, 0)  # the units form (passes of 4 or 8 columns)
