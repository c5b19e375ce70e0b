"""Unit checks of the oracle's building blocks (CPU): the SpMV kernels of
CPUSpMV.c against scipy, the overflow-safe 2-norm of mycblas.c, d2norm of
cblas.h, and the adjoint identity of aprod."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import scipy.sparse as sp


def mats(prob):
    K = sp.csc_matrix((prob.k_csc.val, prob.k_csc.idx, prob.k_csc.ptr), shape=(prob.m_k, prob.n))
    D = sp.csr_matrix((prob.d_csr.val, prob.d_csr.idx, prob.d_csr.ptr), shape=(prob.m_d, prob.n))
    return K, D


def test_spmv_kernels_against_scipy(pkg, orc):
    prob = pkg.generate("tiny")
    K, D = mats(prob)
    rng = np.random.default_rng(0)
    x = rng.standard_normal(prob.n)
    L = orc.lib()
    sk = orc._sparse(prob.k_csc)
    sd = orc._sparse(prob.d_csr)
    sdc = orc._sparse(prob.d_csc)
    y = np.zeros(prob.m_k)
    L.oracle_spmv_csc(C.byref(sk), orc._p(x), orc._p(y))
    assert np.allclose(y, K @ x, rtol=1e-13, atol=1e-15)
    yd = np.ones(prob.m_d)
    L.oracle_spmv_csr(C.byref(sd), orc._p(x), 0, orc._p(yd))
    assert np.allclose(yd, 1.0 + D @ x, rtol=1e-13, atol=1e-15)
    u = rng.standard_normal(prob.m_k)
    t = np.zeros(prob.n)
    L.oracle_spmvT_csc(C.byref(sk), orc._p(u), 0, orc._p(t))
    assert np.allclose(t, K.T @ u, rtol=1e-13, atol=1e-15)
    ud = rng.standard_normal(prob.m_d)
    t2 = np.zeros(prob.n)
    L.oracle_spmvT_csc(C.byref(sdc), orc._p(ud), 0, orc._p(t2))
    assert np.allclose(t2, D.T @ ud, rtol=1e-13, atol=1e-15)


def test_spmv_csr_offset_argument(pkg, orc):
    """cpuSpMV_CSR_v2 indexes x[col - startIdxOfX] (CPUSpMV.c:69)."""
    prob = pkg.generate("tiny")
    _, D = mats(prob)
    x = np.arange(prob.n, dtype=float)
    xs = np.concatenate([np.zeros(5), x])
    y = np.zeros(prob.m_d)
    sd = orc._sparse(prob.d_csr)
    orc.lib().oracle_spmv_csr(C.byref(sd), orc._p(xs[5:]), 0, orc._p(y))
    assert np.allclose(y, D @ x)


@pytest.mark.parametrize("scale", [1.0, 1e-200, 1e200])
def test_dnrm2_is_overflow_safe(orc, scale):
    v = np.array([3.0, 0.0, -4.0, 12.0]) * scale
    r = orc.lib().oracle_dnrm2(4, orc._p(v))
    assert r == pytest.approx(13.0 * scale, rel=1e-15)
    one = np.array([-2.5])
    assert orc.lib().oracle_dnrm2(1, orc._p(one)) == 2.5
    assert orc.lib().oracle_dnrm2(0, orc._p(one)) == 0.0


def test_d2norm(orc):
    L = orc.lib()
    assert L.oracle_d2norm(3.0, 4.0) == pytest.approx(5.0, rel=1e-15)  # scaled form rounds
    assert L.oracle_d2norm(0.0, 0.0) == 0.0
    assert L.oracle_d2norm(1e300, 1e300) == pytest.approx(np.sqrt(2) * 1e300)


def test_aprod_modes_and_adjoint(pkg, orc):
    prob = pkg.generate("tiny")
    K, D = mats(prob)
    A = sp.vstack([K, D]).tocsr()
    rng = np.random.default_rng(1)
    o = orc.OracleProblem(prob)
    x = rng.standard_normal(prob.n)
    y0 = rng.standard_normal(prob.m_k + prob.m_d)
    o.x[:] = x
    o.y_k[:], o.y_d[:] = y0[:prob.m_k], y0[prob.m_k:]
    o.aprod(1)
    y1 = np.concatenate([o.y_k, o.y_d])
    assert np.allclose(y1, y0 + A @ x, rtol=1e-13, atol=1e-14)
    o.aprod(2)
    assert np.allclose(o.x, x + A.T @ y1, rtol=1e-12, atol=1e-13)
    # <A x, y> = <x, A^T y>
    o2 = orc.OracleProblem(prob)
    o2.x[:] = x
    o2.aprod(1)
    ax = np.concatenate([o2.y_k, o2.y_d])
    o3 = orc.OracleProblem(prob)
    o3.y_k[:], o3.y_d[:] = y0[:prob.m_k], y0[prob.m_k:]
    o3.aprod(2)
    assert ax @ y0 == pytest.approx(x @ o3.x, rel=1e-12)


def test_lsqr_converges_to_normal_equations_solution(pkg, orc):
    prob = pkg.generate("tiny")
    K, D = mats(prob)
    A = sp.vstack([K, D]).toarray()
    b = np.concatenate([prob.b_k, np.zeros(prob.m_d)])
    xs = np.linalg.lstsq(A, b, rcond=None)[0]
    out = orc.OracleProblem(prob).lsqr(300)
    assert np.linalg.norm(out["x"] - xs) <= 1e-9 * np.linalg.norm(xs)
