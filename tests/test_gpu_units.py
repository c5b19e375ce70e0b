"""The unit layout (csrc/units.cuh) on matrices shaped to reach its edge
cases: a single ray, fewer rays than a unit's 32 lines, a ray far longer
than a lane's run (one line over many lanes and slabs), empty rays and
columns, a column count that is not a multiple of the slab, many slabs of
1,024 entries, two blocks per SM.  The FP64 operator against the oracle
(1e-12 of |A||x| + |y|), LSQR against the oracle (1e-10), and the mixed
solver's hi + lo products through a solve that reaches the FP64 solution."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

APROD_TOL = 1e-12
ENVS = [{}, {"PLSQR_SLAB_SIZE": "1024", "PLSQR_UNIT_SIZE_F": "1024"},
        {"PLSQR_UNIT_THREADS": "512", "PLSQR_SLAB_SIZE": "12288", "PLSQR_UNIT_SIZE_F": "12288"}]


def problem(pkg, row_lens, n, seed):
    """Kernel rays with the given entry counts over n columns (ascending
    column order in each ray, values in (0.1, 1)), the identity plus x
    second differences as damping, b = K x_true."""
    S = pkg.synth
    rng = np.random.default_rng(seed)
    rows = [np.sort(rng.choice(n, k, replace=False)) for k in row_lens]
    vals = [rng.uniform(0.1, 1.0, k) for k in row_lens]
    m_k = len(row_lens)
    ptr = np.zeros(m_k + 1, np.int64)
    np.cumsum(row_lens, out=ptr[1:])
    k_csr = S.Lines(ptr, np.concatenate(rows).astype(np.int32) if ptr[-1] else np.zeros(0, np.int32),
                    np.concatenate(vals) if ptr[-1] else np.zeros(0), m_k, n)
    k_csc = k_csr.transposed(by_col=False)
    d_rows, d_vals = [], []
    for c in range(n):
        d_rows.append([c])
        d_vals.append([1.0])
    for c in range(n - 2):
        d_rows.append([c, c + 1, c + 2])
        d_vals.append([0.5, -1.0, 0.5])
    m_d = len(d_rows)
    dptr = np.zeros(m_d + 1, np.int64)
    np.cumsum([len(r) for r in d_rows], out=dptr[1:])
    d_csr = S.Lines(dptr, np.concatenate(d_rows).astype(np.int32), np.concatenate(d_vals), m_d, n)
    d_csc = d_csr.transposed(by_col=False)
    x_true = rng.standard_normal(n)
    b = np.zeros(m_k)
    for r in range(m_k):
        b[r] = np.dot(vals[r], x_true[rows[r]])
    return S.Problem(k_csc, d_csr, d_csc, b, x_true, iterations=30)


SHAPES = {
    "one_ray": ([6000], 7000),
    "33_rays_long_and_empty": ([0, 9000] + [5, 40, 300, 0, 1] * 6 + [2500], 30011),
    "uneven_columns": ([200] * 100 + [20000], 41000),
}


@pytest.mark.parametrize("env", ENVS, ids=["default", "slab1024", "threads512"])
@pytest.mark.parametrize("shape", list(SHAPES))
def test_unit_layout_edges_match_oracle(shape, env, pkg, orc, monkeypatch):
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    row_lens, n = SHAPES[shape]
    prob = problem(pkg, row_lens, n, seed=len(row_lens))
    if shape == "33_rays_long_and_empty":
        assert np.any(np.diff(prob.k_csc.ptr) == 0)  # empty columns too
    rng = np.random.default_rng(7)
    o = orc.OracleProblem(prob)
    with pkg.Context(prob) as ctx:
        for mode in (1, 2):
            yk, yd = rng.standard_normal(prob.m_k), rng.standard_normal(prob.m_d)
            x = rng.standard_normal(prob.n)
            o.y_k[:], o.y_d[:], o.x[:] = yk, yd, x
            o.aprod(mode)
            gyk, gyd, gx = yk.copy(), yd.copy(), x.copy()
            ctx.aprod_host(mode, gyk, gyd, gx)
            if mode == 1:
                err = np.abs(np.concatenate([gyk - o.y_k, gyd - o.y_d]))
                kabs = np.array([np.abs(prob.k_csc.val[prob.k_csc.idx == r]).sum() for r in range(prob.m_k)])
                scale = np.concatenate([kabs * np.max(np.abs(x)), np.full(prob.m_d, 2.0 * np.max(np.abs(x)))])
                scale += np.abs(np.concatenate([yk, yd]))
            else:
                err = np.abs(gx - o.x)
                cabs = np.diff(np.concatenate([[0.0], np.cumsum(np.abs(prob.k_csc.val))])[prob.k_csc.ptr])
                scale = cabs * np.max(np.abs(yk)) + 3.0 * np.max(np.abs(yd)) + np.abs(x)
            assert np.all(err <= APROD_TOL * scale + 1e-300), (mode, float(np.max(err / scale)))
        out = ctx.lsqr(lsqr_iteration=150)
    # x once converged (by ~100 iterations on these problems; before that a
    # one-ulp raise of the kernel values moves the oracle's own x_30 by up to
    # 3e-6)
    ref = orc.OracleProblem(prob).lsqr(150)
    assert rel(out["x"], ref["x"]) <= 1e-10
    # per-iteration scalars: iterations 0-3 only.  These problems lose their
    # alpha_k to any change of rounding from iteration 4-5 on: raising every
    # kernel value by one ulp moves the oracle's own alpha_4 by 2e-9 on the
    # one-ray problem and alpha_5 by 3e-7 on the 101-ray one, and a
    # different summation order moves them more (x, above, stays).
    dev = np.abs(out["hist"]["alpha"][:4] - ref["hist"]["alpha"][:4]) / np.abs(ref["hist"]["alpha"][:4])
    assert np.max(dev) <= 1e-10, dev


@pytest.mark.parametrize("env", ENVS, ids=["default", "slab1024", "threads512"])
def test_mixed_hilo_products_on_edge_shapes(env, pkg, monkeypatch):
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    row_lens, n = SHAPES["33_rays_long_and_empty"]
    prob = problem(pkg, row_lens, n, seed=5)
    with pkg.Context(prob) as c64:
        xs = c64.lsqr(lsqr_iteration=300)["x"]
        h64 = c64.lsqr(lsqr_iteration=5)["hist"]
    with pkg.Context(prob, precision="mixed") as cm:
        hm = cm.lsqr(sweeps=1, inner=5)["hist"]
        out = cm.lsqr(sweeps=3, inner=150)
    # the first iterations follow FP64 to the FP32 rounding of the values
    for key in ("alpha", "beta"):
        assert np.max(np.abs(hm[key] - h64[key]) / np.abs(h64[key])) <= 1e-5, key
    assert rel(out["x"], xs) <= 1e-6
