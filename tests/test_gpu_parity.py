"""Parity of the GB300 path (through the C ABI) with the reference.

Tolerances: the FP64 path must reproduce the reference's x and the
per-iteration alpha, beta, rnorm, arnorm within 1e-10 relative (the
parity bar of the FP64 path); a single aprod must match the oracle within 1e-12 of
(|A| |x| + |y|) per element (the GPU sums a row in a different order)."""
from __future__ import annotations

import re
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

from conftest import GOLDEN, golden, rel

pytestmark = pytest.mark.gpu

LSQR_TOL = 1e-10
APROD_TOL = 1e-12


def per_iter_rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.size == 0:
        return 0.0
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def scipy_ops(prob):
    K = sp.csc_matrix((prob.k_csc.val, prob.k_csc.idx, prob.k_csc.ptr), shape=(prob.m_k, prob.n))
    D = sp.csr_matrix((prob.d_csr.val, prob.d_csr.idx, prob.d_csr.ptr), shape=(prob.m_d, prob.n))
    return sp.vstack([K, D]).tocsr()


@pytest.mark.parametrize("case", ["tiny", "grid32"])
def test_lsqr_fp64_matches_reference(case, pkg, orc, problems, tmp_path):
    g = golden(case)
    prob = problems(case)
    it = g["meta"]["iterations"]
    with pkg.Context(prob) as ctx:
        out = ctx.lsqr(lsqr_iteration=it, result_txt=str(tmp_path / "result.txt"))
    assert rel(out["x"], g["x"]) <= LSQR_TOL
    assert per_iter_rel(out["hist"]["alpha"], g["alpha"]) <= LSQR_TOL
    assert per_iter_rel(out["hist"]["beta"], g["beta"]) <= LSQR_TOL
    ref = orc.OracleProblem(prob).lsqr(it)  # bitwise equal to the reference (CPU tests)
    for k in ("rnorm", "arnorm", "anorm", "xnorm", "test1", "test2"):
        assert per_iter_rel(out["hist"][k][1:], ref["hist"][k][1:]) <= LSQR_TOL, k
    r = out["result"]
    for k in ("rnorm", "xnorm", "anorm", "arnorm_out"):
        assert abs(r[k] - ref["result"][k]) <= LSQR_TOL * abs(ref["result"][k]), k
    assert r["istop"] == ref["result"]["istop"] and r["itn"] == it
    # result.txt: same lines; numbers equal to the printed precision
    mine = (tmp_path / "result.txt").read_text().splitlines()
    theirs = g["result_txt"].splitlines()
    assert len(mine) == len(theirs)
    num = re.compile(r"[-+]?\d+\.\d+e[-+]\d+")
    for a, b in zip(mine, theirs):
        assert num.sub("#", a) == num.sub("#", b)
        for x, y in zip(num.findall(a), num.findall(b)):
            assert abs(float(x) - float(y)) <= 1e-6 * abs(float(y)) + 1e-300, (a, b)


@pytest.mark.parametrize("case", ["tiny", "grid32"])
def test_aprod_matches_oracle(case, pkg, orc, problems):
    prob = problems(case)
    rng = np.random.default_rng(3)
    A = scipy_ops(prob)
    absA = abs(A)
    with pkg.Context(prob) as ctx:
        for mode in (1, 2):
            yk, yd = rng.standard_normal(prob.m_k), rng.standard_normal(prob.m_d)
            x = rng.standard_normal(prob.n)
            o = orc.OracleProblem(prob)
            o.y_k[:], o.y_d[:], o.x[:] = yk, yd, x
            o.aprod(mode)
            gyk, gyd, gx = yk.copy(), yd.copy(), x.copy()
            ctx.aprod_host(mode, gyk, gyd, gx)
            if mode == 1:
                scale = absA @ np.abs(x) + np.abs(np.concatenate([yk, yd]))
                err = np.abs(np.concatenate([gyk - o.y_k, gyd - o.y_d]))
                assert np.array_equal(gx, x)
            else:
                scale = absA.T @ np.abs(np.concatenate([yk, yd])) + np.abs(x)
                err = np.abs(gx - o.x)
                assert np.array_equal(gyk, yk) and np.array_equal(gyd, yd)
            assert np.all(err <= APROD_TOL * scale + 1e-300), (mode, float(np.max(err / scale)))


def test_aprod_device_vectors_and_damping_order(pkg, orc, problems):
    """Device-resident aprod; the damping part is summed in the reference's
    order, so with a zero kernel part it is bitwise equal."""
    prob = problems("tiny")
    rng = np.random.default_rng(5)
    x = rng.standard_normal(prob.n)
    with pkg.Context(prob) as ctx:
        ctx.set_u(np.zeros(prob.m_k), np.zeros(prob.m_d))
        ctx.set_v(x)
        ctx.aprod(1)
        yk, yd = ctx.get_u()
    o = orc.OracleProblem(prob)
    o.x[:] = x
    o.aprod(1)
    assert np.array_equal(yd, o.y_d)
    assert rel(yk, o.y_k) <= 1e-14


def test_adjoint_identity(pkg, problems):
    prob = problems("grid32")
    rng = np.random.default_rng(9)
    x = rng.standard_normal(prob.n)
    yk, yd = rng.standard_normal(prob.m_k), rng.standard_normal(prob.m_d)
    with pkg.Context(prob) as ctx:
        ax_k, ax_d, v = np.zeros(prob.m_k), np.zeros(prob.m_d), x.copy()
        ctx.aprod_host(1, ax_k, ax_d, v)
        aty = np.zeros(prob.n)
        ctx.aprod_host(2, yk.copy(), yd.copy(), aty)
    lhs = ax_k @ yk + ax_d @ yd
    rhs = x @ aty
    assert abs(lhs - rhs) <= 1e-12 * (np.abs(ax_k) @ np.abs(yk) + np.abs(ax_d) @ np.abs(yd))


def test_visit_order_changes_only_rounding(pkg, problems):
    prob = problems("grid32")
    with pkg.Context(prob) as c1, pkg.Context(prob, grid=(0, 0, 0)) as c2:
        a, b = c1.lsqr(lsqr_iteration=60), c2.lsqr(lsqr_iteration=60)
    assert rel(a["x"], b["x"]) <= 1e-12


def test_graph_replay_equals_stream_launch_and_is_deterministic(pkg, problems):
    prob = problems("grid32")
    outs = []
    for graph in (True, False, True):
        with pkg.Context(prob, use_graph=graph) as ctx:
            outs.append(ctx.lsqr(lsqr_iteration=30))
    for o in outs[1:]:
        assert np.array_equal(o["x"], outs[0]["x"])
        assert np.array_equal(o["hist"]["alpha"], outs[0]["hist"]["alpha"])


def test_context_from_files_equals_context_from_arrays(pkg, problems):
    g = golden("tiny")
    files = dict(g["meta"]["files"], dir=str(GOLDEN / "tiny" / "inputs"))
    it = g["meta"]["iterations"]
    with pkg.Context(files=files) as c1:
        a = c1.lsqr(lsqr_iteration=it)
        assert np.array_equal(c1.get_b(), problems("tiny").b_k)
    # same column visit order as the file-loaded context (no grid known)
    with pkg.Context(problems("tiny"), grid=(0, 0, 0)) as c2:
        b = c2.lsqr(lsqr_iteration=it)
    assert np.array_equal(a["x"], b["x"])
    assert rel(a["x"], g["x"]) <= LSQR_TOL


def test_repeated_solves_reuse_the_context(pkg, problems):
    prob = problems("tiny")
    with pkg.Context(prob) as ctx:
        a = ctx.lsqr(lsqr_iteration=20)
        b = ctx.lsqr(lsqr_iteration=40)
        c = ctx.lsqr(lsqr_iteration=20)
    assert np.array_equal(a["x"], c["x"])
    assert np.array_equal(a["hist"]["beta"], b["hist"]["beta"][:21])


@pytest.mark.parametrize("variant", ["damped", "want_se", "zero_rhs", "sparse_rays", "one_iter",
                                     "zero_iter"])
def test_lsqr_edge_cases_match_oracle(variant, pkg, orc, problems):
    prob = problems("tiny")
    kw = dict(damp=0.0, want_se=False)
    b = None
    it = 15
    if variant == "damped":
        kw["damp"] = 0.3
    elif variant == "want_se":
        kw["want_se"] = True
    elif variant == "zero_rhs":
        b = np.zeros(prob.m_k)
    elif variant == "sparse_rays":
        # thin tubes: empty kernel rows, empty columns, 1-3 nonzero rows
        prob = pkg.generate("tiny", tube_radius=0.45, n_rays=80)
        assert np.any(np.diff(prob.k_csc.ptr) == 0)
    elif variant == "one_iter":
        it = 1
    elif variant == "zero_iter":
        it = 0
    with pkg.Context(prob) as ctx:
        g = ctx.lsqr(b, lsqr_iteration=it, **kw)
    r = orc.OracleProblem(prob).lsqr(it, b_k=b, **kw)
    assert np.all(np.isfinite(g["x"]))
    if variant == "zero_rhs":
        assert np.array_equal(g["x"], np.zeros(prob.n)) and g["hist"]["beta"][0] == 0.0
        assert g["result"]["itn"] == 0 and r["result"]["itn"] == 0
        return
    assert rel(g["x"], r["x"]) <= LSQR_TOL
    assert per_iter_rel(g["hist"]["alpha"], r["hist"]["alpha"]) <= LSQR_TOL
    assert per_iter_rel(g["hist"]["rnorm"][1:], r["hist"]["rnorm"][1:]) <= LSQR_TOL
    if kw["want_se"]:
        assert rel(g["se"], r["se"]) <= LSQR_TOL


def test_cli_program_matches_reference_outputs(pkg, tmp_path):
    g = golden("tiny")
    f = g["meta"]["files"]
    exe = pkg._native.LIB_DIR / "plsqr3_gpu"
    it = g["meta"]["iterations"]
    cmd = [str(exe), "-dir", str(GOLDEN / "tiny" / "inputs"), "-quiet"]
    for k in ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol", "damp_i_bycol", "b_k"):
        cmd += [f"-{k}", f[k]]
    cmd += ["-row_k", str(f["row_k"]), "-row_d", str(f["row_d"]), "-col", str(f["col"]),
            "-itn", str(it)]
    subprocess.run(cmd, cwd=tmp_path, check=True, capture_output=True)
    x = np.fromfile(tmp_path / f"p_resultx_itn={it}_NProc=1_float64_mpiio.bin", dtype=np.float64)
    assert rel(x, g["x"]) <= LSQR_TOL
    assert (tmp_path / "result.txt").read_text().splitlines()[0] == g["result_txt"].splitlines()[0]


def test_mixed_precision_reaches_1e6_of_fp64_solution(pkg, problems):
    prob = problems("grid32")
    with pkg.Context(prob) as c64:
        xstar = c64.lsqr(lsqr_iteration=400)["x"]
    with pkg.Context(prob, precision="mixed") as cm:
        cm.set_reference_x(xstar)
        out = cm.lsqr(sweeps=5, inner=60)
    err = out["hist"]["err"]
    assert err[0] == 1.0
    assert rel(out["x"], xstar) <= 1e-6
    assert abs(err[-1] - rel(out["x"], xstar)) <= 1e-3 * err[-1] + 1e-12


def test_mixed_precision_refuses_damped_refinement(pkg, problems):
    """A refinement sweep regularises the correction, not the solution, so a
    damped solve allows one sweep only."""
    prob = problems("grid32")
    with pkg.Context(prob, precision="mixed") as cm:
        with pytest.raises(pkg._native.PlsqrError) as e:
            cm.lsqr(damp=0.1, sweeps=2, inner=10)
        assert e.value.code == -1
        out = cm.lsqr(damp=0.1, sweeps=1, inner=10)
        assert np.all(np.isfinite(out["x"]))


def test_mixed_precision_warm_start(pkg, problems):
    """x0 near the solution is kept and saves iterations; an x0 that raises
    the residual falls back to the cold start, bit for bit; the FP64 path and
    damped solves refuse x0."""
    prob = problems("grid32")
    with pkg.Context(prob) as c64:
        xstar = c64.lsqr(lsqr_iteration=400)["x"]
        with pytest.raises(pkg._native.PlsqrError) as e:
            c64.lsqr(lsqr_iteration=5, x0=xstar)
        assert e.value.code == -1
    rng = np.random.default_rng(3)
    with pkg.Context(prob, precision="mixed") as cm:
        cm.set_reference_x(xstar)
        cold = cm.lsqr(sweeps=2, inner=200)
        x0 = xstar + 1e-3 * np.linalg.norm(xstar) / np.sqrt(prob.n) * rng.standard_normal(prob.n)
        warm = cm.lsqr(sweeps=2, inner=200, x0=x0)
        assert cold["result"]["warm"] == 0 and warm["result"]["warm"] == 1
        assert abs(warm["hist"]["err"][0] - rel(x0, xstar)) <= 1e-12
        k_cold = int(np.argmax(cold["hist"]["err"] <= 1e-6))
        k_warm = int(np.argmax(warm["hist"]["err"] <= 1e-6))
        assert 0 < k_warm < k_cold
        bad = cm.lsqr(sweeps=2, inner=200, x0=1e6 * rng.standard_normal(prob.n))
        assert bad["result"]["warm"] == 0
        assert np.array_equal(bad["x"], cold["x"])
        assert np.array_equal(bad["hist"]["err"], cold["hist"]["err"])
        with pytest.raises(pkg._native.PlsqrError) as e:
            cm.lsqr(damp=0.1, sweeps=1, inner=10, x0=x0)
        assert e.value.code == -1


def test_cli_warm_start_from_a_solution_file(pkg, problems, tmp_path):
    """-x0 FILE (the program's own float64 solution format) starts the mixed
    solver from that solution, which it keeps and does not make worse in the
    least-squares residual; the FP64 path refuses it."""
    g = golden("tiny")
    f = g["meta"]["files"]
    exe = pkg._native.LIB_DIR / "plsqr3_gpu"
    it = g["meta"]["iterations"]
    base = [str(exe), "-dir", str(GOLDEN / "tiny" / "inputs"), "-quiet"]
    for k in ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol", "damp_i_bycol", "b_k"):
        base += [f"-{k}", f[k]]
    base += ["-row_k", str(f["row_k"]), "-row_d", str(f["row_d"]), "-col", str(f["col"]),
             "-itn", str(it)]
    out = tmp_path / f"p_resultx_itn={it}_NProc=1_float64_mpiio.bin"
    subprocess.run(base, cwd=tmp_path, check=True, capture_output=True)
    x0 = tmp_path / "x0.bin"
    x0.write_bytes(out.read_bytes())
    mixed = base + ["-precision", "mixed", "-sweeps", "1", "-inner", "20", "-x0", str(x0)]
    p = subprocess.run(mixed, cwd=tmp_path, check=True, capture_output=True, text=True)
    assert "x0 kept" in p.stdout
    prob = problems("tiny")
    A = scipy_ops(prob)
    b = np.concatenate([prob.b_k, np.zeros(prob.m_d)])
    r0 = np.linalg.norm(b - A @ np.fromfile(x0, dtype=np.float64))
    r1 = np.linalg.norm(b - A @ np.fromfile(out, dtype=np.float64))
    assert np.isfinite(r1) and r1 <= r0 * (1 + 1e-9)
    p = subprocess.run(base + ["-x0", str(x0)], cwd=tmp_path, capture_output=True, text=True)
    assert p.returncode != 0 and "mixed-precision" in p.stderr


def test_rhs_magnitudes_scale_and_out_of_range_is_refused(pkg, problems):
    """Scaling b by 2^480 or 2^-480 scales x by the same power of two (the
    sums of squares of the norms still hold the values); beyond 2^500, or
    with every entry below 2^-500, the solve is refused with
    PLSQR_ERR_NUMERIC instead of running on an overflowed norm."""
    prob = problems("tiny")
    with pkg.Context(prob) as ctx:
        ref = ctx.lsqr(lsqr_iteration=15)["x"]
        for f in (2.0 ** 480, 2.0 ** -480):
            x = ctx.lsqr(prob.b_k * f, lsqr_iteration=15)["x"]
            assert rel(x / f, ref) <= 1e-13
        for f in (2.0 ** 520, 2.0 ** -560):
            with pytest.raises(pkg._native.PlsqrError) as e:
                ctx.lsqr(prob.b_k * f, lsqr_iteration=15)
            assert e.value.code == -10
