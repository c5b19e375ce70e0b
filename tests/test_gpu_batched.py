"""Batched right-hand sides (Context.batch_lsqr): k solves in lock step on one
operator, one k-wide product per matrix read.

There is no batched solver in the reference; the yardstick of every solve is
the FP64 one-right-hand-side path (itself pinned to the reference), run on the
same instance with the same damping weight."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def grid32(pkg, problems):
    prob = problems("grid32")
    with pkg.Context(prob) as ctx:
        insts = pkg.batch.instances(ctx, prob, "grid32")
    return prob, insts


def fp64_solution(pkg, prob, inst, iterations):
    with pkg.Context(prob) as c:
        if inst.lam != 1.0:
            c.set_damping_weight(inst.lam)
        return c.lsqr(inst.b_k, lsqr_iteration=iterations)


def test_instances_reach_their_fp64_solutions(pkg, grid32):
    prob, insts = grid32
    sel = pkg.batch.pick(insts, 6)
    assert {i.name[:5] for i in sel} == {"noise", "lambd", "check"}
    xstar = np.stack([fp64_solution(pkg, prob, i, 800)["x"] for i in sel])
    with pkg.Context(prob) as ctx:
        out = ctx.batch_lsqr(np.stack([i.b_k for i in sel]), lam=[i.lam for i in sel],
                             x_ref=xstar, sweeps=5, inner=60)
    for j, inst in enumerate(sel):
        e = rel(out["x"][j], xstar[j])
        assert e <= 1e-6, (inst.name, e)
        err = out["hist"]["err"][j]
        assert err[0] == 1.0
        assert abs(err[-1] - e) <= 1e-3 * e + 1e-12, inst.name


def test_columns_are_independent(pkg, grid32):
    """A right-hand side gives the same bits alone and in a batch of the same
    block width and product variants."""
    prob, insts = grid32
    sel = [insts[0], insts[16], insts[24]]
    b = np.stack([i.b_k for i in sel])
    lam = [i.lam for i in sel]
    kw = dict(sweeps=2, inner=10, variant_rows=1, variant_cols=1)
    with pkg.Context(prob) as ctx:
        both = ctx.batch_lsqr(b, lam=lam, **kw)
        for j in range(3):
            one = ctx.batch_lsqr(b[j:j + 1], lam=lam[j:j + 1], **kw)
            assert np.array_equal(one["x"][0], both["x"][j])
            assert np.array_equal(one["hist"][0], both["hist"][j])


def test_start_and_first_iteration_match_fp64(pkg, grid32):
    prob, insts = grid32
    sel = [insts[1], insts[20], insts[27]]
    with pkg.Context(prob) as ctx:
        out = ctx.batch_lsqr(np.stack([i.b_k for i in sel]), lam=[i.lam for i in sel],
                             sweeps=1, inner=3)
    for j, inst in enumerate(sel):
        h64 = fp64_solution(pkg, prob, inst, 3)["hist"]
        h = out["hist"][j]
        assert h["beta"][0] == pytest.approx(np.linalg.norm(inst.b_k), rel=1e-14)
        # FP32 kernel products: alpha and beta agree to FP32 accuracy
        for f in ("alpha", "beta", "rnorm", "arnorm"):
            assert np.allclose(h[f][:4], h64[f][:4], rtol=2e-5, atol=0), (inst.name, f)


@pytest.mark.parametrize("k", [4, 32])
def test_every_variant_gives_the_same_iterates(pkg, grid32, k):
    prob, insts = grid32
    sel = pkg.batch.pick(insts, k)
    b = np.stack([i.b_k for i in sel])
    lam = [i.lam for i in sel]
    kw = 4 if k <= 4 else 32
    ok = []
    for v in range(64):
        try:
            vw, lpr, u = pkg._native.batch_variant(v)
        except pkg._native.PlsqrError:
            break
        # lpr 0: slab form; lpr -1: units form (passes of 4 or 8 columns)
        if lpr <= 0 or (kw % vw == 0 and kw // vw <= lpr):
            ok.append(v)
    assert len(ok) >= 7
    with pkg.Context(prob) as ctx:
        ref = ctx.batch_lsqr(b, lam=lam, sweeps=1, inner=6, variant_rows=ok[0],
                             variant_cols=ok[0])
        for v in ok[1:]:
            out = ctx.batch_lsqr(b, lam=lam, sweeps=1, inner=6, variant_rows=v, variant_cols=v)
            for f in ("alpha", "beta", "rnorm"):
                assert np.allclose(out["hist"][f], ref["hist"][f], rtol=2e-5, atol=0), (v, f)
            assert rel(out["x"], ref["x"]) <= 1e-4


def test_tuning_is_cached_and_bench_runs(pkg, grid32):
    prob, insts = grid32
    # 12 right-hand sides: a block width (16) no other test here uses, so the
    # process-wide choice is not cached yet
    b = np.stack([i.b_k for i in insts[:12]])
    with pkg.Context(prob) as ctx:
        first = ctx.batch_lsqr(b, sweeps=1, inner=2)
        assert first["info"]["tuned"] == 1 and first["info"]["kp"] == 16
        assert first["info"]["ms_rows"] > 0 and first["info"]["ms_cols"] > 0
        again = ctx.batch_lsqr(b, sweeps=1, inner=2)
        assert again["info"]["tuned"] == 0
        assert again["info"]["variant_rows"] == first["info"]["variant_rows"]
        assert np.array_equal(again["x"], first["x"])
        for mode in (1, 2):
            assert ctx.batch_bench_aprod(12, mode, reps=2) > 0


def test_zero_right_hand_side_stays_zero(pkg, grid32):
    prob, insts = grid32
    b = np.stack([insts[0].b_k, np.zeros(prob.m_k), insts[24].b_k])
    with pkg.Context(prob) as ctx:
        out = ctx.batch_lsqr(b, sweeps=2, inner=20)
        alone = ctx.batch_lsqr(b[[0, 2]], sweeps=2, inner=20, variant_rows=out["info"][
            "variant_rows"], variant_cols=out["info"]["variant_cols"])
    assert np.all(out["x"][1] == 0.0)
    assert np.all(np.isfinite(out["hist"]["rnorm"]))
    assert np.array_equal(out["x"][[0, 2]], alone["x"])


def test_batch_arguments_are_checked(pkg, grid32):
    prob, insts = grid32
    with pkg.Context(prob) as ctx:
        for bad in (dict(b_k=np.zeros((33, prob.m_k))), dict(b_k=np.zeros((2, prob.m_k)),
                                                            sweeps=0),
                    dict(b_k=np.zeros((2, prob.m_k)), variant_rows=99),
                    dict(b_k=np.zeros((2, prob.m_k)), lam=[1.0, -1.0]),
                    dict(b_k=np.zeros((2, prob.m_k)), damp=0.1, sweeps=2)):
            b = bad.pop("b_k")
            with pytest.raises(pkg._native.PlsqrError) as e:
                ctx.batch_lsqr(b, **bad)
            assert e.value.code == -1
        # a variant too narrow for the block: float2 gathers of 32 columns on
        # 8 lanes
        narrow = [v for v in range(13) if pkg._native.batch_variant(v) == (2, 8, 2)]
        with pytest.raises(pkg._native.PlsqrError):
            ctx.batch_lsqr(np.zeros((32, prob.m_k)), variant_rows=narrow[0])


def test_damping_weight_round_trip(pkg, problems):
    prob = problems("grid32")
    with pkg.Context(prob) as c:
        ref = c.lsqr(lsqr_iteration=20)
        c.set_damping_weight(3.0)
        w3 = c.lsqr(lsqr_iteration=20)
        c.set_damping_weight(1.0)
        back = c.lsqr(lsqr_iteration=20)
    assert np.array_equal(ref["x"], back["x"])
    assert not np.array_equal(ref["x"], w3["x"])


def test_warm_start_and_cold_fallback(pkg, grid32):
    """x0 near the solution is kept and saves iterations; an x0 that does not
    lower the residual falls back to the cold start, bit for bit."""
    prob, insts = grid32
    sel = [insts[0], insts[24]]
    b = np.stack([i.b_k for i in sel])
    xstar = np.stack([fp64_solution(pkg, prob, i, 800)["x"] for i in sel])
    rng = np.random.default_rng(5)
    near = xstar * (1.0 + 0.01 * rng.standard_normal(xstar.shape))
    far = 100.0 * rng.standard_normal(xstar.shape)
    kw = dict(x_ref=xstar, sweeps=3, inner=60, variant_rows=1, variant_cols=1)
    with pkg.Context(prob) as ctx:
        cold = ctx.batch_lsqr(b, **kw)
        warm = ctx.batch_lsqr(b, x0=near, **kw)
        back = ctx.batch_lsqr(b, x0=np.stack([near[0], far[1]]), **kw)
    assert cold["info"]["warm"] == 0 and warm["info"]["warm"] == 0b11
    assert back["info"]["warm"] == 0b01
    for j in range(2):
        e_cold, e_warm = cold["hist"]["err"][j], warm["hist"]["err"][j]
        assert e_warm[0] == pytest.approx(rel(near[j], xstar[j]), rel=1e-12)
        assert rel(warm["x"][j], xstar[j]) <= 1e-6
        k_cold = int(np.argmax(e_cold <= 1e-6))
        k_warm = int(np.argmax(e_warm <= 1e-6))
        assert e_warm[k_warm] <= 1e-6 and k_warm < k_cold
    # the far start fell back: the same bits as the cold solve
    assert np.array_equal(back["x"][1], cold["x"][1])
    assert np.array_equal(back["x"][0], warm["x"][0])


def units_variant(pkg):
    for v in range(64):
        try:
            if pkg._native.batch_variant(v)[1] < 0:
                return v
        except pkg._native.PlsqrError:
            break
    raise AssertionError("no units form among the product variants")


@pytest.mark.parametrize("k", [3, 8, 20])
def test_units_form_matches_team_form(pkg, grid32, k):
    """The units form (FP32 unit layout, the block's rows staged per slab in
    shared memory; a block of 20 in passes of 8 columns, the last one partly
    padding) gives the team form's iterates to FP32 accuracy, reaches the
    FP64 solutions, and a right-hand side gives the same bits alone and
    inside a block of the same width."""
    prob, insts = grid32
    sel = pkg.batch.pick(insts, k)
    b = np.stack([i.b_k for i in sel])
    lam = [i.lam for i in sel]
    vu = units_variant(pkg)
    xstar = np.stack([fp64_solution(pkg, prob, i, 800)["x"] for i in sel])
    with pkg.Context(prob) as ctx:
        team = ctx.batch_lsqr(b, lam=lam, sweeps=1, inner=6, variant_rows=1, variant_cols=1)
        unit = ctx.batch_lsqr(b, lam=lam, sweeps=1, inner=6, variant_rows=vu, variant_cols=vu)
        assert unit["info"]["variant_rows"] == vu and unit["info"]["variant_cols"] == vu
        for f in ("alpha", "beta", "rnorm"):
            assert np.allclose(unit["hist"][f], team["hist"][f], rtol=2e-5, atol=0), f
        assert rel(unit["x"], team["x"]) <= 1e-4
        full = ctx.batch_lsqr(b, lam=lam, x_ref=xstar, sweeps=5, inner=60, variant_rows=vu,
                              variant_cols=vu)
        for j in range(k):
            assert rel(full["x"][j], xstar[j]) <= 1e-6, sel[j].name
        if k == 3:  # width 4 either way: the first right-hand side alone
            one = ctx.batch_lsqr(b[:1], lam=lam[:1], sweeps=1, inner=6, variant_rows=vu,
                                 variant_cols=vu)
            assert np.array_equal(one["x"][0], unit["x"][0])
            assert np.array_equal(one["hist"][0], unit["hist"][0])


def first_at_or_below(err, tol, start=1):
    idx = np.nonzero(err[start:] <= tol)[0]
    return None if idx.size == 0 else int(idx[0]) + start


def test_retirement_on_error_packs_the_rest(pkg, grid32):
    """retire_every / retire_err: every R iterations the right-hand sides
    within retire_err of x_ref leave with x = X + DX and their state, the
    others go on in a narrower block.  Up to the first retirement the run is
    the lock-step run bit for bit; every retiree is within the tolerance at
    its retirement and was not at the check before; the ones that never get
    there end where the lock-step run ends, to the rounding of the narrower
    blocks' products."""
    prob, insts = grid32
    # the 32 instances come within 1e-5 between iterations 73 and 80: a check
    # every iteration retires them over several checks, packing 32 -> 16 -> 8
    # -> 4
    tol, R, inner = 1e-5, 1, 600
    b = np.stack([i.b_k for i in insts])
    lam = [i.lam for i in insts]
    xstar = np.stack([fp64_solution(pkg, prob, i, 800)["x"] for i in insts])
    kw = dict(lam=lam, x_ref=xstar, sweeps=1, inner=inner, variant_rows=1, variant_cols=1)
    with pkg.Context(prob) as ctx:
        lock = ctx.batch_lsqr(b, **kw)
        ret = ctx.batch_lsqr(b, retire_every=R, retire_err=tol, **kw)
    err_l, err_r = lock["hist"]["err"], ret["hist"]["err"]
    ks = [first_at_or_below(err_l[j], tol) for j in range(len(insts))]
    reached = [j for j, k in enumerate(ks) if k is not None and k < inner - 2 * R]
    assert len(reached) >= 16
    t1 = min(-(-ks[j] // R) * R for j in reached)
    assert np.array_equal(ret["hist"][:, :t1 + 1], lock["hist"][:, :t1 + 1])
    itns = [r["itn"] for r in ret["results"]]
    left_at = set()
    for j in range(len(insts)):
        it = itns[j]
        if err_l[j][t1] <= tol:
            assert it == t1, (insts[j].name, it, t1)
        if it < inner:
            left_at.add(it)
            assert it % R == 0
            assert err_r[j][it] <= tol
            if it > R:
                assert err_r[j][it - R] > tol
            assert rel(ret["x"][j], xstar[j]) <= tol * (1 + 1e-9)
            assert np.all(ret["hist"][j][it + 1:]["beta"] == 0.0)
        else:
            e_l, e_r = err_l[j][inner], err_r[j][inner]
            assert abs(e_r - e_l) <= 0.1 * e_l, (insts[j].name, e_l, e_r)
            assert rel(ret["x"][j], xstar[j]) == pytest.approx(e_r, rel=1e-6)
    # retirements at several checks: the block was packed more than once
    assert len(left_at) >= 3
    assert ret["results"][0]["seconds"] > 0
    assert ret["info"]["k"] == len(insts) and ret["info"]["kp"] == 32


def test_retirement_on_lsqr_stop(pkg, grid32):
    """Without x_ref a right-hand side retires on LSQR's own stopping test
    (istop != 0) in the last sweep; the retirees' results carry that istop
    and the iteration they left at.  (conlim = 0: no condition-number stop,
    which at the default conlim = 100 would end these solves at once.)"""
    prob, insts = grid32
    sel = pkg.batch.pick(insts, 8)
    b = np.stack([i.b_k for i in sel])
    R, inner = 8, 800
    kw = dict(lam=[i.lam for i in sel], sweeps=1, inner=inner, atol=1e-5, btol=1e-5,
              conlim=0.0, variant_rows=1, variant_cols=1)
    with pkg.Context(prob) as ctx:
        lock = ctx.batch_lsqr(b, **kw)
        ret = ctx.batch_lsqr(b, retire_every=R, **kw)
    stop = []
    for j in range(len(sel)):
        nz = np.nonzero(lock["hist"]["istop"][j][1:])[0]
        stop.append(int(nz[0]) + 1 if nz.size else None)
    stopped = [j for j, s0 in enumerate(stop) if s0 is not None and s0 < inner - 2 * R]
    assert len(stopped) >= 4, stop
    t1 = min(-(-stop[j] // R) * R for j in stopped)
    assert np.array_equal(ret["hist"][:, :t1 + 1], lock["hist"][:, :t1 + 1])
    for j in range(len(sel)):
        r = ret["results"][j]
        if r["itn"] == inner:
            assert j not in stopped or -(-stop[j] // R) * R != t1
            continue
        assert r["istop"] != 0 and r["itn"] % R == 0, (sel[j].name, r)
        assert ret["hist"]["istop"][j][r["itn"]] != 0
        if r["itn"] > R:
            assert ret["hist"]["istop"][j][r["itn"] - R] == 0
        if stop[j] is not None and -(-stop[j] // R) * R == t1:
            assert r["itn"] == t1
    if all(r["itn"] < inner for r in ret["results"]):
        # everything retired before the limit: less device time
        assert ret["results"][0]["seconds"] < lock["results"][0]["seconds"]


def test_retirement_across_sweeps(pkg, grid32):
    """Error retirement in any refinement sweep: a retiree's x is X + DX of
    its sweep, the rest go on through the following sweeps."""
    prob, insts = grid32
    sel = pkg.batch.pick(insts, 12)
    tol = 3e-6
    xstar = np.stack([fp64_solution(pkg, prob, i, 800)["x"] for i in sel])
    kw = dict(lam=[i.lam for i in sel], x_ref=xstar, sweeps=4, inner=60, variant_rows=1,
              variant_cols=1)
    b = np.stack([i.b_k for i in sel])
    with pkg.Context(prob) as ctx:
        lock = ctx.batch_lsqr(b, **kw)
        ret = ctx.batch_lsqr(b, retire_every=15, retire_err=tol, **kw)
        with pytest.raises(pkg._native.PlsqrError):
            ctx.batch_lsqr(b, retire_every=-1, **kw)
        with pytest.raises(pkg._native.PlsqrError):
            ctx.batch_lsqr(b, retire_every=5, retire_err=-1.0, **kw)
        with pytest.raises(pkg._native.PlsqrError):
            ctx.batch_lsqr(b, retire_every=5, retire_err=1e-6, sweeps=1, inner=10)
    for j in range(len(sel)):
        it = ret["results"][j]["itn"]
        e = rel(ret["x"][j], xstar[j])
        if it < 240:
            assert e <= tol * (1 + 1e-9), (sel[j].name, it, e)
            assert ret["hist"]["err"][j][it] <= tol
        else:
            e_l = rel(lock["x"][j], xstar[j])
            assert abs(e - e_l) <= 0.1 * e_l + 1e-9, (sel[j].name, e, e_l)
    assert min(r["itn"] for r in ret["results"]) < 240
