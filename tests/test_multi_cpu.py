"""Host side of the persistent multi-problem launch: the 24-problem set and
the block planner (no GPU)."""
from __future__ import annotations

import numpy as np


def test_uneven_set(pkg):
    cfgs = pkg.multi.uneven_configs()
    assert len(cfgs) == 24
    sides = [c["nx"] for c in cfgs]
    rays = sorted(c["n_rays"] for c in cfgs)
    assert sides[0] == 16 and sides[-1] == 64 and sides == sorted(sides)
    assert rays[0] == 500 and rays[-1] == 20000 and len(set(rays)) == 24
    # grid size and ray count do not grow together
    r = [c["n_rays"] for c in cfgs]
    assert np.corrcoef(sides, r)[0, 1] < 0.9
    assert all(c["tube_radius"] == 1.5 and c["iterations"] == 100 for c in cfgs)
    assert len({c["seed"] for c in cfgs}) == 24


def test_plan_gives_big_problems_more_blocks(pkg):
    work = np.array([1e6, 1e8, 1e7, 1e5])
    group, gb = pkg.multi.plan_host(work, [100] * 4, blocks=64, bw_block=6e12 / 64)
    assert sorted(group.tolist()) == [0, 1, 2, 3]
    nb = gb[group]
    assert nb.sum() <= 64
    assert nb[1] > nb[2] > nb[3] >= 1 and nb[2] >= nb[0]
    assert nb.min() >= 1


def test_plan_stops_when_blocks_stop_helping(pkg):
    # tiny problems: the barrier cost of a larger group outweighs its bandwidth
    group, gb = pkg.multi.plan_host([1e4, 1e4], [100, 100], blocks=500, bw_block=1e10)
    assert gb.tolist() == [1, 1]


def test_plan_queues_when_problems_outnumber_blocks(pkg):
    rng = np.random.default_rng(0)
    work = rng.uniform(1e5, 1e7, 50)
    group, gb = pkg.multi.plan_host(work, [100] * 50, blocks=8, bw_block=1e9)
    assert gb.tolist() == [1] * 8
    assert set(group.tolist()) == set(range(8))
    # longest-first packing keeps the groups' work within the largest problem
    load = np.zeros(8)
    np.add.at(load, group, work)
    assert load.max() - load.min() <= work.max()


def test_plan_rejects_bad_input(pkg):
    import pytest
    with pytest.raises(pkg._native.PlsqrError):
        pkg.multi.plan_host([], [], blocks=8, bw_block=1e9)
    with pytest.raises(pkg._native.PlsqrError):
        pkg.multi.plan_host([1.0], [1], blocks=0, bw_block=1e9)
