"""The timing report keyed by the reference's GPTL timer names
(source/lsqr.c:473-842, aprod_impl.c:69-497): a timed solve records CUDA
events around five regions of every iteration; the report lists them per
region and per iteration, and the solve's results do not change."""
from __future__ import annotations

import json
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden

pytestmark = pytest.mark.gpu

NAMES = ["spmv", "norm1", "spmvT", "update_x", "krylov_p1"]


@pytest.mark.parametrize("order", ["fast", "reference"])
def test_timed_solve_report_and_same_results(order, pkg, problems, tmp_path):
    prob = problems("grid32")
    it = 40
    with pkg.Context(prob, order=order) as ctx:
        plain = ctx.lsqr(lsqr_iteration=it)
        with pytest.raises(pkg._native.PlsqrError):
            ctx.write_timing(str(tmp_path / "none.json"))  # no timed solve yet
        ctx.set_timing(True)
        timed = ctx.lsqr(lsqr_iteration=it)
        rep = ctx.write_timing(str(tmp_path / "timing.json"))
        ctx.set_timing(False)
        again = ctx.lsqr(lsqr_iteration=it)
    assert np.array_equal(timed["x"], plain["x"]) and np.array_equal(again["x"], plain["x"])
    assert np.array_equal(timed["hist"]["alpha"], plain["hist"]["alpha"])
    assert rep["iterations"] == it and rep["order"] == order
    assert [r["name"] for r in rep["regions"]] == NAMES
    assert sorted(rep["per_iteration_ms"]) == sorted(NAMES)
    for r in rep["regions"]:
        per = rep["per_iteration_ms"][r["name"]]
        assert len(per) == it and min(per) >= 0.0
        assert r["covers"]
        assert abs(r["seconds"] - 1e-3 * sum(per)) <= 1e-6 + 1e-3 * r["seconds"]
    regions = sum(r["seconds"] for r in rep["regions"])
    loop = rep["LSQR_MAIN_ITERATION"]["seconds"]
    assert 0 < regions <= loop * (1 + 1e-3) + 1e-6  # the regions tile the loop
    assert regions >= 0.5 * loop


def test_cli_timing_and_reference_order(pkg, tmp_path):
    g = golden("tiny")
    f = g["meta"]["files"]
    exe = pkg._native.LIB_DIR / "plsqr3_gpu"
    it = g["meta"]["iterations"]
    cmd = [str(exe), "-dir", str(GOLDEN / "tiny" / "inputs"), "-quiet"]
    for k in ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol", "damp_i_bycol", "b_k"):
        cmd += [f"-{k}", f[k]]
    cmd += ["-row_k", str(f["row_k"]), "-row_d", str(f["row_d"]), "-col", str(f["col"]),
            "-itn", str(it), "-order", "reference", "-timing", "timing.json"]
    subprocess.run(cmd, cwd=tmp_path, check=True, capture_output=True)
    x = np.fromfile(tmp_path / f"p_resultx_itn={it}_NProc=1_float64_mpiio.bin", dtype=np.float64)
    assert np.array_equal(x, g["x"])  # the reference's bits
    assert (tmp_path / "result.txt").read_text() == g["result_txt"]
    rep = json.loads((tmp_path / "timing.json").read_text())
    assert rep["iterations"] == it and [r["name"] for r in rep["regions"]] == NAMES
