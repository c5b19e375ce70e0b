"""The reference's own program with the GPU operator in place of its aprod.c:
the shim of plsqr3.2013.09_gb300/integration/aprod_gpu.c compiled against
the reference's headers (warnings as errors) and linked to libplsqr_gpu, where
the reference tree is mounted.  Without a GPU the program reads its files,
starts lsqr(), reaches the first aprod() and stops there with the library's
error text; with one, it must reproduce the reference's own solution."""
from __future__ import annotations

import subprocess

import numpy as np
import pytest

from conftest import golden, rel


def test_reference_program_runs_the_gpu_operator(pkg, orc, tmp_path):
    binary = orc.build_gpu_aprod()
    if binary is None:
        pytest.skip("the reference tree is not mounted here")
    prob = pkg.generate("tiny")
    it = pkg.CONFIGS["tiny"]["iterations"]
    files = pkg.write_files(prob, tmp_path / "in")
    run = tmp_path / "run"
    run.mkdir()
    cmd = [str(binary), "-dir", str(tmp_path / "in")]
    for k in ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol", "damp_i_bycol", "b_k"):
        cmd += [f"-{k}", files[k]]
    cmd += ["-row_k", str(prob.m_k), "-row_d", str(prob.m_d), "-col", str(prob.n),
            "-itn", str(it)]
    r = subprocess.run(cmd, cwd=run, capture_output=True, text=True, timeout=120)
    if pkg._native.device_count() == 0:
        assert r.returncode != 0
        assert "aprod on GPU: no usable CUDA device" in r.stderr
        assert "ORACLE_beta" in r.stdout  # lsqr() started and called aprod()
        return
    assert r.returncode == 0, r.stderr[-2000:]
    x = np.fromfile(run / f"p_resultx_itn={it}_NProc=1_float64_mpiio.bin", dtype=np.float64)
    assert rel(x, golden("tiny")["x"]) <= 1e-10
