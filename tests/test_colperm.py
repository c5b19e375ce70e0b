"""Column permutation (the reference's COL_PERM build): the kernel matrix is
loaded with its column i taken from file column perm[i]; the damping files
and b_k are read as given and x comes out in the permuted order.

tests/golden/grid32p is the reference program's solve of the 32^3 problem
with the kernel file written so (the COL_PERM build itself cannot run, see
make_golden.run_col_perm); the oracle on the permuted matrix must give its
bits.  GPU: the context built from the original files plus the permutation
file reproduces it, bit for bit in the reference's order."""
from __future__ import annotations

import hashlib
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden, rel

def perm_of(g, n):
    return np.random.default_rng(g["meta"]["perm_seed"]).permutation(n).astype(np.int32)


def test_permute_columns_selects_columns_in_stored_order(pkg):
    prob = pkg.generate("tiny")
    perm = np.random.default_rng(5).permutation(prob.n).astype(np.int32)
    perm[3] = perm[4]  # a repeated column is a selection the loader allows
    kp = pkg.synth.permute_columns(prob.k_csc, perm)
    K = prob.k_csc
    for i, c in enumerate(perm):
        a, b = K.ptr[c], K.ptr[c + 1]
        assert np.array_equal(kp.idx[kp.ptr[i]:kp.ptr[i + 1]], K.idx[a:b])
        assert np.array_equal(kp.val[kp.ptr[i]:kp.ptr[i + 1]], K.val[a:b])


def test_read_col_perm_file(pkg, tmp_path):
    N = pkg._native
    perm = np.random.default_rng(1).permutation(50).astype(np.int32)
    pkg.synth.write_col_perm(tmp_path / "p", perm)
    got = np.empty(50, np.int32)
    assert N.lib().plsqr_io_read_col_perm(str(tmp_path / "p").encode(), 50, N.ptr(got)) == 0
    assert np.array_equal(got, perm)
    for text in ("1\n2\n", "0\n" * 50, "51\n" * 50):  # short, below 1, above n
        (tmp_path / "bad").write_text(text)
        assert N.lib().plsqr_io_read_col_perm(str(tmp_path / "bad").encode(), 50,
                                              N.ptr(got)) == -3  # PLSQR_ERR_FORMAT
    assert N.lib().plsqr_io_read_col_perm(str(tmp_path / "none").encode(), 50,
                                          N.ptr(got)) == -2  # PLSQR_ERR_IO


def test_oracle_on_permuted_columns_is_the_reference(pkg, orc, tmp_path):
    g = golden("grid32p")
    prob = pkg.generate(g["meta"]["base"])
    perm = perm_of(g, prob.n)
    pkg.synth.write_col_perm(tmp_path / "colPerm", perm)
    assert hashlib.sha256((tmp_path / "colPerm").read_bytes()).hexdigest() == \
        g["meta"]["col_perm_sha256"]
    kp = pkg.synth.permute_columns(prob.k_csc, perm)
    pp = pkg.Problem(kp, prob.d_csr, prob.d_csc, prob.b_k, prob.x_true, 0, prob.meta)
    out = orc.OracleProblem(pp).lsqr(g["meta"]["iterations"], result_txt=str(tmp_path / "r.txt"))
    assert np.array_equal(out["x"], g["x"])
    assert np.array_equal(out["hist"]["alpha"], g["alpha"])
    assert np.array_equal(out["hist"]["beta"], g["beta"])
    assert (tmp_path / "r.txt").read_text() == g["result_txt"]


def _files_with_perm(pkg, g, tmp_path):
    prob = pkg.generate(g["meta"]["base"])
    files = pkg.write_files(prob, tmp_path)  # the original, unpermuted files
    pkg.synth.write_col_perm(tmp_path / "colPerm", perm_of(g, prob.n))
    return prob, dict(files, col_perm="colPerm")


@pytest.mark.gpu
@pytest.mark.parametrize("order", ["reference", "fast"])
def test_gpu_col_perm_reproduces_reference(order, pkg, tmp_path):
    g = golden("grid32p")
    _, files = _files_with_perm(pkg, g, tmp_path)
    with pkg.Context(files=files, order=order) as ctx:
        out = ctx.lsqr(lsqr_iteration=g["meta"]["iterations"])
    if order == "reference":
        assert np.array_equal(out["x"], g["x"])
        assert np.array_equal(out["hist"]["alpha"], g["alpha"])
        assert np.array_equal(out["hist"]["beta"], g["beta"])
    else:
        assert rel(out["x"], g["x"]) <= 1e-10


@pytest.mark.gpu
def test_gpu_cli_col_perm(pkg, tmp_path):
    g = golden("grid32p")
    prob, files = _files_with_perm(pkg, g, tmp_path)
    it = g["meta"]["iterations"]
    exe = pkg._native.LIB_DIR / "plsqr3_gpu"
    cmd = [str(exe), "-dir", str(tmp_path), "-quiet", "-order", "reference"]
    for k in ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol", "damp_i_bycol", "b_k",
              "col_perm"):
        cmd += [f"-{k}", files[k]]
    cmd += ["-row_k", str(prob.m_k), "-row_d", str(prob.m_d), "-col", str(prob.n), "-itn", str(it)]
    run = tmp_path / "run"
    run.mkdir()
    subprocess.run(cmd, cwd=run, check=True, capture_output=True)
    x = np.fromfile(run / f"p_resultx_itn={it}_NProc=1_float64_mpiio.bin", dtype=np.float64)
    assert np.array_equal(x, g["x"])
    assert (run / "result.txt").read_text() == g["result_txt"]
