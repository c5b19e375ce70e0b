"""Ray kernels in their ASCII exchange format (raykernels) and the damping
generator's full form, on the CPU.

The fixture tests/golden/socal25 holds the first 25 rays of the reference's
data/ sample in a lossless compact form; its kernel files were made by the
reference's own kernel-format tools and matched the restated conversion
byte for byte when the fixture was made.  Here: the fixture decodes to the
same arrays and files, the damping matrix of the sample's README has the
reference's sizes and row layout, the oracle reproduces the reference
program's run on the fixture bit for bit, and, where the reference tree is
mounted, the conversion of all 100 rays equals the reference tools' output."""
from __future__ import annotations

import hashlib
import importlib.util
import json

import numpy as np
import pytest

from conftest import GOLDEN

SOCAL = GOLDEN / "socal25"


def _make_golden():
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    return mg


def socal_fixture(pkg):
    z = np.load(SOCAL / "rays.npz")
    rays = pkg.raykernels.socal_from_compact(z)
    return pkg.raykernels.socal_from_rays(rays, z["b_k"]), json.loads((SOCAL / "meta.json").read_text())


def test_fixture_decodes_to_the_reference_tools_files(pkg, tmp_path):
    prob, meta = socal_fixture(pkg)
    assert (prob.m_k, prob.m_d, prob.n) == (meta["m_k"], meta["m_d"], meta["n"])
    assert prob.meta["nnz_k"] == meta["nnz_k"] and prob.meta["nnz_d"] == meta["nnz_d"]
    assert _make_golden().array_digest(prob) == meta["array_sha256"]
    files = pkg.write_files(prob, tmp_path)
    for name, digest in meta["kernel_files_sha256"].items():
        assert hashlib.sha256((tmp_path / name).read_bytes()).hexdigest() == digest, name
    # and the files read back to the same matrix
    back = pkg.read_files(files)
    for a, b in ((back.k_csc, prob.k_csc), (back.d_csr, prob.d_csr), (back.d_csc, prob.d_csc)):
        assert np.array_equal(a.ptr, b.ptr) and np.array_equal(a.idx, b.idx)
        assert np.array_equal(a.val, b.val)


def test_socal_damping_sizes_match_the_reference_run():
    """data/README:19 (every weight 1.0, 2 fields on 99 x 153 x 10) gives the
    -row_d of data/LSQR_run/LSQR3.pbs:10 and the damping nonzeros of
    data/load_balance.sh:1."""
    import __graft_entry__ as g
    R = g.load_package().raykernels
    d_csr, d_csc = R.damping()
    assert d_csr.num_row == 1910672 and d_csr.nnz == 5895716
    assert d_csr.num_col == 302940 and d_csc.nnz == d_csr.nnz


def test_damping_rows_in_damping_binary_order(pkg):
    """Per cell: identity, xx, yy, zz, xy, xz, yz (each where its stencil
    fits), the second field repeating the first with columns and rows
    offset (damping_binary.py:84-511, 578-610)."""
    nx, ny, nz = 4, 3, 3
    d_csr, _ = pkg.raykernels.damping(grid=(nx, ny, nz), fields=2, weights=(0.5, 2.0, 4.0))
    ncell = nx * ny * nz
    rows = []
    for r in range(d_csr.num_row):
        a, b = d_csr.ptr[r], d_csr.ptr[r + 1]
        rows.append(list(zip(d_csr.idx[a:b].tolist(), d_csr.val[a:b].tolist())))
    half = len(rows) // 2
    assert len(rows) == 2 * half
    for r in range(half):
        assert rows[half + r] == [(c + ncell, v) for c, v in rows[r]]
    sx, sy, sz = 1, nx, nx * ny
    expect = []
    for iz in range(nz):
        for iy in range(ny):
            for ix in range(nx):
                c = iz * sz + iy * sy + ix
                expect.append([(c, 0.5)])
                fx, fy, fz = ix < nx - 2, iy < ny - 2, iz < nz - 2
                for f, s in ((fx, sx), (fy, sy), (fz, sz)):
                    if f:
                        expect.append([(c, 2.0), (c + s, -4.0), (c + 2 * s, 2.0)])
                for f, s1, s2 in ((fx and fy, sx, sy), (fx and fz, sx, sz), (fy and fz, sy, sz)):
                    if f:
                        expect.append([(c, 2.0), (c + 2 * s1, -2.0), (c + 2 * s2, -2.0),
                                       (c + 2 * s1 + 2 * s2, 2.0)])
    assert rows[:half] == expect


def test_oracle_reproduces_the_reference_run_on_the_fixture(pkg, orc):
    prob, meta = socal_fixture(pkg)
    it = meta["iterations"]
    out = orc.OracleProblem(prob).lsqr(it)
    ab = np.loadtxt(SOCAL / "alpha_beta.txt")
    assert np.array_equal(out["hist"]["alpha"], ab[:, 1])
    assert np.array_equal(out["hist"]["beta"], ab[:, 2])
    assert hashlib.sha256(out["x"].tobytes()).hexdigest() == meta["x_sha256"]


def test_compact_form_is_lossless():
    import __graft_entry__ as g
    R = g.load_package().raykernels
    rng = np.random.default_rng(3)
    vals = np.array([float(f"{m}e{q}") for m, q in zip(rng.integers(-9999999, 9999999, 200),
                                                          rng.integers(-30, 5, 200))])
    vals = np.array([float(f"{v:.6e}") for v in vals])
    rays = [(np.sort(rng.choice(1000, 200, replace=False)).astype(np.int32), vals)]
    back = R.socal_from_compact(R.socal_compact(rays))
    assert np.array_equal(back[0][0], rays[0][0]) and np.array_equal(back[0][1], rays[0][1])
    with pytest.raises(ValueError):
        R.socal_compact([(np.array([0], np.int32), np.array([1.0 / 3.0]))])


def test_full_sample_conversion_equals_the_reference_tools(pkg, orc, tmp_path):
    """All 100 rays of data/, converted here and by the reference's own
    ker_ascii2bin, Ker2PLSQR3_preprocess and Ker2PLSQR3: the same bytes."""
    mg = _make_golden()
    data = mg.reference_data_dir(orc)
    if not (data / "ker.list").exists() or not orc.reference_available():
        pytest.skip("the reference tree is not mounted here")
    R = pkg.raykernels
    names = R.read_list(data / "ker.list")
    prob = R.socal_problem(data)
    assert prob.m_k == 100 and prob.meta["nnz_k"] == 1266788
    files = pkg.write_files(prob, tmp_path / "in")
    tool_dir = mg.convert_with_reference_tools(orc, data, names, prob.n, tmp_path / "tools")
    for k, fn in (("ker_f", "matrix_bycol.mm2.bin"), ("ker_i", "matrix_bycol.mm2.info")):
        assert (tmp_path / "in" / files[k]).read_bytes() == (tool_dir / fn).read_bytes(), fn
