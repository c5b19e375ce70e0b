"""The reference's file formats: writers, readers, and the error codes that
replace the reference loaders' exit(-1) (source/plsqr3.c:1008-1626)."""
from __future__ import annotations

import ctypes as C
import shutil
import struct

import numpy as np
import pytest

from conftest import GOLDEN, golden


@pytest.fixture()
def tiny_files(tmp_path):
    src = GOLDEN / "tiny" / "inputs"
    dst = tmp_path / "in"
    shutil.copytree(src, dst)
    f = dict(golden("tiny")["meta"]["files"], dir=str(dst))
    return f


def _create_files_rc(pkg, f):
    """plsqr_ctx_create_files: every file is read and checked before the
    device is touched, so format errors are reported without a GPU."""
    N = pkg._native
    ff = N.Files()
    for k in ("ker_f", "ker_i", "damp_f", "damp_i", "damp_f_bycol", "damp_i_bycol", "b_k"):
        setattr(ff, k, str(f[k]).encode())
    ff.dir = str(f["dir"]).encode()
    ff.row_k, ff.row_d, ff.col = int(f["row_k"]), int(f["row_d"]), int(f["col"])
    h = N.vp()
    rc = N.lib().plsqr_ctx_create_files(C.byref(ff), None, C.byref(h))
    if h.value:
        N.lib().plsqr_ctx_destroy(h)
    return rc


def test_round_trip(pkg, tmp_path):
    prob = pkg.generate("tiny")
    f = pkg.write_files(prob, tmp_path)
    back = pkg.read_files(f)
    for a, b in ((prob.k_csc, back.k_csc), (prob.d_csr, back.d_csr), (prob.d_csc, back.d_csc)):
        assert np.array_equal(a.ptr, b.ptr) and np.array_equal(a.idx, b.idx)
        assert np.array_equal(a.val, b.val)
    assert np.array_equal(prob.b_k, back.b_k)  # %.17e round-trips exactly


def test_record_layout_and_info_text(pkg, tiny_files):
    d = tiny_files["dir"]
    raw = open(f"{d}/{tiny_files['ker_f']}", "rb").read()
    assert len(raw) % 16 == 0
    r, c, v = struct.unpack("<iid", raw[:16])
    lines = open(f"{d}/{tiny_files['ker_i']}").read().split("\n")
    col, nnz, start = map(int, lines[0].split())
    assert col == 1 and (start == 1 if nnz else start == 0)
    first_nonempty = next(l for l in lines if l and int(l.split()[1]) > 0)
    assert int(first_nonempty.split()[2]) == 1
    assert r >= 1 and c == int(first_nonempty.split()[0]) and v > 0
    # empty columns carry start 0 (Ker2PLSQR3.c:507-508)
    for l in lines:
        if l and int(l.split()[1]) == 0:
            assert int(l.split()[2]) == 0


def test_kernel_column_field_is_not_used_like_the_reference(pkg, tiny_files, tmp_path):
    """The reference assigns kernel records to columns by the info counts and
    ignores the record's column field (plsqr3.c:1596-1619)."""
    d = tiny_files["dir"]
    p = f"{d}/{tiny_files['ker_f']}"
    a = np.fromfile(p, dtype=np.dtype([("r", "<i4"), ("c", "<i4"), ("v", "<f8")]))
    a["c"] = 12345
    a.tofile(p)
    back = pkg.read_files(tiny_files)
    ref = pkg.read_files(dict(tiny_files, dir=str(GOLDEN / "tiny" / "inputs")))
    assert np.array_equal(back.k_csc.idx, ref.k_csc.idx)
    assert np.array_equal(back.k_csc.val, ref.k_csc.val)


def _damage(tiny_files, key, fn):
    p = f"{tiny_files['dir']}/{tiny_files[key]}"
    data = bytearray(open(p, "rb").read())
    data = fn(data)
    open(p, "wb").write(bytes(data))


REC = np.dtype([("r", "<i4"), ("c", "<i4"), ("v", "<f8")])


def _recs(tiny_files, key, fn):
    p = f"{tiny_files['dir']}/{tiny_files[key]}"
    a = np.fromfile(p, dtype=REC)
    fn(a)
    a.tofile(p)


@pytest.mark.parametrize("case,expected", [
    ("missing_kernel", -2),
    ("truncated_kernel", -3),
    ("kernel_row_too_large", -3),       # plsqr3.c:1610-1615 exits
    ("kernel_row_zero", -3),            # 0 in a 1-based file
    ("info_short", -3),
    ("damping_row_out_of_range", -3),   # plsqr3.c:1149-1153 exits
    ("damping_col_out_of_range", -3),
    ("damping_unsorted", -3),
    ("damping_info_mismatch", -3),
    ("damping_bycol_info_total", -3),
    ("bycol_out_of_range", -3),         # plsqr3.c:1178-1182 exits
    ("rhs_short", -3),
    ("negative_count", -3),
])
def test_malformed_inputs_are_rejected(case, expected, pkg, tiny_files):
    f = tiny_files
    if case == "missing_kernel":
        f = dict(f, ker_f="no_such_file.bin")
    elif case == "truncated_kernel":
        _damage(f, "ker_f", lambda d: d[:-16])
    elif case == "kernel_row_too_large":
        _recs(f, "ker_f", lambda a: a["r"].__setitem__(3, f["row_k"] + 1))
    elif case == "kernel_row_zero":
        _recs(f, "ker_f", lambda a: a["r"].__setitem__(3, 0))
    elif case == "info_short":
        p = f"{f['dir']}/{f['ker_i']}"
        lines = open(p).read().splitlines()
        open(p, "w").write("\n".join(lines[:-5]) + "\n")
    elif case == "damping_row_out_of_range":
        _recs(f, "damp_f", lambda a: a["r"].__setitem__(-1, f["row_d"] + 1))
    elif case == "damping_col_out_of_range":
        _recs(f, "damp_f", lambda a: a["c"].__setitem__(5, f["col"] + 1))
    elif case == "damping_unsorted":
        def swap(a):
            a[[10, 200]] = a[[200, 10]]
        _recs(f, "damp_f", swap)
    elif case == "damping_info_mismatch":
        p = f"{f['dir']}/{f['damp_i']}"
        c = np.fromfile(p, dtype="<i4")
        c[0] += 1
        c[1] -= 1
        c.tofile(p)
    elif case == "damping_bycol_info_total":
        p = f"{f['dir']}/{f['damp_i_bycol']}"
        c = np.fromfile(p, dtype="<i4")
        c[0] -= 1
        c.tofile(p)
    elif case == "bycol_out_of_range":
        _recs(f, "damp_f_bycol", lambda a: a["r"].__setitem__(7, f["row_d"] + 1))
    elif case == "rhs_short":
        p = f"{f['dir']}/{f['b_k']}"
        lines = open(p).read().splitlines()
        open(p, "w").write("\n".join(lines[:-1]) + "\n")
    elif case == "negative_count":
        p = f"{f['dir']}/{f['damp_i']}"
        c = np.fromfile(p, dtype="<i4")
        c[3] = -1
        c.tofile(p)
    assert _create_files_rc(pkg, f) == expected


def test_valid_files_pass_every_check(pkg, tiny_files, has_gpu):
    rc = _create_files_rc(pkg, tiny_files)
    assert rc == (0 if has_gpu else -6)


def test_write_x_is_raw_float64(pkg, tmp_path):
    x = np.linspace(-1, 1, 37)
    N = pkg._native
    assert N.lib().plsqr_io_write_x(str(tmp_path / "x.bin").encode(), x.size, N.ptr(x)) == 0
    assert np.array_equal(np.fromfile(tmp_path / "x.bin", dtype=np.float64), x)


def test_readers_reject_bad_arguments(pkg):
    L = pkg._native.lib()
    assert L.plsqr_io_read_rhs(None, 3, None) == -1
    assert L.plsqr_io_read_kernel_info(b"/nonexistent", 3, None, None, None) == -1
    assert L.plsqr_io_read_int32_counts(b"/nonexistent/x", 0, None, None) == -2
