"""The C ABI library loads without a GPU, exports every symbol the public
header declares, and rejects bad input before touching a device."""
from __future__ import annotations

import ctypes as C
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = ROOT / "include" / "plsqr_gpu.h"


def declared_symbols():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(plsqr_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(pkg):
    so = pkg._native.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", str(so)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r" T (plsqr_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, f"declared but not exported: {missing}"
    assert len(declared_symbols()) >= 35


def test_binding_covers_header(pkg):
    assert set(declared_symbols()) == set(pkg._native.SIGNATURES)


def test_struct_sizes_match_header(pkg):
    N = pkg._native
    # sizes the C compiler gives the header's structs (x86_64 and aarch64 LP64)
    src = "#include <stdio.h>\n#include \"plsqr_gpu.h\"\nint main(){printf(\"%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n\"," \
          "sizeof(plsqr_sparse),sizeof(plsqr_files),sizeof(plsqr_opts),sizeof(plsqr_info)," \
          "sizeof(plsqr_lsqr_args),sizeof(plsqr_iter),sizeof(plsqr_result),sizeof(plsqr_synth_params),0," \
          "sizeof(plsqr_batch_args),sizeof(plsqr_batch_info),sizeof(plsqr_problem),sizeof(plsqr_multi_info));}"
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        (open(f"{d}/s.c", "w")).write(src)
        subprocess.run(["gcc", "-I", str(ROOT / "include"), f"{d}/s.c", "-o", f"{d}/s"], check=True)
        sizes = list(map(int, subprocess.run([f"{d}/s"], capture_output=True, text=True).stdout.split()))
    mine = [C.sizeof(N.Sparse), C.sizeof(N.Files), C.sizeof(N.Opts), C.sizeof(N.Info),
            C.sizeof(N.LsqrArgs), N.ITER_DTYPE.itemsize, C.sizeof(N.Result), C.sizeof(N.SynthParams), 0,
            C.sizeof(N.BatchArgs), C.sizeof(N.BatchInfo), C.sizeof(N.ProblemDesc), C.sizeof(N.MultiInfo)]
    assert sizes == mine


def test_strerror_and_version(pkg):
    L = pkg._native.lib()
    assert L.plsqr_abi_version() == 4
    assert L.plsqr_strerror(0) == b"success"
    assert L.plsqr_strerror(-3) == b"file or matrix content is inconsistent"
    assert L.plsqr_strerror(-99) == b"unknown error"


def test_defaults_are_call_lsqr_constants(pkg):
    N = pkg._native
    a = N.LsqrArgs()
    N.lib().plsqr_default_lsqr_args(C.byref(a))
    assert (a.damp, a.atol, a.btol, a.conlim, a.itnlim) == (0.0, 1e-10, 1e-10, 100.0, 1000)


def _sp(N, rows, cols, ptr, idx, val):
    s = N.Sparse()
    s.num_row, s.num_col, s.nnz = rows, cols, int(ptr[-1])
    s.ptr32, s.ptr64 = None, N.ptr(ptr)
    s.idx, s.val = N.ptr(idx), N.ptr(val)
    return s


@pytest.mark.parametrize("bad", ["row_out_of_range", "ptr_not_monotone", "ptr_end", "d_nnz"])
def test_create_rejects_bad_matrices_before_device(pkg, bad):
    N = pkg._native
    prob = pkg.generate("tiny")
    K = prob.k_csc
    kp, ki, kv = K.ptr.copy(), K.idx.copy(), K.val.copy()
    dc = prob.d_csc
    dcp = dc.ptr
    if bad == "row_out_of_range":
        ki[5] = prob.m_k
    elif bad == "ptr_not_monotone":
        kp[3], kp[4] = kp[4], kp[3] - 1
    k = _sp(N, prob.m_k, prob.n, kp, ki, kv)
    if bad == "ptr_end":
        k.nnz += 1  # pointer array ends below the declared nonzero count
    d = prob.d_csr.as_native()
    if bad == "d_nnz":
        dcp = dc.ptr.copy()
        dcp[-1] -= 1
    dcs = _sp(N, prob.m_d, prob.n, dcp, dc.idx, dc.val)
    h = N.vp()
    rc = N.lib().plsqr_ctx_create(C.byref(k), C.byref(d), C.byref(dcs), None, C.byref(h))
    assert rc == -3 and not h.value


@pytest.mark.parametrize("bad", ["huge", "nan"])
def test_create_rejects_values_outside_the_norm_range(pkg, bad):
    """Matrix values the FP64 sums of squares cannot hold (largest magnitude
    above 2^500) or NaN: PLSQR_ERR_NUMERIC, before any device work."""
    N = pkg._native
    prob = pkg.generate("tiny")
    K = prob.k_csc
    kv = K.val.copy()
    if bad == "huge":
        kv[7] = 2.0 ** 520
    else:
        kv[7] = np.nan
    k = _sp(N, prob.m_k, prob.n, K.ptr, K.idx, kv)
    d, dc = prob.d_csr.as_native(), prob.d_csc.as_native()
    h = N.vp()
    rc = N.lib().plsqr_ctx_create(C.byref(k), C.byref(d), C.byref(dc), None, C.byref(h))
    assert rc == -10 and not h.value
    assert "2^500" in N.lib().plsqr_strerror(-10).decode()


def test_create_without_device_reports_nodev(pkg, has_gpu):
    if has_gpu:
        pytest.skip("a device is visible")
    N = pkg._native
    prob = pkg.generate("tiny")
    h = N.vp()
    k, d, dc = prob.k_csc.as_native(), prob.d_csr.as_native(), prob.d_csc.as_native()
    assert N.lib().plsqr_ctx_create(C.byref(k), C.byref(d), C.byref(dc), None, C.byref(h)) == -6
    with pytest.raises(pkg._native.PlsqrError):
        pkg.Context(prob)


def test_null_arguments(pkg):
    L = pkg._native.lib()
    assert L.plsqr_ctx_create(None, None, None, None, None) == -1
    assert L.plsqr_aprod(None, 1, 0, 0) == -1
    assert L.plsqr_ctx_info(None, None) == -1
    L.plsqr_ctx_destroy(None)
