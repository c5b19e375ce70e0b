"""The product entry point that allocates no device memory.

Callers whose device memory belongs to another allocator or a fixed budget,
or that cannot block on the driver's allocator, cannot let the library call
cudaMalloc; plsqr_aprod1_nrm2_noalloc takes all of its buffers from the caller
and keeps its only scratch (one partial sum per block) in a static device
array of the library.  This file is collected last so that a failure here
stops a -x run only after every other test has run; it passes alone and
after the others.

Checked through the C ABI against the existing entry point (plsqr_aprod_host
on a context of the same matrix) with the product tolerance of the parity
tests, on two calls in a row, plus the size limit, an empty matrix and the
refusal of unaligned indices or values."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

APROD_TOL = 1e-12


def _call(pkg, torch, dev_csr, x, y):
    N = pkg._native
    ptr, idx, val = dev_csr
    xd = torch.from_numpy(x).cuda()
    yd = torch.from_numpy(y).cuda()
    nrm = torch.zeros(1, dtype=torch.float64, device="cuda")
    rc = N.lib().plsqr_aprod1_nrm2_noalloc(
        int(ptr.numel() - 1), C.c_void_p(ptr.data_ptr()), C.c_void_p(idx.data_ptr()),
        C.c_void_p(val.data_ptr()), C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()),
        C.c_void_p(nrm.data_ptr()), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    return yd.cpu().numpy(), float(nrm.cpu()[0])


@pytest.mark.parametrize("case", ["tiny", "grid32"])
def test_noalloc_matches_existing_entry_point_twice(case, pkg):
    torch = pytest.importorskip("torch")
    import scipy.sparse as sp
    prob = pkg.generate(case, keep_rows=True)
    K = prob.meta["k_csr"]
    dev_csr = (torch.from_numpy(K.ptr).cuda(), torch.from_numpy(K.idx).cuda(),
               torch.from_numpy(K.val).cuda())
    absK = abs(sp.csr_matrix((K.val, K.idx, K.ptr), shape=(prob.m_k, prob.n)))
    rng = np.random.default_rng(11)
    with pkg.Context(prob) as ctx:
        for _ in range(2):  # two calls in a row share the static scratch
            x = rng.standard_normal(prob.n)
            yk = rng.standard_normal(prob.m_k)
            got, nrm = _call(pkg, torch, dev_csr, x, yk.copy())
            ref_k, ref_d, xx = yk.copy(), np.zeros(prob.m_d), x.copy()
            ctx.aprod_host(1, ref_k, ref_d, xx)  # existing entry point: y_k += K x
            scale = absK @ np.abs(x) + np.abs(yk)
            assert np.all(np.abs(got - ref_k) <= APROD_TOL * scale + 1e-300)
            assert abs(nrm - np.linalg.norm(ref_k)) <= APROD_TOL * np.linalg.norm(ref_k)


def test_noalloc_rejects_sizes_beyond_its_scratch(pkg):
    N = pkg._native
    rc = N.lib().plsqr_aprod1_nrm2_noalloc(N.NOALLOC_MAX_ROWS + 1, C.c_void_p(16), C.c_void_p(16),
                                           C.c_void_p(16), C.c_void_p(16), C.c_void_p(16),
                                           C.c_void_p(16), None)
    assert rc == -1  # PLSQR_ERR_ARG, before any device work


def test_noalloc_empty_and_misaligned(pkg):
    """n_rows = 0 writes ||y|| = 0; indices or values that are not 16-byte
    aligned (the product's vector loads) are refused."""
    torch = pytest.importorskip("torch")
    N = pkg._native
    ptr = torch.zeros(1, dtype=torch.int64, device="cuda")
    nrm = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    idx = torch.zeros(8, dtype=torch.int32, device="cuda")
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = N.lib().plsqr_aprod1_nrm2_noalloc(0, C.c_void_p(ptr.data_ptr()), None, None, None,
                                           None, C.c_void_p(nrm.data_ptr()), s)
    assert rc == 0
    torch.cuda.synchronize()
    assert float(nrm.cpu()[0]) == 0.0
    for i_off, v_off in ((0, 8), (4, 0)):
        rc = N.lib().plsqr_aprod1_nrm2_noalloc(
            1, C.c_void_p(ptr.data_ptr()), C.c_void_p(idx.data_ptr() + i_off),
            C.c_void_p(buf.data_ptr() + v_off), C.c_void_p(buf.data_ptr()),
            C.c_void_p(buf.data_ptr()), C.c_void_p(nrm.data_ptr()), s)
        assert rc == -1  # PLSQR_ERR_ARG
