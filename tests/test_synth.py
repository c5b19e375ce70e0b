"""The synthetic problem generator: geometry of the ray tubes (checked against
an independent Python restatement of the counter-based hash), the damping
matrix against damping_binary.py's row order and counts, and the transposes."""
from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp

M64 = (1 << 64) - 1


def mix64(x):
    x ^= x >> 30
    x = (x * 0xBF58476D1CE4E5B9) & M64
    x ^= x >> 27
    x = (x * 0x94D049BB133111EB) & M64
    x ^= x >> 31
    return x


def hash4(seed, stream, a, b, c=0):
    h = mix64((seed + 0x9E3779B97F4A7C15 * (stream + 1)) & M64)
    h = mix64(h ^ ((a + 0x632BE59BD9B4E019) & M64))
    h = mix64(h ^ ((b + 0x8CB92BA72F3D8DD7) & M64))
    h = mix64(h ^ ((c + 0x3C6EF372FE94F82B) & M64))
    return h


def u01(h):
    return (h >> 11) * 2.0 ** -53


def ray_cells(cfg, r):
    """Brute force: every cell centre within the radius of ray r."""
    dims = (cfg["nx"], cfg["ny"], cfg["nz"])
    axis = cfg["face_axis"]
    p0, p1 = np.zeros(3), np.zeros(3)
    for c in range(3):
        if c == axis:
            p0[c], p1[c] = 0.0, dims[c]
        else:
            p0[c] = u01(hash4(cfg["seed"], 1, r, c)) * dims[c]
            p1[c] = u01(hash4(cfg["seed"], 1, r, c + 3)) * dims[c]
    iz, iy, ix = np.meshgrid(np.arange(dims[2]), np.arange(dims[1]), np.arange(dims[0]),
                             indexing="ij")
    q = np.stack([ix + 0.5, iy + 0.5, iz + 0.5], -1).reshape(-1, 3)
    d = p1 - p0
    t = np.clip(((q - p0) @ d) / (d @ d), 0.0, 1.0)
    dist2 = ((q - (p0 + t[:, None] * d)) ** 2).sum(1)
    return np.nonzero(dist2 <= cfg["tube_radius"] ** 2)[0]


@pytest.mark.parametrize("name", ["tiny", "grid32"])
def test_kernel_rows_are_the_ray_tubes(name, pkg):
    cfg = pkg.CONFIGS[name]
    prob = pkg.generate(name, keep_rows=True)
    K = prob.meta["k_csr"]
    for r in (0, 1, 7, cfg["n_rays"] - 1):
        cols = K.idx[K.ptr[r]:K.ptr[r + 1]]
        assert np.all(np.diff(cols) > 0), "columns of a row must ascend"
        exp = ray_cells(cfg, r)
        # a cell on the tube surface may go either way by one rounding
        assert abs(len(cols) - len(exp)) <= 1 and len(np.intersect1d(cols, exp)) >= len(exp) - 1
    assert np.all(K.val > 0) and np.all(K.val < 0.1)
    assert abs(K.val.mean() / 1e-2 - np.sqrt(2 / np.pi)) < 0.02  # |N(0,1)| * 1e-2


def test_damping_matches_damping_binary_layout(pkg):
    cfg = pkg.CONFIGS["tiny"]
    nx, ny, nz = cfg["nx"], cfg["ny"], cfg["nz"]
    prob = pkg.generate("tiny")
    D = prob.d_csr
    n = nx * ny * nz
    # damping_binary.py:51 / :61 totals for one parameter, cross terms omitted
    rows = n + (nx - 2) * ny * nz + nx * (ny - 2) * nz + nx * ny * (nz - 2)
    nnz = n + 3 * ((nx - 2) * ny * nz + nx * (ny - 2) * nz + nx * ny * (nz - 2))
    assert (D.num_row, D.nnz) == (rows, nnz)
    # per-cell order: identity, then xx, yy, zz when the stencil fits
    r = 0
    for c in range(n):
        ix, iy, iz = c % nx, (c // nx) % ny, c // (nx * ny)
        assert D.idx[D.ptr[r]] == c and D.val[D.ptr[r]] == cfg["damp_identity"]
        r += 1
        for fits, stride in ((ix < nx - 2, 1), (iy < ny - 2, nx), (iz < nz - 2, nx * ny)):
            if fits:
                e = D.ptr[r]
                assert list(D.idx[e:e + 3]) == [c, c + stride, c + 2 * stride]
                assert list(D.val[e:e + 3]) == [1.0, -2.0, 1.0]
                r += 1
    assert r == rows


@pytest.mark.parametrize("name", ["tiny", "grid32"])
def test_orientations_agree(name, pkg):
    prob = pkg.generate(name, keep_rows=True)
    Kr = prob.meta["k_csr"]
    A = sp.csr_matrix((Kr.val, Kr.idx, Kr.ptr), shape=(prob.m_k, prob.n))
    B = sp.csc_matrix((prob.k_csc.val, prob.k_csc.idx, prob.k_csc.ptr), shape=(prob.m_k, prob.n))
    assert (A != B).nnz == 0
    # rows ascend inside every column (the reference's column scatter order)
    for c in range(0, prob.n, max(1, prob.n // 50)):
        seg = prob.k_csc.idx[prob.k_csc.ptr[c]:prob.k_csc.ptr[c + 1]]
        assert np.all(np.diff(seg) > 0)
    D = sp.csr_matrix((prob.d_csr.val, prob.d_csr.idx, prob.d_csr.ptr), shape=(prob.m_d, prob.n))
    DC = sp.csc_matrix((prob.d_csc.val, prob.d_csc.idx, prob.d_csc.ptr), shape=(prob.m_d, prob.n))
    assert (D != DC).nnz == 0


def test_rhs_and_xtrue(pkg):
    prob = pkg.generate("grid32", keep_rows=True)
    Kr = prob.meta["k_csr"]
    A = sp.csr_matrix((Kr.val, Kr.idx, Kr.ptr), shape=(prob.m_k, prob.n))
    clean = A @ prob.x_true
    noise = prob.b_k - clean
    ratio = noise.std() / np.sqrt(np.mean(clean ** 2))
    assert 0.008 < ratio < 0.012
    again = pkg.generate("grid32")
    assert np.array_equal(again.b_k, prob.b_k) and np.array_equal(again.x_true, prob.x_true)
    other = pkg.generate("grid32", seed=1)
    assert not np.array_equal(other.b_k, prob.b_k)


def test_checkerboard(pkg):
    a = pkg.generate("tiny", n_blobs=0, checker_amp=0.1, checker_period=4)
    x = a.x_true.reshape(6, 8, 10)
    assert set(np.unique(x)) == {-0.1, 0.1}
    assert x[0, 0, 0] == 0.1 and x[0, 0, 2] == -0.1 and x[0, 2, 2] == 0.1


def test_transpose_rejects_out_of_range(pkg):
    N = pkg._native
    ptr = np.array([0, 2], np.int64)
    idx = np.array([0, 5], np.int32)
    val = np.ones(2)
    tp, ti, tv = np.zeros(4, np.int64), np.zeros(2, np.int32), np.zeros(2)
    assert N.lib().plsqr_transpose(1, 3, N.ptr(ptr), N.ptr(idx), N.ptr(val), N.ptr(tp),
                                   N.ptr(ti), N.ptr(tv)) == -3
