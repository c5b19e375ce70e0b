"""Synthetic tomography problems in PLSQR3's data model and file formats.

The generator itself is native (csrc/synth.cpp, counter-based random numbers,
identical bits on x86_64 and aarch64); this module holds the named
configurations and turns a parameter set into the in-memory operator the C
ABI takes (kernel matrix by column, damping matrix by row and by column) and,
on request, into the reference's input files (the outputs of the
PLSQR3_tools programs: Ker2PLSQR3.c:499-608, damping_binary.py:75-616).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _native as N

# Named problems.  "tiny" is small enough for pure-Python checks; "grid32"
# and "grid96" are the 32x32x32 / 2,000-ray and 96x96x32 / 200,000-ray
# tomography problems (100 and 300 LSQR iterations).
CONFIGS: dict[str, dict] = {
    "tiny": dict(nx=10, ny=8, nz=6, n_rays=60, tube_radius=1.5, face_axis=2, n_blobs=3,
                 blob_sigma=2.0, checker_amp=0.0, checker_period=8, noise_frac=0.01,
                 value_scale=1e-2, damp_identity=0.5, damp_lap=1.0, seed=7, iterations=40),
    "grid32": dict(nx=32, ny=32, nz=32, n_rays=2000, tube_radius=1.5, face_axis=2, n_blobs=8,
                   blob_sigma=3.0, checker_amp=0.0, checker_period=8, noise_frac=0.01,
                   value_scale=1e-2, damp_identity=0.5, damp_lap=1.0, seed=0, iterations=100),
    "grid96": dict(nx=96, ny=96, nz=32, n_rays=200000, tube_radius=6.0, face_axis=2, n_blobs=64,
                   blob_sigma=3.0, checker_amp=0.1, checker_period=8, noise_frac=0.01,
                   value_scale=1e-2, damp_identity=0.5, damp_lap=1.0, seed=0, iterations=300),
}
# the 96x96x32 grid with a tenth of the rays (~1.3e8 kernel nonzeros, ~3 GB on
# the device): large enough to stream from HBM, small enough to profile
CONFIGS["grid96s"] = dict(CONFIGS["grid96"], n_rays=20000)
# a 48x48x32 grid with 40,000 radius-6 rays (~1.8e8 nonzeros, ~4,500 per row
# and ~2,500 per column, ~4.5 GB on the device): line lengths close to the
# 96x96x32 problem's, for kernel profiles
CONFIGS["grid48p"] = dict(CONFIGS["grid96"], nx=48, ny=48, n_rays=40000)

# the reference's file names for a generated problem (data/LSQR_run/LSQR3.pbs:10)
FILE_NAMES = dict(ker_f="matrix_bycol.mm2.bin", ker_i="matrix_bycol.mm2.info",
                  damp_f="damp_row_data.bin", damp_i="damp_row_info.bin",
                  damp_f_bycol="damp_col_data.bin", damp_i_bycol="damp_col_info.bin",
                  b_k="measure.list")


def params(name_or_dict, **over) -> N.SynthParams:
    cfg = dict(CONFIGS[name_or_dict]) if isinstance(name_or_dict, str) else dict(name_or_dict)
    cfg.update(over)
    p = N.SynthParams()
    N.lib().plsqr_synth_default_params(C.byref(p))
    for k, v in cfg.items():
        if k == "iterations":
            continue
        setattr(p, k, v)
    return p


@dataclass
class Lines:
    """Compressed sparse lines: ptr over lines (int64), idx (int32), val (f64)."""
    ptr: np.ndarray
    idx: np.ndarray
    val: np.ndarray
    num_row: int
    num_col: int

    @property
    def nnz(self) -> int:
        return int(self.ptr[-1])

    def as_native(self) -> N.Sparse:
        s = N.Sparse()
        s.num_row, s.num_col, s.nnz = self.num_row, self.num_col, self.nnz
        s.ptr32, s.ptr64 = None, N.ptr(self.ptr)
        s.idx, s.val = N.ptr(self.idx), N.ptr(self.val)
        return s

    def transposed(self, by_col: bool) -> "Lines":
        """The other orientation; by_col tells which one self is."""
        n_lines = self.num_col if by_col else self.num_row
        n_out = self.num_row if by_col else self.num_col
        tptr = np.empty(n_out + 1, np.int64)
        tidx = np.empty(self.nnz, np.int32)
        tval = np.empty(self.nnz, np.float64)
        N.check(N.lib().plsqr_transpose(n_lines, n_out, N.ptr(self.ptr), N.ptr(self.idx),
                                        N.ptr(self.val), N.ptr(tptr), N.ptr(tidx), N.ptr(tval)),
                "plsqr_transpose")
        return Lines(tptr, tidx, tval, self.num_row, self.num_col)


def permute_columns(k_csc: Lines, perm) -> Lines:
    """The by-column matrix with column i taken from column perm[i] (the
    COL_PERM loader, source/plsqr3.c:1695-1713)."""
    perm = np.ascontiguousarray(perm, np.int32)
    n = k_csc.num_col
    if perm.shape != (n,):
        raise ValueError(f"perm must hold {n} column numbers")
    cnt = k_csc.ptr[perm.astype(np.int64) + 1] - k_csc.ptr[perm]
    tptr = np.zeros(n + 1, np.int64)
    np.cumsum(cnt, out=tptr[1:])
    tidx = np.empty(int(tptr[-1]), np.int32)
    tval = np.empty(int(tptr[-1]), np.float64)
    N.check(N.lib().plsqr_permute_columns(n, N.ptr(k_csc.ptr), N.ptr(k_csc.idx),
                                          N.ptr(k_csc.val), N.ptr(perm), N.ptr(tptr),
                                          N.ptr(tidx), N.ptr(tval)), "plsqr_permute_columns")
    return Lines(tptr, tidx, tval, k_csc.num_row, n)


def write_col_perm(path, perm) -> None:
    """A column permutation file: one 1-based column number per line."""
    Path(path).write_text("".join(f"{int(c) + 1}\n" for c in perm))


@dataclass
class Problem:
    """The operator in the reference's in-memory layout plus b_k and x_true."""
    k_csc: Lines
    d_csr: Lines
    d_csc: Lines
    b_k: np.ndarray
    x_true: np.ndarray
    iterations: int = 100
    meta: dict = field(default_factory=dict)

    @property
    def m_k(self) -> int:
        return self.k_csc.num_row

    @property
    def m_d(self) -> int:
        return self.d_csr.num_row

    @property
    def n(self) -> int:
        return self.k_csc.num_col


def damping_from_params(p: N.SynthParams) -> tuple[Lines, Lines]:
    """The damping matrix of the parameters, by row and by column (the
    rows of every column in ascending order, as damping_binary.py's sorted
    column file holds them)."""
    L = N.lib()
    m_d, nnz_d = N.i64(0), N.i64(0)
    N.check(L.plsqr_synth_damping_size(C.byref(p), C.byref(m_d), C.byref(nnz_d)), "damping_size")
    drp = np.empty(m_d.value + 1, np.int64)
    dci = np.empty(nnz_d.value, np.int32)
    dv = np.empty(nnz_d.value, np.float64)
    N.check(L.plsqr_synth_damping_fill(C.byref(p), N.ptr(drp), N.ptr(dci), N.ptr(dv)),
            "damping_fill")
    n = p.nx * p.ny * p.nz * max(1, p.n_params)
    d_csr = Lines(drp, dci, dv, int(m_d.value), n)
    return d_csr, d_csr.transposed(by_col=False)


def generate(name_or_dict="grid32", keep_rows: bool = False, **over) -> Problem:
    """Build a synthetic problem.  keep_rows also returns the kernel by row
    (meta['k_csr']); otherwise it is dropped after the transpose."""
    L = N.lib()
    p = params(name_or_dict, **over)
    iters = (CONFIGS[name_or_dict] if isinstance(name_or_dict, str) else name_or_dict).get(
        "iterations", 100)
    n = p.nx * p.ny * p.nz
    m_k = p.n_rays
    rp = np.empty(m_k + 1, np.int64)
    N.check(L.plsqr_synth_kernel_counts(C.byref(p), N.ptr(rp)), "synth_kernel_counts")
    nnz = int(rp[-1])
    ci = np.empty(nnz, np.int32)
    kv = np.empty(nnz, np.float64)
    N.check(L.plsqr_synth_kernel_fill(C.byref(p), N.ptr(rp), N.ptr(ci), N.ptr(kv)),
            "synth_kernel_fill")
    k_csr = Lines(rp, ci, kv, m_k, n)
    x_true = np.empty(n, np.float64)
    N.check(L.plsqr_synth_xtrue(C.byref(p), N.ptr(x_true)), "synth_xtrue")
    b = np.empty(m_k, np.float64)
    N.check(L.plsqr_synth_rhs(C.byref(p), N.ptr(rp), N.ptr(ci), N.ptr(kv), N.ptr(x_true),
                              N.ptr(b)), "synth_rhs")
    k_csc = k_csr.transposed(by_col=False)
    d_csr, d_csc = damping_from_params(p)
    meta = dict(grid=(p.nx, p.ny, p.nz), n_rays=m_k, tube_radius=p.tube_radius,
                nnz_k=nnz, nnz_d=d_csr.nnz, seed=int(p.seed))
    if keep_rows:
        meta["k_csr"] = k_csr
    else:
        del k_csr
    return Problem(k_csc, d_csr, d_csc, b, x_true, iters, meta)


def write_files(prob: Problem, directory: str | Path, names: dict | None = None) -> dict:
    """Write the problem as the reference's input files; returns the file
    names (relative to directory) and the sizes the CLI needs."""
    names = dict(FILE_NAMES, **(names or {}))
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    L = N.lib()
    f = lambda k: str(d / names[k]).encode()
    K, D, DC = prob.k_csc, prob.d_csr, prob.d_csc
    N.check(L.plsqr_io_write_kernel(f("ker_f"), f("ker_i"), prob.m_k, prob.n, N.ptr(K.ptr),
                                    N.ptr(K.idx), N.ptr(K.val)), "write_kernel")
    N.check(L.plsqr_io_write_damping(f("damp_f"), f("damp_i"), f("damp_f_bycol"),
                                     f("damp_i_bycol"), prob.m_d, prob.n, N.ptr(D.ptr),
                                     N.ptr(D.idx), N.ptr(D.val), N.ptr(DC.ptr), N.ptr(DC.idx),
                                     N.ptr(DC.val)), "write_damping")
    N.check(L.plsqr_io_write_rhs(f("b_k"), prob.m_k, N.ptr(prob.b_k)), "write_rhs")
    return dict(names, dir=str(d), row_k=prob.m_k, row_d=prob.m_d, col=prob.n)


def read_files(files: dict) -> Problem:
    """Load a problem from the reference's files with the native readers."""
    L = N.lib()
    d = Path(files["dir"])
    f = lambda k: str(d / files[k]).encode()
    m_k, m_d, n = int(files["row_k"]), int(files["row_d"]), int(files["col"])
    cnt = np.empty(n, np.int32)
    st = np.empty(n, np.int64)
    tot = N.i64(0)
    N.check(L.plsqr_io_read_kernel_info(f("ker_i"), n, N.ptr(cnt), N.ptr(st), C.byref(tot)),
            "read_kernel_info")
    kp = np.empty(n + 1, np.int64)
    kr = np.empty(tot.value, np.int32)
    kv = np.empty(tot.value, np.float64)
    N.check(L.plsqr_io_read_kernel(f("ker_f"), f("ker_i"), m_k, n, N.ptr(kp), N.ptr(kr),
                                   N.ptr(kv)), "read_kernel")
    rc_ = np.empty(m_d, np.int32)
    N.check(L.plsqr_io_read_int32_counts(f("damp_i"), m_d, N.ptr(rc_), C.byref(tot)),
            "read_damp_info")
    dp = np.empty(m_d + 1, np.int64)
    di = np.empty(tot.value, np.int32)
    dv = np.empty(tot.value, np.float64)
    N.check(L.plsqr_io_read_damping(f("damp_f"), 0, m_d, n, tot.value, N.ptr(dp), N.ptr(di),
                                    N.ptr(dv)), "read_damping_rows")
    cc = np.empty(n, np.int32)
    N.check(L.plsqr_io_read_int32_counts(f("damp_i_bycol"), n, N.ptr(cc), C.byref(tot)),
            "read_damp_col_info")
    cp = np.empty(n + 1, np.int64)
    cr = np.empty(tot.value, np.int32)
    cv = np.empty(tot.value, np.float64)
    N.check(L.plsqr_io_read_damping(f("damp_f_bycol"), 1, m_d, n, tot.value, N.ptr(cp),
                                    N.ptr(cr), N.ptr(cv)), "read_damping_cols")
    b = np.empty(m_k, np.float64)
    N.check(L.plsqr_io_read_rhs(f("b_k"), m_k, N.ptr(b)), "read_rhs")
    return Problem(Lines(kp, kr, kv, m_k, n), Lines(dp, di, dv, m_d, n),
                   Lines(cp, cr, cv, m_d, n), b, np.zeros(n), 0, {})
