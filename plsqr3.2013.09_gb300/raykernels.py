"""Ray sensitivity kernels in their ASCII exchange format, and their
conversion into the kernel files PLSQR3 reads.

The reference's kernel_format tools take one ASCII file per ray, one line
per nonzero, "col ix iy iz value" with a 1-based column (the cell's index
(iz-1)*ny*nx + (iy-1)*nx + ix, plus the parameter field's offset):
ker_ascii2bin writes each line as a 16-byte record (PLSQR3_tools/
kernel_format/ker_ascii2bin.c:106-113), and Ker2PLSQR3 makes the kernel
matrix by column from the records of all rays, with row = the ray's 1-based
position in the list (Ker2PLSQR3.c:389, 587-608), each column's entries in
the order the rays were read, and the info file "col nnz start" (1-based,
"0 0" for an empty column, Ker2PLSQR3.c:499-513).  The same steps are
restated here on arrays; synth.write_files writes the result.

The reference's data/ sample is such a set: 100 rays of the Southern
California model, 99 x 153 x 10 cells and 2 parameter fields (302,940
columns), with its measurement vector and the damping matrix of
damping_binary.py with every weight 1.0 (data/README:1-27).  socal_problem
assembles it; socal_compact / socal_from_compact store and restore its
kernel rays losslessly in a small form.
"""
from __future__ import annotations

from pathlib import Path

import numpy as np

from . import synth as S

# data/README:1-5 and the damping_binary.py call of data/README:19
SOCAL_GRID = (99, 153, 10)
SOCAL_FIELDS = 2


def read_list(path: str | Path) -> list[str]:
    """A kernel list: the ray files in row order.  ker.list starts with the
    count of rays; ker_bin.list lines are "name nnz" (the first field is
    taken)."""
    lines = [ln.split() for ln in Path(path).read_text().splitlines() if ln.strip()]
    if len(lines[0]) == 1 and lines[0][0].isdigit() and int(lines[0][0]) == len(lines) - 1:
        lines = lines[1:]
    return [ln[0] for ln in lines]


def read_ascii_ray(path: str | Path) -> tuple[np.ndarray, np.ndarray]:
    """0-based columns and values of one ray file, in file order.  Values are
    parsed to the nearest double, as fscanf("%lf") does."""
    cols, vals = [], []
    with open(path) as f:
        for ln in f:
            p = ln.split()
            if len(p) < 5:
                continue
            cols.append(int(p[0]) - 1)
            vals.append(float(p[4]))
    return np.asarray(cols, np.int32), np.asarray(vals, np.float64)


def kernel_by_column(rays: list[tuple[np.ndarray, np.ndarray]], n: int) -> S.Lines:
    """The kernel matrix by column from the rays (row i = rays[i]): within a
    column the entries of lower rows first, and a row's entries in its file
    order (Ker2PLSQR3.c:419-429 appends them so)."""
    m = len(rays)
    rows = np.concatenate([np.full(len(c), i, np.int32) for i, (c, _) in enumerate(rays)]) \
        if m else np.zeros(0, np.int32)
    cols = np.concatenate([c for c, _ in rays]) if m else np.zeros(0, np.int32)
    vals = np.concatenate([v for _, v in rays]) if m else np.zeros(0)
    if cols.size and (cols.min() < 0 or cols.max() >= n):
        raise ValueError(f"a ray column lies outside 1..{n}")
    order = np.argsort(cols, kind="stable")
    ptr = np.zeros(n + 1, np.int64)
    np.add.at(ptr, cols.astype(np.int64) + 1, 1)
    np.cumsum(ptr, out=ptr)
    return S.Lines(ptr, rows[order].copy(), vals[order].copy(), m, n)


def damping(grid=SOCAL_GRID, fields=SOCAL_FIELDS, weights=(1.0, 1.0, 1.0)):
    """D by row and by column as damping_binary.py makes them: identity,
    xx, yy, zz and the xy, xz, yz cross rows per cell, fields repeated.
    weights = (identity, second difference, cross)."""
    nx, ny, nz = grid
    p = S.params(dict(nx=nx, ny=ny, nz=nz, n_rays=0, damp_identity=weights[0],
                      damp_lap=weights[1], damp_cross=weights[2], n_params=fields))
    return S.damping_from_params(p)


def socal_problem(data_dir: str | Path, n_rays: int | None = None) -> S.Problem:
    """The reference's data/ sample (or its first n_rays rays) as a Problem:
    kernel rows from ker.list and ker_ASCII/, b_k from measure_fake.list, the
    damping matrix with every weight 1.0."""
    d = Path(data_dir)
    names = read_list(d / "ker.list")[: n_rays]
    rays = [read_ascii_ray(d / "ker_ASCII" / nm) for nm in names]
    return socal_from_rays(rays, np.loadtxt(d / "measure_fake.list")[: len(rays)])


def socal_from_rays(rays, b_k) -> S.Problem:
    nx, ny, nz = SOCAL_GRID
    n = nx * ny * nz * SOCAL_FIELDS
    k = kernel_by_column(rays, n)
    d_csr, d_csc = damping()
    meta = dict(grid=SOCAL_GRID, fields=SOCAL_FIELDS, n_rays=len(rays), nnz_k=k.nnz,
                nnz_d=d_csr.nnz, source="reference data/ sample")
    return S.Problem(k, d_csr, d_csc, np.asarray(b_k, np.float64).copy(), np.zeros(n), 100, meta)


# ---- lossless compact form of the rays ------------------------------------------
# Every value of the sample is printed with 7 significant digits ("%e"), so a
# value is an integer mantissa m (|m| < 10^7) and a decimal exponent q with
# value = m * 10^(q - 6); the double parsed from "<m>e<q-6>" equals the one
# parsed from the original text (both are the nearest double to the same
# decimal).  Columns are stored as differences within each ray.

def socal_compact(rays) -> dict:
    cols, mant, expo, lens = [], [], [], []
    for c, v in rays:
        lens.append(len(c))
        d = np.diff(c.astype(np.int64), prepend=0)
        cols.append(d.astype(np.int32))
        text = [f"{x:.6e}" for x in v]
        mm = np.array([int(t.split("e")[0].replace(".", "")) for t in text], np.int64)
        qq = np.array([int(t.split("e")[1]) for t in text], np.int64)
        back = np.array([float(f"{a}e{b - 6}") for a, b in zip(mm, qq)])
        if not np.array_equal(back, v):
            raise ValueError("a value has more than 7 significant digits")
        mant.append(mm.astype(np.int32))
        expo.append(qq.astype(np.int8))
    return dict(lens=np.asarray(lens, np.int64), dcol=np.concatenate(cols),
                mant=np.concatenate(mant), expo=np.concatenate(expo))


def socal_from_compact(z) -> list[tuple[np.ndarray, np.ndarray]]:
    lens = np.asarray(z["lens"], np.int64)
    off = np.concatenate([[0], np.cumsum(lens)])
    rays = []
    for i in range(len(lens)):
        a, b = off[i], off[i + 1]
        c = np.cumsum(np.asarray(z["dcol"][a:b], np.int64)).astype(np.int32)
        v = np.array([float(f"{m}e{q - 6}") for m, q in zip(z["mant"][a:b].tolist(),
                                                              z["expo"][a:b].tolist())])
        rays.append((c, v))
    return rays
