"""The tuning switches (environment variables read when a context is
created) select other layouts and launch shapes of the same products; each
one must keep the FP64 solve within 1e-10 of the reference's golden run and
the mixed solve within 1e-6 of the FP64 solution."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu

LSQR_TOL = 1e-10


def per_iter_rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


FP64_CASES = [
    {"PLSQR_SLABS": "0"},                                   # per-line products (k_aprod1/2)
    {"PLSQR_SLABS": "0", "PLSQR_M2_BLOCKS_PER_SM": "3"},
    {"PLSQR_SLABS": "2"},                                   # k_aprod1 for A x, units for A^T y
    {"PLSQR_SLAB_SIZE": "1024"},                            # many slabs, short segments
    {"PLSQR_SLAB_SIZE": "28672"},                           # units do not fit: slab kernels
    {"PLSQR_SLAB_UNITS": "0"},                              # slab kernels, persistent
    {"PLSQR_SLAB_UNITS": "0", "PLSQR_SLAB_SCHED": "0"},     # slab kernels, static blocks
    {"PLSQR_SLAB_UNITS": "0", "PLSQR_SLAB_SIZE": "1024"},
    {"PLSQR_SLAB_UNITS": "0", "PLSQR_SLAB_GROUP": "4"},
    {"PLSQR_SLAB_UNITS": "0", "PLSQR_SLAB_GROUP": "16"},
    {"PLSQR_SLAB_UNITS": "0", "PLSQR_SLAB_GROUP": "32"},
    {"PLSQR_SLAB_UNITS": "0", "PLSQR_SLAB_CHUNK": "1"},
    {"PLSQR_SLAB_UNITS": "0", "PLSQR_SLAB_SCHED": "0", "PLSQR_SLAB_BLOCKS": "7"},
    {"PLSQR_SLABS": "2", "PLSQR_UNROLL": "1"},
    {"PLSQR_SLABS": "2", "PLSQR_UNROLL": "4"},
    {"PLSQR_SLABS": "2", "PLSQR_BLOCKS_PER_SM": "1"},
    {"PLSQR_UNIT_THREADS": "512", "PLSQR_SLAB_SIZE": "12288"},  # two unit blocks per SM
    {"PLSQR_UNIT_CHAINS": "4"},                              # four accumulator chains
    {"PLSQR_UNIT_BANKS": "1"},                               # bank-aware entry order
    {"PLSQR_UNIT_LINES": "8"},                               # short units
    {"PLSQR_NATURAL_ORDER": "1", "PLSQR_SLABS": "0"},
]


@pytest.mark.parametrize("env", FP64_CASES, ids=lambda e: ",".join(f"{k}={v}" for k, v in e.items()))
def test_fp64_switches_match_reference(env, pkg, problems, monkeypatch):
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    g = golden("grid32")
    prob = problems("grid32")
    it = g["meta"]["iterations"]
    with pkg.Context(prob) as ctx:
        out = ctx.lsqr(lsqr_iteration=it)
    assert rel(out["x"], g["x"]) <= LSQR_TOL
    assert per_iter_rel(out["hist"]["alpha"], g["alpha"]) <= LSQR_TOL
    assert per_iter_rel(out["hist"]["beta"], g["beta"]) <= LSQR_TOL


MIXED_CASES = [
    {},                                                     # FP32 units, hi + lo mirrors (default)
    {"PLSQR_MIXED_F32VEC": "1"},                            # FP32 vectors (no lo halves)
    {"PLSQR_UNIT_SIZE_F": "1024"},                          # many slabs, short segments
    {"PLSQR_UNIT_SIZE_F": "12288", "PLSQR_UNIT_THREADS": "512"},  # two blocks per SM
    {"PLSQR_UNIT_BANKS": "0"},                              # entries in fill order
    {"PLSQR_MIXED_HILO": "0"},                              # the FP32 mirror alone
    {"PLSQR_MIXED_HILO": "0", "PLSQR_UNIT_BANKS": "1"},
    {"PLSQR_MIXED_HILO": "0", "PLSQR_UNIT_SIZE_F": "24576", "PLSQR_UNIT_THREADS": "512"},
    {"PLSQR_MIXED_UNITS": "0"},                             # FP32 slab kernels
    {"PLSQR_MIXED_UNITS": "0", "PLSQR_MIXED_F32VEC": "1"},
    {"PLSQR_MIXED_UNITS": "0", "PLSQR_SLAB_SIZE_F": "1024"},
    {"PLSQR_MIXED_UNITS": "0", "PLSQR_SLAB_GROUP_F": "4"},  # transposed chunks of other widths
    {"PLSQR_MIXED_UNITS": "0", "PLSQR_SLAB_GROUP_F": "8"},
    {"PLSQR_MIXED_UNITS": "0", "PLSQR_SLAB_GROUP_F": "32"},
    {"PLSQR_SLABS": "0"},
]


@pytest.mark.parametrize("env", MIXED_CASES, ids=lambda e: ",".join(f"{k}={v}" for k, v in e.items()))
def test_mixed_switches_reach_the_fp64_solution(env, pkg, problems, monkeypatch):
    prob = problems("grid32")
    with pkg.Context(prob) as c64:
        xstar = c64.lsqr(lsqr_iteration=400)["x"]
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    with pkg.Context(prob, precision="mixed") as cm:
        out = cm.lsqr(sweeps=5, inner=60)
    assert rel(out["x"], xstar) <= 1e-6
