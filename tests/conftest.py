"""Shared fixtures.  Tests marked `gpu` need a CUDA device and the built
library; everything else runs on the CPU (the oracle, the file formats, the
generator, and the C ABI up to the first device call)."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(ROOT))

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
    config.addinivalue_line("markers", "slow: large problem sizes")


@pytest.fixture(scope="session")
def pkg():
    from importlib import util  # noqa: F401
    so = graft.PKG_DIR / "lib" / "libplsqr_gpu.so"
    if not so.exists():
        graft.build()
    return graft.load_package()


@pytest.fixture(scope="session")
def orc():
    o = graft.load_oracle()
    if not o.LIB_PATH.exists():
        o.build()
    return o


@pytest.fixture(scope="session")
def has_gpu(pkg):
    return pkg._native.device_count() > 0


@pytest.fixture(autouse=True)
def _gpu_guard(request):
    if request.node.get_closest_marker("gpu"):
        p = graft.load_package()
        if p._native.device_count() < 1:
            pytest.fail("test marked gpu but no CUDA device is visible")


def golden(case: str) -> dict:
    """A golden run of the reference program; x is None for the large cases,
    which keep its sha256 (meta["x_sha256"]) instead."""
    d = GOLDEN / case
    meta = json.loads((d / "meta.json").read_text())
    ab = np.loadtxt(d / "alpha_beta.txt")
    xf = d / "x.f64"
    return dict(dir=d, meta=meta, x=np.fromfile(xf, dtype=np.float64) if xf.exists() else None,
                alpha=ab[:, 1], beta=ab[:, 2], result_txt=(d / "result.txt").read_text())


@pytest.fixture(scope="session")
def problems(pkg):
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = pkg.generate(name)
        return cache[name]

    return get


def rel(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    d = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (d if d > 0 else 1.0))
