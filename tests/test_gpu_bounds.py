"""The bounds-checked build of the library (-DPLSQR_CHECK): its unit-layout
kernels check every slot, gather index, line and lane they touch, record a
failed check and skip the access.  A child process loads that build
(PLSQR_LIB), runs the FP64 and mixed-precision products and solves on
problems shaped for the layout's edge cases, under the launch shapes the
switches select, and the batched solver's k-wide unit products on blocks of
4, 8 and 32 (passes of 8 columns), and reads the flags: no check may fail and every result is
finite."""
from __future__ import annotations

import json
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r"""
import json, os, sys, importlib.util
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, os.path.join(sys.argv[1], "tests"))
import numpy as np
import __graft_entry__ as g
pkg = g.load_package()
N = pkg._native
spec = importlib.util.spec_from_file_location("units_t", os.path.join(sys.argv[1], "tests", "test_gpu_units.py"))
ut = importlib.util.module_from_spec(spec)
spec.loader.exec_module(ut)
checked, _ = N.check_flags(reset=True)
probs = {"tiny": pkg.generate("tiny"), "grid32": pkg.generate("grid32")}
for name, (rl, n) in ut.SHAPES.items():
    probs[name] = ut.problem(pkg, rl, n, seed=len(rl))
envs = [{}, {"PLSQR_SLAB_SIZE": "1024", "PLSQR_UNIT_SIZE_F": "1024"},
        {"PLSQR_UNIT_THREADS": "512", "PLSQR_SLAB_SIZE": "12288", "PLSQR_UNIT_SIZE_F": "12288"},
        {"PLSQR_UNIT_LINES": "8", "PLSQR_UNIT_BANKS": "1"}]
out = {"checked": checked, "runs": []}
vu = next(v for v in range(64) if N.batch_variant(v)[1] < 0)
rng = np.random.default_rng(1)
for env in envs:
    for k in ("PLSQR_SLAB_SIZE", "PLSQR_UNIT_SIZE_F", "PLSQR_UNIT_THREADS", "PLSQR_UNIT_LINES",
              "PLSQR_UNIT_BANKS"):
        os.environ.pop(k, None)
    os.environ.update(env)
    for name, p in probs.items():
        with pkg.Context(p) as c:
            x64 = c.lsqr(lsqr_iteration=30)["x"]
            yk, yd, x = rng.standard_normal(p.m_k), rng.standard_normal(p.m_d), rng.standard_normal(p.n)
            c.aprod_host(1, yk, yd, x)
            c.aprod_host(2, yk, yd, x)
        with pkg.Context(p, precision="mixed") as cm:
            xm = cm.lsqr(sweeps=1, inner=30)["x"]
        # the batched solver's units form: blocks of 4, 8 and 32 (passes of 8)
        with pkg.Context(p) as cb:
            for kk in (3, 8, 20):
                bb = np.stack([p.b_k * (1.0 + 0.1 * t) for t in range(kk)])
                xb = cb.batch_lsqr(bb, sweeps=1, inner=10, variant_rows=vu, variant_cols=vu)["x"]
                x = np.concatenate([x, xb.ravel()])
        out["runs"].append({"env": env, "case": name, "flags": N.check_flags(reset=True)[1],
                            "finite": bool(np.all(np.isfinite(x64)) and np.all(np.isfinite(xm))
                                           and np.all(np.isfinite(yk)) and np.all(np.isfinite(x)))})
print(json.dumps(out))
"""


def test_checked_build_finds_no_out_of_bounds_access(pkg):
    spec_build = ROOT / "plsqr3.2013.09_gb300" / "build.py"
    import importlib.util
    spec = importlib.util.spec_from_file_location("plsqr_build_check", spec_build)
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    so = b.build(check=True)
    env = dict(os.environ, PLSQR_LIB=str(so))
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], env=env, capture_output=True,
                       text=True, timeout=1800)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res["checked"], "the child did not load the bounds-checked build"
    bad = [run for run in res["runs"] if run["flags"] or not run["finite"]]
    assert not bad, bad
    assert len(res["runs"]) == 4 * 5
