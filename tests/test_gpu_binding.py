"""The reference's LSQR loop driving the GPU operator through the aprod
signature (source/aprod.h:10-13), the binding a maintainer adds in place of
the reference's aprod.c (plsqr3.2013.09_gb300/integration/aprod_gpu.c).

The loop is the oracle's restatement of source/lsqr.c:195-917, bitwise
equal to the reference program on the golden runs; its operator is a
callback with aprod_gpu.c's per-call behaviour: the first call builds a GPU
context from the matrices the reference holds (kernel by column, damping by
row and by column), every call hands the reference's own host vectors to
plsqr_aprod_host (input copied to the device, the updated vector copied
back), and the final iteration's mode-2 call releases the context.  Two
calls per iteration (lsqr.c:507, 564) plus one at start-up (lsqr.c:366).

The result must match the reference's golden x, alpha_k and beta_k within
the FP64 path's bar (1e-10 relative)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden, rel

pytestmark = pytest.mark.gpu

TOL = 1e-10


def per_iter_rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


class GpuAprod:
    """aprod_gpu.c's aprod() over an OracleProblem's vectors."""

    def __init__(self, pkg, prob, o):
        self.pkg, self.prob, self.o = pkg, prob, o
        self.ctx = None
        self.calls = []
        self.contexts = 0

    def __call__(self, mode, m, n, is_final, iteration):
        assert m == self.prob.m_k + self.prob.m_d and n == self.prob.n
        if self.ctx is None:
            self.ctx = self.pkg.Context(self.prob)
            self.contexts += 1
        self.ctx.aprod_host(mode, self.o.y_k, self.o.y_d, self.o.x, iteration=iteration,
                            is_final=is_final)
        self.calls.append((mode, iteration, is_final))
        if is_final and mode == 2:
            self.ctx.close()
            self.ctx = None
        return 0


@pytest.mark.parametrize("case", ["tiny", "grid32"])
def test_reference_loop_with_gpu_aprod_matches_reference(case, pkg, orc, problems):
    g = golden(case)
    prob = problems(case)
    it = g["meta"]["iterations"]
    o = orc.OracleProblem(prob)
    op = GpuAprod(pkg, prob, o)
    out = o.lsqr(it, op=op)
    assert op.ctx is None and op.contexts == 1, "the final iteration releases the one context"
    assert op.calls[0] == (2, 0, 0)
    assert len(op.calls) == 1 + 2 * it
    assert op.calls[-2:] == [(1, it, 1), (2, it, 1)]
    assert rel(out["x"], g["x"]) <= TOL
    assert per_iter_rel(out["hist"]["alpha"], g["alpha"]) <= TOL
    assert per_iter_rel(out["hist"]["beta"], g["beta"]) <= TOL
    # and the same loop on the device through plsqr_lsqr
    with pkg.Context(prob) as ctx:
        dev = ctx.lsqr(lsqr_iteration=it)
    assert rel(dev["x"], out["x"]) <= TOL
