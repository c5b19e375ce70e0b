"""Host side of the warm start: the model class and the column norms (no GPU)."""
from __future__ import annotations

import numpy as np
import pytest


def test_model_instances_are_seeded(pkg):
    a = pkg.warm.model_instance((16, 12, 8), 3)
    b = pkg.warm.model_instance((16, 12, 8), 3)
    c = pkg.warm.model_instance((16, 12, 8), 4)
    assert a.shape == (16 * 12 * 8,) and np.array_equal(a, b) and not np.array_equal(a, c)
    assert np.all(np.isfinite(a)) and np.abs(a).max() > 0.1


def test_column_norms(pkg):
    prob = pkg.generate("tiny")
    cn = pkg.warm.column_norms2(prob)
    for L in (prob.k_csc, prob.d_csc):
        assert L.ptr[-1] == L.nnz
    ref = np.zeros(prob.n)
    for L in (prob.k_csc, prob.d_csc):
        for c in range(prob.n):
            v = L.val[L.ptr[c]:L.ptr[c + 1]]
            ref[c] += v @ v
    assert np.allclose(cn, ref, rtol=1e-14, atol=0)


def test_torch_ops_register_and_check_their_tensors(pkg):
    torch = pytest.importorskip("torch")
    ops = pkg.warm.torch_ops()
    assert pkg.warm.torch_ops() is ops
    with pytest.raises(ValueError):
        ops.unet_predict(0, torch.zeros(8))
