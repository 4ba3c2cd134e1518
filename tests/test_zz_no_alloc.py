"""The host-buffer apply that allocates no device memory (qsi_op_apply_static).

It exists for callers whose process cannot make new device allocations, e.g.
when another allocator already owns the GPU's memory.  It must give the same
result as the ordinary host-pointer apply, call after call, since every call
reuses the same fixed staging arrays, and a call must leave the device's free
memory unchanged.  This file is collected last on purpose.
"""
import numpy as np
import pytest

import qsi_subspace_ed_gb300 as q
from qsi_subspace_ed_gb300 import workloads

pytestmark = pytest.mark.gpu


def _op():
    w = workloads.q0_32spin()
    return q.LazyOpSum(q.ZBasis(w.basis_lohi), w.hamiltonian())


def test_static_apply_reserves_no_device_memory():
    """A fresh operator (no ordinary apply before, so no staging buffers of its own): the first static calls and
    the ones after them leave the device's free memory unchanged."""
    import torch

    torch.cuda.init()
    op = _op()
    rng = np.random.default_rng(3)
    x = rng.standard_normal(op.rows())
    y = np.zeros_like(x)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        op.evaluate_static(x, y)
        op.evaluate_static(x, y, accumulate=True)
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, f"static applies changed free device memory by {free0 - free1} bytes"


def test_static_apply_matches_ordinary_apply_twice():
    op = _op()
    rng = np.random.default_rng(17)
    for call in range(2):
        x = rng.standard_normal(op.rows())
        y_ref = np.zeros_like(x)
        op.evaluate(x, y_ref)
        y = np.full_like(x, np.nan)  # stale contents must not leak into the result
        op.evaluate_static(x, y)
        np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max(), err_msg=f"call {call}")
    # accumulate: y += H x, twice in a row
    x = rng.standard_normal(op.rows())
    y0 = rng.standard_normal(op.rows())
    y_ref = y0.copy()
    op.evaluate_add(x, y_ref)
    y = y0.copy()
    op.evaluate_static(x, y, accumulate=True)
    np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())
    op.evaluate_add(x, y_ref)
    op.evaluate_static(x, y, accumulate=True)
    np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())


def test_static_apply_checks_its_arguments():
    op = _op()
    n = op.rows()
    good = np.zeros(n)
    for bad in (np.zeros(n, np.float32), np.zeros(n + 1), np.zeros(2 * n)[::2], [0.0] * n):
        with pytest.raises(ValueError):
            op.evaluate_static(bad, good)
        with pytest.raises(ValueError):
            op.evaluate_static(good, bad)


def test_static_apply_rejects_bases_above_the_limit():
    lat = workloads.lattice("pyro_1x2x2")
    basis = q.ZBasis(q.enumerate_basis(lat))  # 2,891,562 states > 262,144
    op = q.LazyOpSum(basis, q.build_ring_zeeman(lat, [1, .8, .6, .4], [0.1, 0.0, 0.0]))
    x = np.zeros(op.rows())
    y = np.zeros(op.rows())
    with pytest.raises(q.QsiError) as e:
        op.evaluate_static(x, y)
    assert e.value.status == q._lib.QSI_INVALID_ARG and "262144" in str(e.value)
