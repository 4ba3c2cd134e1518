"""The reference-side adaptor's C-ABI calls on the GPU.

include/gb300_lazy_op.hpp (GB300LazyOpSum) needs the reference's operator.hpp, which only the build container
has, so tests/test_host.py runs it there, against the reference's own operator code, and records the qsi_term
array it hands to the library (tests/golden/adaptor_terms_q0_32.bin).  Here the adaptor's calls are made with that
array, argument for argument: qsi_basis_create(lohi, n, 0), qsi_op_create(terms), then qsi_op_apply with host
pointers and accumulate 0 (evaluate, LazyOpSumProd::perform_op) and 1 (evaluate_add, projED::RealApplyFn), and
the results are compared with the reference's stored apply of the same Hamiltonian.
"""
import ctypes as C

import numpy as np
import pytest

import qsi_subspace_ed_gb300 as q
from qsi_subspace_ed_gb300 import _lib, workloads
from helpers import GOLDEN

pytestmark = pytest.mark.gpu


def test_adaptor_calls_reproduce_the_reference_apply():
    lib = q.load()
    w = workloads.q0_32spin()
    lohi = np.ascontiguousarray(w.basis_lohi, dtype=np.uint64)
    raw = (GOLDEN / "adaptor_terms_q0_32.bin").read_bytes()
    n_terms = len(raw) // C.sizeof(_lib.Term)
    terms = (_lib.Term * n_terms).from_buffer_copy(raw)
    x, y_ref = np.load(GOLDEN / "apply_q0_32.npy")
    qb, op = C.c_void_p(), C.c_void_p()
    _lib.check(lib.qsi_basis_create(lohi.ctypes.data_as(C.c_void_p), len(lohi), 0, C.byref(qb)))
    try:
        _lib.check(lib.qsi_op_create(qb, C.cast(terms, C.c_void_p), n_terms, C.byref(op)))
        try:
            y = np.zeros(len(lohi))
            _lib.check(lib.qsi_op_apply(op, x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), 0,
                                        _lib.QSI_PTR_HOST, None))
            np.testing.assert_allclose(y, y_ref, rtol=0, atol=1e-12 * np.abs(y_ref).max())
            _lib.check(lib.qsi_op_apply(op, x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), 1,
                                        _lib.QSI_PTR_HOST, None))
            np.testing.assert_allclose(y, 2 * y_ref, rtol=0, atol=2e-12 * np.abs(y_ref).max())
        finally:
            lib.qsi_op_destroy(op)
    finally:
        lib.qsi_basis_destroy(qb)
