"""gbqv_expval_pauli_many_noalloc: Pauli expectation values on a device
state for callers that cannot allocate device memory (a framework whose
allocator owns the GPU's memory, or a loop that must not pay cudaMalloc's
synchronisation).  Its partial sums live in a static __device__ array
instead of cudaMalloc'd scratch.  Checked against gbqv_expval_pauli_many on
the same state, on two calls in a row with different terms (the array keeps
the previous call's contents), and against the oracle's expval_pauli, within
the tolerance of the other expval tests.  This file sorts last so a failure here comes after every other test.
"""
import ctypes as C

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _terms(rng, n, count):
    out = []
    for _ in range(count):
        k = int(rng.integers(1, 6))
        q = [int(x) for x in rng.choice(n, k, replace=False)]
        out.append((q, "".join(rng.choice(list("IXYZ"), k))))
    return out


def _noalloc(qv, terms, coeffs, precision, offset_shift=0):
    P = pkg()
    L = P.lib()
    qs, offs, labels = [], [0], []
    for q, lab in terms:
        qs.extend(q)
        offs.append(len(qs))
        labels.append(lab.encode())
    offs = [o + offset_shift for o in offs]
    qa = np.ascontiguousarray(np.asarray(qs, dtype=np.uint64))
    oa = (C.c_int * len(offs))(*offs)
    la = (C.c_char_p * len(labels))(*labels)
    ca = np.ascontiguousarray(np.asarray(coeffs, dtype=np.float64))
    out = np.empty(len(terms), dtype=np.float64)
    total = C.c_double()
    rc = L.gbqv_expval_pauli_many_noalloc(C.c_void_p(qv.device_pointer()), qv.num_qubits(), 1 if precision == "double" else 0,
                                          len(terms), qa.ctypes.data_as(C.POINTER(C.c_uint64)), oa, la,
                                          ca.ctypes.data_as(C.POINTER(C.c_double)), C.c_void_p(qv.stream()),
                                          out.ctypes.data_as(C.POINTER(C.c_double)), C.byref(total))
    if rc != 0:
        raise P.GBQVError(rc, L.gbqv_last_error(None).decode())
    return out, total.value


@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("single", 5e-6)])
def test_noalloc_matches_expval_many_twice(precision, tol):
    P = pkg()
    rng = np.random.default_rng(4242)
    n = 16
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    with P.QubitVector(n, precision) as qv:
        qv.initialize_from_vector(psi)
        for count in (48, 7):  # the second call reuses the array with fewer terms
            terms = _terms(rng, n, count)
            coeffs = rng.normal(size=count)
            got, got_total = _noalloc(qv, terms, coeffs, precision)
            want, want_total = qv.expval_pauli_many(terms, coeffs)
            np.testing.assert_allclose(got, want, atol=tol, rtol=0)
            assert abs(got_total - want_total) < tol * 10
            # and directly against the oracle's expval_pauli on the same state
            o = O.OracleQV(n, data=psi)
            np.testing.assert_allclose(got, [o.expval_pauli(q, lab) for q, lab in terms], atol=tol, rtol=0)


def test_noalloc_rejects_too_many_terms():
    P = pkg()
    rng = np.random.default_rng(1)
    with P.QubitVector(8) as qv:
        qv.initialize()
        with pytest.raises(P.GBQVError) as e:
            _noalloc(qv, _terms(rng, 8, 65), np.ones(65), "double")
        assert e.value.code == 1 and "terms per call" in str(e.value)


def test_noalloc_rejects_nonzero_first_offset():
    """offsets[0] must be 0: a negative start would read before the caller's
    qubit array."""
    P = pkg()
    rng = np.random.default_rng(2)
    with P.QubitVector(8) as qv:
        qv.initialize()
        with pytest.raises(P.GBQVError) as e:
            _noalloc(qv, _terms(rng, 8, 3), np.ones(3), "double", offset_shift=-1)
        assert e.value.code == 1 and "offsets[0]" in str(e.value)
