"""Operator sizes beyond the small-matrix kernels, against the oracle:
probabilities(qubits) over 11..n qubits in any order (statevector and
density-matrix diagonal), apply_matrix on 11..13 qubits and
norm(qubits, mat) on 6..11 qubits (QubitVector::probabilities,
qubitvector.hpp:2106-2143; apply_matrix, transformer.hpp:89-232;
norm(qubits, mat), qubitvector.hpp:1878-2082)."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL = {"double": 1e-12, "single": 2e-6}


def _state(rng, n):
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return psi / np.linalg.norm(psi)


def _unitary(rng, k):
    z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("k", [11, 13, 16])
def test_probabilities_wide_statevector(precision, k):
    P = pkg()
    rng = np.random.default_rng(100 + k)
    n = 16
    psi = _state(rng, n)
    qubits = [int(x) for x in rng.permutation(n)[:k]]
    with P.QubitVector(n, precision) as qv:
        qv.initialize_from_vector(psi)
        got = qv.probabilities(qubits)
    want = O.OracleQV(n, data=psi).probabilities(qubits)
    assert got.shape == (1 << k,)
    np.testing.assert_allclose(got, want, atol=TOL[precision] * 4, rtol=0)
    assert abs(got.sum() - 1) < (1e-10 if precision == "double" else 1e-5)


def test_probabilities_wide_density_matrix():
    P = pkg()
    rng = np.random.default_rng(7)
    n = 11
    a = rng.normal(size=(1 << n, 4)) + 1j * rng.normal(size=(1 << n, 4))
    rho = a @ a.conj().T
    rho /= np.trace(rho)
    qubits = [int(x) for x in rng.permutation(n)]
    with P.DensityMatrix(n) as dm:
        dm.initialize_from_matrix(rho)
        got = dm.probabilities(qubits)
    want = O.OracleDM(n, data=rho.reshape(-1, order="F")).probabilities(qubits)
    np.testing.assert_allclose(got, want, atol=1e-12, rtol=0)


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("k", [11, 13])
def test_apply_matrix_wide(precision, k):
    P = pkg()
    rng = np.random.default_rng(200 + k)
    n = 15
    psi = _state(rng, n)
    qubits = [int(x) for x in rng.permutation(n)[:k]]
    u = _unitary(rng, k)
    with P.QubitVector(n, precision) as qv:
        qv.initialize_from_vector(psi)
        qv.apply_matrix(qubits, u)
        got = qv.copy_to_vector()
    o = O.OracleQV(n, data=psi)
    o.apply_matrix(qubits, u)
    np.testing.assert_allclose(got, o.data, atol=TOL[precision] * 10, rtol=0)


@pytest.mark.parametrize("k", [6, 11])
def test_norm_matrix_wide(k):
    P = pkg()
    rng = np.random.default_rng(300 + k)
    n = 14
    psi = _state(rng, n)
    qubits = [int(x) for x in rng.permutation(n)[:k]]
    m = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        got = qv.norm(qubits, m)
        after = qv.copy_to_vector()
    want = O.OracleQV(n, data=psi).norm_matrix(qubits, m)
    assert abs(got - want) <= 1e-12 * max(1.0, abs(want)), (got, want)
    np.testing.assert_array_equal(after, psi)  # the state is left as it is
