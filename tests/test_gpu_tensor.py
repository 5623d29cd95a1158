"""complex128 dense 4/5-qubit gates on the tensor cores (exact digit slices)
against the oracle and against the native-FP64 kernel: every gate within
1e-12 of the oracle, including target qubits in the lowest positions,
partial tiles (small n), a dominant-amplitude state and long sequences."""
import itertools

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def haar(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("n", [5, 6, 9, 14, 21])
@pytest.mark.parametrize("k", [4, 5])
def test_tensor_gate_sequences(n, k):
    if k > n:
        pytest.skip("gate larger than the register")
    P = pkg()
    rng = np.random.default_rng(100 * n + k)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    o = O.OracleQV(n, psi)
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        placements = [list(range(k)), list(range(n - k, n))[::-1]]
        placements += [[int(x) for x in rng.choice(n, k, replace=False)] for _ in range(10)]
        for q in placements:
            m = haar(rng, 1 << k)
            qv.apply_matrix(q, m)
            o.apply_matrix(q, m)
        np.testing.assert_allclose(qv.copy_to_vector(), o.data, atol=1e-12, rtol=0)


def test_tensor_matches_fp64_kernel_from_basis_state():
    P = pkg()
    rng = np.random.default_rng(7)
    n = 18
    ops = [([int(x) for x in rng.choice(n, 4, replace=False)], haar(rng, 16)) for _ in range(30)]
    outs = []
    for tensor in (True, False):
        with P.QubitVector(n) as qv:
            qv.set_tensor_c128(tensor)
            qv.initialize()
            for q, m in ops:
                qv.apply_matrix(q, m)
            outs.append(qv.copy_to_vector())
    o = O.OracleQV(n)
    for q, m in ops:
        o.apply_matrix(q, m)
    np.testing.assert_allclose(outs[1], o.data, atol=1e-13)
    np.testing.assert_allclose(outs[0], o.data, atol=1e-12)
    assert abs(np.linalg.norm(outs[0]) - 1.0) < 1e-12


def test_tensor_non_unitary_and_zero_columns():
    """Projector-like and scaled matrices, zero groups (flushed to zero exactly)."""
    P = pkg()
    rng = np.random.default_rng(9)
    n = 10
    psi = np.zeros(1 << n, dtype=complex)
    psi[rng.choice(1 << n, 40, replace=False)] = rng.normal(size=40) + 1j * rng.normal(size=40)
    m = haar(rng, 16) * 3.0
    m[:, 5] = 0
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        qv.apply_matrix([7, 1, 4, 9], m)
        o = O.OracleQV(n, psi)
        o.apply_matrix([7, 1, 4, 9], m)
        np.testing.assert_allclose(qv.copy_to_vector(), o.data, atol=1e-12)


@pytest.mark.parametrize("n", [12, 13, 16, 20, 23])
def test_five_qubit_tcgen05_against_oracle_and_fp64(n):
    """5-qubit complex128 gates on the tcgen05 kernel (two K-halves split by
    the highest target, two output-half accumulators): placements with the
    highest target above the tile's runs (the kernel's case), all targets
    high, qubit 0 a target, and one placement the kernel leaves to the
    warp-level form (every target below 12); against the oracle (1e-12) and
    the FP64-core kernel."""
    P = pkg()
    rng = np.random.default_rng(500 + n)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    placements = [[0, 1, 2, 3, n - 1], [n - 1, n - 2, n - 3, n - 4, n - 5], [n - 1, 0, 5, 2, 9],
                  [n - 2, 3, 7, 1, n - 1], [0, 1, 2, 3, 4]]
    placements += [[int(x) for x in rng.choice(n, 5, replace=False)] for _ in range(6)]
    ops = [(q, haar(rng, 32)) for q in placements]
    o = O.OracleQV(n, psi)
    for q, m in ops:
        o.apply_matrix(q, m)
    outs = []
    for mode in (1, 0):
        with P.QubitVector(n) as qv:
            qv.set_tensor_c128(mode)
            qv.initialize_from_vector(psi)
            for q, m in ops:
                qv.apply_matrix(q, m)
            outs.append(qv.copy_to_vector())
    np.testing.assert_allclose(outs[0], o.data, atol=1e-12, rtol=0)
    np.testing.assert_allclose(outs[0], outs[1], atol=1e-12, rtol=0)


def test_five_qubit_tcgen05_zero_groups_and_exact_permutation():
    """Sparse state (all-zero groups are skipped on store) and a 5-qubit
    permutation on a basis state, which the digit slices carry exactly."""
    P = pkg()
    rng = np.random.default_rng(77)
    n = 14
    psi = np.zeros(1 << n, dtype=complex)
    idx = rng.choice(1 << n, 200, replace=False)
    psi[idx] = rng.normal(size=200) + 1j * rng.normal(size=200)
    m = haar(rng, 32) * 2.0
    m[:, 3] = 0
    ops = [([13, 1, 4, 9, 2], m), ([12, 0, 3, 6, 7], haar(rng, 32) * 0.5)]
    o = O.OracleQV(n, psi)
    for q, mm in ops:
        o.apply_matrix(q, mm)
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        for q, mm in ops:
            qv.apply_matrix(q, mm)
        np.testing.assert_allclose(qv.copy_to_vector(), o.data, atol=1e-12 * max(1.0, np.max(np.abs(o.data))),
                                   rtol=0)
    perm = np.eye(32)[rng.permutation(32)]
    basis = np.zeros(1 << n, dtype=complex)
    basis[9999] = 1.0
    q = [13, 2, 0, 7, 9]
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(basis)
        qv.apply_matrix(q, perm)
        got = qv.copy_to_vector()
    o = O.OracleQV(n, basis)
    o.apply_matrix(q, perm)
    np.testing.assert_array_equal(got, o.data)
