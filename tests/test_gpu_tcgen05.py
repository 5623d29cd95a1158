"""complex128 dense 4-qubit gates on tcgen05 (TMEM accumulators, warp-
specialised pipeline) against the oracle and against the same digit slices on
mma.sync (tensor mode 2): one tile (11 qubits), two tiles, many tiles per CTA
(every mbarrier phase of both pipeline lanes), zero groups, non-unitary
matrices, targets in the lowest positions and a wide dynamic range.  Bound:
1e-12 absolute against the oracle per test, as for every complex128 path."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def haar(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def run(P, n, psi, ops, mode):
    with P.QubitVector(n) as qv:
        qv.set_tensor_c128(mode)
        qv.initialize_from_vector(psi)
        for q, m in ops:
            qv.apply_matrix(q, m)
        return qv.copy_to_vector()


def oracle(n, psi, ops):
    o = O.OracleQV(n, psi)
    for q, m in ops:
        o.apply_matrix(q, m)
    return o.data


@pytest.mark.parametrize("n", [11, 12, 13, 17, 20])
def test_tcgen05_sequences_against_oracle(n):
    P = pkg()
    rng = np.random.default_rng(4000 + n)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    placements = [[0, 1, 2, 3], [3, 2, 1, 0], [n - 1, n - 2, n - 3, n - 4], [0, n - 1, 5, 2]]
    placements += [[int(x) for x in rng.choice(n, 4, replace=False)] for _ in range(8)]
    ops = [(q, haar(rng, 16)) for q in placements]
    got = run(P, n, psi, ops, 1)
    np.testing.assert_allclose(got, oracle(n, psi, ops), atol=1e-12, rtol=0)
    ref2 = run(P, n, psi, ops, 2)
    np.testing.assert_allclose(got, ref2, atol=5e-13, rtol=0)


def test_tcgen05_many_tiles_per_cta():
    """2^23 amplitudes = 4096 tiles: ~27 tiles per CTA, so both pipeline lanes
    cycle through many mbarrier phases; compared with the mma.sync path and
    checked for unitarity (the oracle is too slow at this size)."""
    P = pkg()
    rng = np.random.default_rng(11)
    n = 23
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    ops = [([int(x) for x in rng.choice(n, 4, replace=False)], haar(rng, 16)) for _ in range(6)]
    a = run(P, n, psi, ops, 1)
    b = run(P, n, psi, ops, 2)
    assert np.max(np.abs(a - b)) < 1e-12
    assert abs(np.linalg.norm(a) - 1.0) < 1e-12


def test_tcgen05_zero_groups_and_non_unitary():
    P = pkg()
    rng = np.random.default_rng(12)
    n = 13
    psi = np.zeros(1 << n, dtype=complex)
    idx = rng.choice(1 << n, 300, replace=False)
    psi[idx] = rng.normal(size=300) + 1j * rng.normal(size=300)
    m = haar(rng, 16) * 3.0
    m[:, 5] = 0
    m[7, :] = 0
    ops = [([7, 1, 4, 9], m), ([12, 0, 3, 6], haar(rng, 16) * 0.25)]
    np.testing.assert_allclose(run(P, n, psi, ops, 1), oracle(n, psi, ops), atol=1e-12, rtol=0)


def test_tcgen05_dynamic_range():
    """Groups mixing amplitudes ~1 with ~1e-12 and matrices with tiny entries:
    the error stays within the bound relative to each group's largest entry."""
    P = pkg()
    rng = np.random.default_rng(13)
    n = 12
    psi = (rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)) * 1e-12
    psi[rng.choice(1 << n, 64, replace=False)] = 1.0
    psi /= np.linalg.norm(psi)
    m = haar(rng, 16)
    m[np.abs(m) < 0.2] *= 1e-9
    ops = [([2, 5, 8, 11], m), ([0, 1, 10, 6], haar(rng, 16))]
    np.testing.assert_allclose(run(P, n, psi, ops, 1), oracle(n, psi, ops), atol=1e-12, rtol=0)


def test_tcgen05_basis_state_and_identity():
    """A basis state through an identity then a permutation matrix is
    reproduced exactly (digits of 1.0 and 0.0 are exact)."""
    P = pkg()
    n = 14
    psi = np.zeros(1 << n, dtype=complex)
    psi[12345] = 1.0
    perm = np.eye(16)[:, np.random.default_rng(3).permutation(16)].astype(complex)
    ops = [([0, 4, 8, 12], np.eye(16, dtype=complex)), ([1, 2, 3, 13], perm)]
    got = run(P, n, psi, ops, 1)
    np.testing.assert_array_equal(got, oracle(n, psi, ops))


def test_tensor_mode_argument_checked():
    P = pkg()
    with P.QubitVector(11) as qv:
        with pytest.raises(Exception):
            qv.set_tensor_c128(3)


@pytest.mark.parametrize("n,k", [(12, 2), (12, 3), (17, 2), (17, 3)])
def test_small_dense_gates_padded_onto_tcgen05(n, k):
    """complex128 2- and 3-qubit dense gates run as U (x) I on idle qubits
    through the 4-qubit kernel: same results as the oracle, including gates
    on the highest qubits (the padding then picks lower idle qubits)."""
    P = pkg()
    rng = np.random.default_rng(700 + 10 * n + k)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    placements = [list(range(n - k, n)), list(range(k)), [n - 1] + list(range(k - 1))]
    placements += [[int(x) for x in rng.choice(n, k, replace=False)] for _ in range(5)]
    ops = [(q, haar(rng, 1 << k)) for q in placements]
    got = run(P, n, psi, ops, 1)
    np.testing.assert_allclose(got, oracle(n, psi, ops), atol=1e-12, rtol=0)
