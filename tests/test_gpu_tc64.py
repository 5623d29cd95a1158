"""complex64 dense 4-qubit gates on tcgen05 in split precision (3xTF32, fp32
accumulation in TMEM) against the oracle (complex128) and against the fp32-FMA
kernel (tensor mode 0): one tile (11 qubits), two tiles, many tiles per CTA,
targets in the lowest and highest positions, zero groups, non-unitary
matrices, and exactness on a basis state through a permutation.  Tolerance:
the complex64 parity tolerance of the engine (fp32 arithmetic, 12 gates)."""
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
    with P.QubitVector(n, "single") as qv:
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
def test_tc64_sequences_against_oracle_and_fma(n):
    P = pkg()
    rng = np.random.default_rng(5000 + n)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    placements = [[0, 1, 2, 3], [3, 2, 1, 0], [n - 1, n - 2, n - 3, n - 4], [0, n - 1, 5, 2]]
    placements += [[int(x) for x in rng.choice(n, 4, replace=False)] for _ in range(8)]
    ops = [(q, haar(rng, 16)) for q in placements]
    got = run(P, n, psi, ops, 1)
    scale = np.max(np.abs(psi))
    np.testing.assert_allclose(got, oracle(n, psi, ops), atol=2e-6 * scale * 12, rtol=0)
    fma = run(P, n, psi, ops, 0)
    np.testing.assert_allclose(got, fma, atol=2e-6 * scale * 12, rtol=0)


def test_tc64_many_tiles_per_cta():
    P = pkg()
    rng = np.random.default_rng(21)
    n = 23
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    ops = [([int(x) for x in rng.choice(n, 4, replace=False)], haar(rng, 16)) for _ in range(6)]
    a = run(P, n, psi, ops, 1)
    b = run(P, n, psi, ops, 0)
    assert np.max(np.abs(a - b)) < 1e-5 * np.max(np.abs(psi))
    assert abs(np.linalg.norm(a) - 1.0) < 1e-5


def test_tc64_zero_groups_and_non_unitary():
    P = pkg()
    rng = np.random.default_rng(22)
    n = 13
    psi = np.zeros(1 << n, dtype=complex)
    idx = rng.choice(1 << n, 300, replace=False)
    psi[idx] = rng.normal(size=300) + 1j * rng.normal(size=300)
    m = haar(rng, 16) * 3.0
    m[:, 5] = 0
    m[7, :] = 0
    ops = [([7, 1, 4, 9], m), ([12, 0, 3, 6], haar(rng, 16) * 0.25)]
    want = oracle(n, psi, ops)
    np.testing.assert_allclose(run(P, n, psi, ops, 1), want, atol=1e-5 * np.max(np.abs(want)), rtol=0)


def test_tc64_basis_state_through_permutation_is_exact():
    P = pkg()
    n = 14
    psi = np.zeros(1 << n, dtype=complex)
    psi[12345] = 1.0
    perm = np.eye(16)[:, np.random.default_rng(3).permutation(16)].astype(complex)
    ops = [([0, 4, 8, 12], np.eye(16, dtype=complex)), ([1, 2, 3, 13], perm)]
    np.testing.assert_array_equal(run(P, n, psi, ops, 1), oracle(n, psi, ops))


@pytest.mark.parametrize("n", [12, 13, 16, 20])
def test_tc64_five_qubit_gates_against_oracle_and_fma(n):
    """5-qubit gates (K = 64 reals, N = 64 TMEM columns per lane, 2-stage raw
    ring of 32 KB tiles): every placement kind — all targets low, all high
    (the loader's 4-request descriptor), qubit 0 a target or not — against
    the oracle and the fp32-FMA kernel."""
    P = pkg()
    rng = np.random.default_rng(5100 + n)
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    placements = [[0, 1, 2, 3, 4], [4, 3, 2, 1, 0], [n - 1, n - 2, n - 3, n - 4, n - 5], [0, n - 1, 5, 2, 9],
                  [7, 8, 9, 10, 11], [1, 3, n - 2, 6, 8]]
    placements += [[int(x) for x in rng.choice(n, 5, replace=False)] for _ in range(6)]
    ops = [(q, haar(rng, 32)) for q in placements]
    got = run(P, n, psi, ops, 1)
    scale = np.max(np.abs(psi))
    np.testing.assert_allclose(got, oracle(n, psi, ops), atol=2e-6 * scale * 12, rtol=0)
    fma = run(P, n, psi, ops, 0)
    np.testing.assert_allclose(got, fma, atol=2e-6 * scale * 12, rtol=0)


def test_tc64_five_qubit_many_tiles_and_permutation_exact():
    """23 qubits (many tiles per CTA) against the FMA kernel, and a basis
    state through a 5-qubit permutation stays exact (hi * hi carries the 1s,
    the cross terms are zero)."""
    P = pkg()
    rng = np.random.default_rng(23)
    n = 23
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    ops = [([int(x) for x in rng.choice(n, 5, replace=False)], haar(rng, 32)) for _ in range(4)]
    a = run(P, n, psi, ops, 1)
    b = run(P, n, psi, ops, 0)
    assert np.max(np.abs(a - b)) < 1e-5 * np.max(np.abs(psi))
    perm = np.eye(32)[rng.permutation(32)]
    basis = np.zeros(1 << 14, dtype=complex)
    basis[12345] = 1.0
    q = [13, 2, 0, 7, 9]
    got = run(P, 14, basis, [(q, perm)], 1)
    np.testing.assert_array_equal(got, oracle(14, basis, [(q, perm)]))
