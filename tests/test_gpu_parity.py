"""Randomised parity of the engine (GPU, through the C ABI) against the
oracle (oracle/oracle_qv.c) on seeded inputs: every qubit placement for
k <= 3 at small n, all op kinds, reductions, bit-exact sampling, checkpoint
and inner product, and size-independent properties at larger n."""
import itertools

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def rand_state(rng, n):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def haar(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8])
def test_dense_every_placement(n):
    P = pkg()
    rng = np.random.default_rng(n)
    psi = rand_state(rng, n)
    with P.QubitVector(n) as qv:
        o = O.OracleQV(n, psi)
        qv.initialize_from_vector(psi)
        for k in range(1, min(n, 3) + 1):
            for q in itertools.permutations(range(n), k):
                m = haar(rng, 1 << k)
                qv.apply_matrix(list(q), m)
                o.apply_matrix(list(q), m)
        np.testing.assert_allclose(qv.copy_to_vector(), o.data, atol=1e-12)


@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("single", 5e-5)])
@pytest.mark.parametrize("n", [6, 11, 14, 17])
def test_random_ops(precision, tol, n):
    P = pkg()
    rng = np.random.default_rng(1000 + n)
    psi = rand_state(rng, n)
    with P.QubitVector(n, precision) as qv:
        o = O.OracleQV(n, psi)
        qv.initialize_from_vector(psi)
        for step in range(80):
            kind = rng.integers(0, 9)
            if kind <= 2:
                k = int(rng.integers(1, min(n, 6) + 1))
                q = [int(x) for x in rng.choice(n, k, replace=False)]
                m = haar(rng, 1 << k)
                qv.apply_matrix(q, m); o.apply_matrix(q, m)
            elif kind == 3:
                k = int(rng.integers(1, min(n, 5) + 1))
                q = [int(x) for x in rng.choice(n, k, replace=False)]
                d = np.exp(1j * rng.uniform(0, 6, 1 << k))
                qv.apply_diagonal_matrix(q, d); o.apply_diagonal_matrix(q, d)
            elif kind == 4:
                k = int(rng.integers(1, min(n, 4) + 1))
                q = [int(x) for x in rng.choice(n, k, replace=False)]
                g = rng.integers(0, 3)
                if g == 0:
                    qv.apply_mcx(q); o.apply_mcx(q)
                elif g == 1:
                    qv.apply_mcy(q); o.apply_mcy(q)
                else:
                    ph = np.exp(1j * rng.uniform(0, 6))
                    qv.apply_mcphase(q, ph); o.apply_mcphase(q, ph)
            elif kind == 5 and n >= 2:
                k = int(rng.integers(2, min(n, 4) + 1))
                q = [int(x) for x in rng.choice(n, k, replace=False)]
                qv.apply_mcswap(q); o.apply_mcswap(q)
            elif kind == 6:
                k = int(rng.integers(1, min(n, 3) + 1))
                q = [int(x) for x in rng.choice(n, k, replace=False)]
                m = haar(rng, 2)
                qv.apply_mcu(q, m); o.apply_mcu(q, m)
            elif kind == 7:
                k = int(rng.integers(1, min(n, 6) + 1))
                q = [int(x) for x in rng.choice(n, k, replace=False)]
                lab = "".join(rng.choice(list("IXYZ"), k))
                c = np.exp(1j * rng.uniform(0, 6))
                qv.apply_pauli(q, lab, c); o.apply_pauli(q, lab, c)
            else:
                axis = int(rng.integers(0, 7))
                k = 1 if axis < 3 else 2
                q = [int(x) for x in rng.choice(n, k, replace=False)] if n >= k else None
                if q is None:
                    continue
                th = rng.uniform(-3, 3)
                qv.apply_rotation(q, axis, th); o.apply_rotation(q, axis, th)
        np.testing.assert_allclose(qv.copy_to_vector(), o.data, atol=tol * 4)
        # reductions on the same state
        assert abs(qv.norm() - o.norm()) < tol * 8
        for _ in range(6):
            k = int(rng.integers(1, min(n, 6) + 1))
            q = [int(x) for x in rng.choice(n, k, replace=False)]
            lab = "".join(rng.choice(list("IXYZ"), k))
            assert abs(qv.expval_pauli(q, lab) - o.expval_pauli(q, lab)) < tol * 8
        for k in (1, 3, min(n, 7)):
            q = [int(x) for x in rng.choice(n, k, replace=False)]
            np.testing.assert_allclose(qv.probabilities(q), o.probabilities(q), atol=tol * 8)
        np.testing.assert_allclose(qv.probabilities(), o.probabilities(), atol=tol * 8)


@pytest.mark.parametrize("n", [4, 9, 12, 20])
def test_sampling_bit_exact(n):
    P = pkg()
    rng = np.random.default_rng(77 + n)
    psi = rand_state(rng, n)
    psi[: 1 << (n - 1)] *= 0.2
    psi /= np.linalg.norm(psi)
    rnds = P.uniforms(1234 + n, 5000)
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        got = qv.sample_measure(rnds)
    want = O.OracleQV(n, psi).sample_measure(rnds)
    np.testing.assert_array_equal(got, want)


def test_sampling_edges():
    """r beyond the total, zero-probability prefixes, a single basis state."""
    P = pkg()
    n = 11
    psi = np.zeros(1 << n, dtype=complex)
    psi[1500] = 1.0
    rnds = np.array([0.0, 0.5, 0.999999999, np.nextafter(1.0, 0.0)])
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        np.testing.assert_array_equal(qv.sample_measure(rnds), O.OracleQV(n, psi).sample_measure(rnds))
        assert qv.sample_measure([]).size == 0


def _grid_state(kind, n, rng):
    if kind == "gauss":
        return rand_state(rng, n)
    if kind == "uniform":
        return np.full(1 << n, 2.0 ** (-n / 2), dtype=complex)
    if kind == "dyadic":  # probabilities 2^-2k: ties on most grids of the running sums
        k = rng.integers(n // 2 + 2, n // 2 + 9, size=1 << n)
        psi = (2.0 ** -k) * rng.choice(np.array([1, -1, 1j, -1j]), size=1 << n)
        return psi * 2.0 ** np.floor(np.log2(1 / np.sum(np.abs(psi) ** 2)) / 2)  # total in (1/4, 1]
    psi = rand_state(rng, n) * (rng.random(1 << n) < 0.01)  # sparse
    return psi / np.linalg.norm(psi)


def _edge_uniforms(probs, isz, rng, count):
    """Uniforms on the reference's running sums (in-order accumulation, the
    block totals from 0 and the walk from the block prefix), one step below
    and one above them, plus random ones."""
    nb = 1 << isz
    blocks = probs.reshape(nb, -1)
    idxs = np.add.accumulate(blocks, axis=1)[:, -1]
    pre = np.concatenate([[0.0], np.add.accumulate(idxs)])[:-1]
    out = [rng.random(count)]
    for j in rng.integers(0, nb, size=6):
        walk = np.add.accumulate(np.concatenate([[pre[j]], blocks[j]]))[1:]
        v = walk[rng.integers(0, walk.size, size=count // 12)]
        out += [v, np.nextafter(v, 0.0), np.nextafter(v, 1.0)]
    r = np.concatenate(out)
    return r[(r >= 0) & (r < 1)]


@pytest.mark.parametrize("kind", ["gauss", "uniform", "dyadic", "sparse"])
@pytest.mark.parametrize("isz", [10, 3])
def test_sampling_grid_chains_bit_exact(kind, isz):
    """Long blocks (2^22 outcomes in 2^isz blocks): the block sums and the
    checkpointed walk run as grid-step chains; shots on and beside the
    reference's running sums equal the oracle's."""
    P = pkg()
    n = 22
    rng = np.random.default_rng(["gauss", "uniform", "dyadic", "sparse"].index(kind) * 16 + isz)
    psi = _grid_state(kind, n, rng)
    rnds = _edge_uniforms(np.abs(psi) ** 2, isz, rng, 1200)
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        qv.set_sample_measure_index_size(isz)
        got = qv.sample_measure(rnds)
    want = O.OracleQV(n, psi).sample_measure(rnds, index_size=isz)
    np.testing.assert_array_equal(got, want)


def _walk_samples(probs, rnds, isz):
    """QubitVector::sample_measure (qubitvector.hpp:2148-2228) for n >= the
    index size, restated with numpy's in-order accumulation over given
    probabilities (here a complex64 state's, products in float)."""
    END = probs.size
    L = END >> isz
    idxs = np.add.accumulate(probs.reshape(-1, L), axis=1)[:, -1]
    P = np.add.accumulate(np.concatenate([[0.0], idxs]))
    out = np.empty(rnds.size, dtype=np.uint64)
    walks = {}
    for i, r in enumerate(rnds):
        j = int(np.searchsorted(P[1:], r, side="right"))
        if j == idxs.size:
            out[i] = END
            continue
        if j not in walks:
            walks[j] = np.add.accumulate(np.concatenate([[P[j]], probs[j * L:(j + 1) * L]]))[1:]
        w = walks[j]
        k = int(np.searchsorted(w, r, side="right"))
        s = j * L + k
        if k == L:  # past the block's end: the walk goes on, one index at a time
            p = w[-1]
            s = (j + 1) * L
            while s < END - 1:
                p = p + probs[s]
                if r < p:
                    break
                s += 1
        out[i] = min(s, END - 1)
    return out


@pytest.mark.parametrize("kind", ["gauss", "sparse"])
@pytest.mark.parametrize("isz", [10, 3])
def test_sampling_grid_chains_complex64(kind, isz):
    """The same at complex64, whose probabilities (float products, widened)
    carry 24 bits: the block walk meets a tie on most steps, which the grid
    steps decide by prefix parities; shots equal the reference's walk over
    those probabilities."""
    P = pkg()
    n = 22
    rng = np.random.default_rng(["gauss", "sparse"].index(kind) * 16 + isz + 100)
    psi = _grid_state(kind, n, rng)
    with P.QubitVector(n, "single") as qv:
        qv.initialize_from_vector(psi)
        qv.set_sample_measure_index_size(isz)
        a = np.asarray(qv.copy_to_vector()).astype(np.complex64)
        probs = (a.real * a.real + a.imag * a.imag).astype(np.float64)
        rnds = _edge_uniforms(probs, isz, rng, 1200)
        got = qv.sample_measure(rnds)
    np.testing.assert_array_equal(got, _walk_samples(probs, rnds, isz))


def test_sampling_grid_chain_density_matrix():
    """Two chains over the 2^12 diagonal of a 12-qubit density matrix (index
    size 1), diagonal entries with rounding noise around zero."""
    P = pkg()
    n = 12
    rng = np.random.default_rng(5)
    a = rng.normal(size=(1 << n, 8)) + 1j * rng.normal(size=(1 << n, 8))
    rho = a @ a.conj().T
    rho /= np.trace(rho).real
    d = np.arange(1 << n)
    rho[d[::97], d[::97]] = -1e-19  # negative diagonal entries: added term by term
    vec = rho.reshape(-1, order="F")
    rnds = rng.random(3000)
    with P.DensityMatrix(n) as dm:
        dm.initialize_from_vector(vec)
        dm.set_sample_measure_index_size(1)
        got = dm.sample_measure(rnds)
    want = O.OracleDM(n, vec).sample_measure(rnds, index_size=1)
    np.testing.assert_array_equal(got, want)


def test_checkpoint_inner_product():
    P = pkg()
    rng = np.random.default_rng(2)
    n = 10
    psi = rand_state(rng, n)
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        qv.checkpoint()
        m = haar(rng, 4)
        qv.apply_matrix([2, 7], m)
        o = O.OracleQV(n, psi)
        o.apply_matrix([2, 7], m)
        ip = qv.inner_product()
        assert abs(ip - o.inner_product(psi)) < 1e-12
        qv.revert(True)
        np.testing.assert_allclose(qv.copy_to_vector(), psi, atol=0)


def test_expval_many_matches_single():
    P = pkg()
    rng = np.random.default_rng(9)
    n = 13
    psi = rand_state(rng, n)
    terms = []
    for _ in range(40):
        k = int(rng.integers(1, 5))
        q = [int(x) for x in rng.choice(n, k, replace=False)]
        terms.append((q, "".join(rng.choice(list("IXYZ"), k))))
    coeffs = rng.normal(size=len(terms))
    o = O.OracleQV(n, psi)
    with P.QubitVector(n) as qv:
        qv.initialize_from_vector(psi)
        vals, total = qv.expval_pauli_many(terms, coeffs)
    want = np.array([o.expval_pauli(q, lab) for q, lab in terms])
    np.testing.assert_allclose(vals, want, atol=1e-12)
    assert abs(total - float(coeffs @ want)) < 1e-11


def test_errors_on_device():
    P = pkg()
    with P.QubitVector(5) as qv:
        with pytest.raises(P.GBQVError) as e:
            qv.apply_mcx([0, 5])
        assert e.value.code == 2
        with pytest.raises(P.GBQVError):
            qv.apply_pauli([0, 1], "XQ")
        with pytest.raises(P.GBQVError):
            qv.apply_matrix([0, 1], np.eye(2))
        with pytest.raises(P.GBQVError):
            qv.initialize_from_vector(np.ones(7))
        import ctypes as C
        q = np.zeros(1, dtype=np.uint64)
        m = np.eye(4, dtype=np.complex128).reshape(-1)
        rc = qv._L.gbqv_dm_apply_superop_matrix(qv.handle, q.ctypes.data_as(C.POINTER(C.c_uint64)), 1,
                                                m.ctypes.data_as(C.c_void_p))
        assert rc == 5      # GBQV_ERR_KIND: a superoperator needs a density matrix


def test_large_n_properties():
    """n = 26: unitary circuits keep the norm; U then U^dagger is the identity."""
    P = pkg()
    rng = np.random.default_rng(4)
    n = 26
    with P.QubitVector(n) as qv:
        qv.initialize()
        for q in range(n):
            qv.apply_matrix([q], haar(rng, 2))
        mats = []
        for _ in range(10):
            q = [int(x) for x in rng.choice(n, 3, replace=False)]
            m = haar(rng, 8)
            mats.append((q, m))
            qv.apply_matrix(q, m)
        assert abs(qv.norm() - 1.0) < 1e-12
        qv.checkpoint()
        for q, m in mats[::-1]:
            qv.apply_matrix(q, m.conj().T)
        for q, m in mats:
            qv.apply_matrix(q, m)
        assert abs(qv.inner_product() - 1.0) < 1e-11
