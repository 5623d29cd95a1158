"""Host side of sampled Kraus noise on the statevector method, no GPU: the
canonical Kraus operators of an error (Utils::superop2kraus,
src/framework/noise_utils.hpp:33-87), the per-shot choice of
State::apply_kraus (statevector_state.hpp:1112-1156) against its scalar
loop, and where a noise model's errors go in a circuit run shot by shot."""
import numpy as np
import pytest

from _pkg import pkg


def apply_kraus_choice(probs, r):
    """The reference's loop: running sum over all operators but the last,
    the first whose sum exceeds r, else the last with 1/sqrt(1 - sum)."""
    accum = 0.0
    for j, p in enumerate(probs[:-1]):
        accum += p
        if accum > r:
            return j, 1 / np.sqrt(p)
    return len(probs) - 1, 1 / np.sqrt(1.0 - accum)


def test_canonical_kraus_reproduce_the_channel():
    P = pkg()
    N = P.noise
    errs = [P.amplitude_damping_error(0.1), P.depolarizing_error(0.05, 1), P.depolarizing_error(0.05, 2),
            P.thermal_relaxation_error(50, 70, 10), P.phase_damping_error(0.3),
            P.depolarizing_error(0.05, 1).compose(P.amplitude_damping_error(0.1)),
            P.amplitude_damping_error(0.1).tensor(P.amplitude_damping_error(0.2))]
    for e in errs:
        ks = e.kraus()
        d = 1 << e.num_qubits
        assert 1 <= len(ks) <= d * d
        np.testing.assert_allclose(N.kraus_superop(ks), e.superop, rtol=0, atol=1e-14)
        np.testing.assert_allclose(sum(k.conj().T @ k for k in ks), np.eye(d), rtol=0, atol=1e-14)
        # canonical: Hilbert-Schmidt orthogonal, largest first
        w = [np.vdot(k, k).real for k in ks]
        assert all(a >= b - 1e-15 for a, b in zip(w, w[1:]))
        for i in range(len(ks)):
            for j in range(i + 1, len(ks)):
                assert abs(np.vdot(ks[i], ks[j])) < 1e-13


def test_amplitude_damping_kraus_known_answer():
    """Non-degenerate Choi spectrum: the operators are the textbook pair up
    to a phase, in the reference's order (eigenvalue 2 - g, then g)."""
    P = pkg()
    g = 0.3
    k0, k1 = P.amplitude_damping_error(g).kraus()
    ph0 = k0[0, 0] / abs(k0[0, 0])
    ph1 = k1[0, 1] / abs(k1[0, 1])
    np.testing.assert_allclose(k0 / ph0, np.diag([1.0, np.sqrt(1 - g)]), rtol=0, atol=1e-15)
    np.testing.assert_allclose(k1 / ph1, [[0, np.sqrt(g)], [0, 0]], rtol=0, atol=1e-15)


def test_ideal_and_tiny_eigenvalues_dropped():
    P = pkg()
    N = P.noise
    ks = N.superop_kraus(np.eye(4), 1)
    assert len(ks) == 1
    np.testing.assert_allclose(abs(ks[0]), np.eye(2), atol=1e-15)
    # a mixture with weight below the threshold keeps one operator
    e = N.kraus_error([np.sqrt(1 - 1e-12) * np.eye(2), np.sqrt(1e-12) * np.array([[0, 1], [1, 0]])])
    assert len(e.kraus()) == 1


def test_kraus_draws_follow_the_scalar_loop():
    P = pkg()
    S = P.simulator
    rng = np.random.default_rng(2)
    for m in (1, 2, 4, 7):
        p = rng.uniform(0, 1, size=(500, m))
        p /= p.sum(axis=1, keepdims=True)
        u = rng.uniform(0, 1, 500)
        # uniforms exactly on a running sum, and above every sum but the last
        u[:50] = np.add.accumulate(p[:50, :max(1, m - 1)], axis=1)[:, 0]
        u[50:60] = np.nextafter(1.0, 0.0)
        branch, scale = S.kraus_draws(p, u)
        for s in range(500):
            j, sc = apply_kraus_choice(p[s], u[s])
            assert branch[s] == j
            assert scale[s] == sc


def test_mixture_of_unitaries_needs_no_probability_pass():
    P = pkg()
    S = P.simulator
    dep = S.KrausOp([0], P.depolarizing_error(0.1, 1).kraus())
    assert dep.fixed is not None
    np.testing.assert_allclose(dep.fixed.sum(), 1.0, atol=1e-14)
    dep2 = S.KrausOp([0, 1], P.depolarizing_error(0.1, 2).kraus())
    assert dep2.fixed is not None
    ad = S.KrausOp([3], P.amplitude_damping_error(0.2).kraus())
    assert ad.fixed is None
    # column-major operators one after another
    np.testing.assert_array_equal(ad.colmajor[:4], ad.mats[0].reshape(-1, order="F"))
    with pytest.raises(ValueError):
        S.KrausOp([0, 1], [np.eye(2)])


def test_noise_placement_for_shots():
    """Errors after gates and resets, before measures, per qubit for a
    multi-qubit measure; a circuit run shot by shot when an error applies,
    sampled otherwise."""
    P = pkg()
    nm = P.NoiseModel()
    nm.add_all_qubit_quantum_error(P.amplitude_damping_error(0.1), ["u3"])
    nm.add_all_qubit_quantum_error(P.depolarizing_error(0.1, 1), ["measure", "reset"])
    nm.add_quantum_error(P.depolarizing_error(0.2, 2), ["cx"], [0, 1])
    sim = P.AerSimulator(noise_model=nm)
    qc = P.QuantumCircuit(3, 3)
    qc.u3(0.1, 0.2, 0.3, 0)
    qc.cx(0, 1)
    qc.cx(1, 2)
    qc.reset([2])
    qc.measure([0, 1], [0, 1])
    ops = [sim._error_kraus(ins) for ins in qc.data]
    assert [len(o) for o in ops] == [1, 1, 0, 1, 2]
    assert ops[0][0].qubits == [0] and ops[0][0].fixed is None
    assert ops[1][0].qubits == [0, 1] and ops[1][0].fixed is not None
    assert [o.qubits for o in ops[4]] == [[0], [1]]
    assert sim._sampled_noise(qc)
    quiet = P.QuantumCircuit(3, 3)
    quiet.x(2)
    quiet.measure([2], [2])
    nm2 = P.NoiseModel()
    nm2.add_all_qubit_quantum_error(P.amplitude_damping_error(0.1), ["u3"])
    sim2 = P.AerSimulator(noise_model=nm2)
    assert not sim2._sampled_noise(quiet)
    assert sim2._with_noise(list(quiet.data)) == list(quiet.data)
    assert not P.AerSimulator(method="density_matrix", noise_model=nm)._sampled_noise(qc)
