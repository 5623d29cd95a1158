"""The standard noise channels (qiskit_aer/noise/errors/standard_errors.py)
as superoperators, and NoiseModel's error lookup (noise_model.py:669-806,
NoiseModel::sample_local_quantum_noise, noise_model.hpp:710-780).  No GPU:
the channels are checked by their action on random density matrices, by
trace preservation and complete positivity, and against the reference's own
constructions (the thermal-relaxation Choi matrix, the Pauli mixture of the
depolarizing channel)."""
import numpy as np
import pytest

from _pkg import pkg

X = np.array([[0, 1], [1, 0]], dtype=complex)
Z = np.diag([1.0, -1.0]).astype(complex)


def act(err, rho):
    d = rho.shape[0]
    return (err.superop @ rho.reshape(-1, order="F")).reshape(d, d, order="F")


def random_rho(rng, d):
    a = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    r = a @ a.conj().T
    return r / np.trace(r)


def choi_of(err):
    """Choi matrix sum_ij |i><j| (x) E(|i><j|) (rows (i, a), columns (j, b))."""
    d = 1 << err.num_qubits
    out = np.zeros((d * d, d * d), dtype=complex)
    for i in range(d):
        for j in range(d):
            e = np.zeros((d, d), dtype=complex)
            e[i, j] = 1
            out += np.kron(e, act(err, e))
    return out


def is_cptp(err):
    d = 1 << err.num_qubits
    c = choi_of(err)
    tp = all(abs(np.trace(act(err, np.outer(np.eye(d)[i], np.eye(d)[j]))) - (i == j)) < 1e-12
             for i in range(d) for j in range(d))
    return tp and np.min(np.linalg.eigvalsh((c + c.conj().T) / 2)) > -1e-12


@pytest.mark.parametrize("t1,t2,time,pop", [(50.0, 30.0, 2.0, 0.0), (50.0, 30.0, 2.0, 0.2), (40.0, 70.0, 3.0, 0.0),
                                            (40.0, 80.0, 5.0, 0.3), (np.inf, np.inf, 1.0, 0.0),
                                            (30.0, 60.0, 0.0, 0.1)])
def test_thermal_relaxation(t1, t2, time, pop):
    P = pkg()
    err = P.thermal_relaxation_error(t1, t2, time, pop)
    assert err.num_qubits == 1 and is_cptp(err)
    r = 0.0 if t1 == np.inf else 1 - np.exp(-time / t1)
    e2 = 1.0 if t2 == np.inf else np.exp(-time / t2)
    rho = random_rho(np.random.default_rng(1), 2)
    out = act(err, rho)
    p0, p1 = 1 - pop, pop
    np.testing.assert_allclose(out[0, 0], (1 - p1 * r) * rho[0, 0] + p0 * r * rho[1, 1], atol=1e-14)
    np.testing.assert_allclose(out[1, 1], p1 * r * rho[0, 0] + (1 - p0 * r) * rho[1, 1], atol=1e-14)
    np.testing.assert_allclose(out[0, 1], e2 * rho[0, 1], atol=1e-14)
    # the reference's Choi matrix of the T2 > T1 branch, standard_errors.py:320-330
    choi = np.array([[1 - p1 * r, 0, 0, e2], [0, p1 * r, 0, 0], [0, 0, p0 * r, 0], [e2, 0, 0, 1 - p0 * r]])
    np.testing.assert_allclose(choi_of(err), choi, atol=1e-14)


def test_thermal_relaxation_errors():
    P = pkg()
    for args, msg in [((0, 1, 1), "T_1"), ((1, 0, 1), "T_2"), ((1, 3, 1), "greater than 2"), ((1, 1, -1), "gate_time"),
                      ((1, 1, 1, 1.5), "excited")]:
        with pytest.raises(ValueError, match=msg):
            P.thermal_relaxation_error(*args)


def test_reset_error_action():
    P = pkg()
    rho = random_rho(np.random.default_rng(2), 2)
    err = P.reset_error(0.2, 0.1)
    want = 0.7 * rho + np.trace(rho) * np.diag([0.2, 0.1])
    np.testing.assert_allclose(act(err, rho), want, atol=1e-15)
    assert is_cptp(err)
    with pytest.raises(ValueError):
        P.reset_error(0.7, 0.5)


def test_pauli_error_labels_and_depolarizing():
    P = pkg()
    rho = random_rho(np.random.default_rng(3), 4)
    err = P.pauli_error([("XZ", 0.3), ("II", 0.7)])
    m = np.kron(X, Z)  # X on qubit 1, Z on qubit 0 (qiskit's label order)
    np.testing.assert_allclose(act(err, rho), 0.7 * rho + 0.3 * m @ rho @ m.conj().T, atol=1e-15)
    dep = P.depolarizing_error(0.12, 1)
    mix = P.pauli_error([("I", 1 - 0.12 * 3 / 4), ("X", 0.03), ("Y", 0.03), ("Z", 0.03)])
    np.testing.assert_allclose(dep.superop, mix.superop, atol=1e-15)
    with pytest.raises(ValueError, match="normalized"):
        P.pauli_error([("X", 0.5)])
    with pytest.raises(ValueError, match="same length"):
        P.pauli_error([("X", 0.5), ("XX", 0.5)])
    with pytest.raises(ValueError, match="Invalid Pauli"):
        P.pauli_error([("Q", 1.0)])


def test_unitary_and_kraus_errors():
    P = pkg()
    rng = np.random.default_rng(4)
    q, _ = np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))
    rho = random_rho(rng, 4)
    err = P.mixed_unitary_error([(q, 0.25), (np.eye(4), 0.75)])
    np.testing.assert_allclose(act(err, rho), 0.25 * q @ rho @ q.conj().T + 0.75 * rho, atol=1e-14)
    coh = P.coherent_unitary_error(q)
    np.testing.assert_allclose(act(coh, rho), q @ rho @ q.conj().T, atol=1e-14)
    with pytest.raises(ValueError, match="not unitary"):
        P.mixed_unitary_error([(np.diag([1.0, 2.0]), 1.0)])
    with pytest.raises(ValueError, match="different size"):
        P.mixed_unitary_error([(np.eye(2), 0.5), (np.eye(4), 0.5)])
    g = 0.3
    k = [np.array([[1, 0], [0, np.sqrt(1 - g)]]), np.array([[0, np.sqrt(g)], [0, 0]])]
    np.testing.assert_allclose(P.kraus_error(k).superop, P.amplitude_damping_error(g).superop, atol=1e-15)
    with pytest.raises(ValueError, match="CPTP"):
        P.kraus_error([np.eye(2) * 2])
    pd = P.phase_damping_error(0.4)
    r1 = random_rho(rng, 2)
    np.testing.assert_allclose(act(pd, r1), [[r1[0, 0], np.sqrt(0.6) * r1[0, 1]], [np.sqrt(0.6) * r1[1, 0], r1[1, 1]]],
                               atol=1e-15)


def test_noise_model_lookup_and_composition():
    P = pkg()
    nm = P.NoiseModel()
    assert nm.is_ideal()
    nm.add_all_qubit_quantum_error(P.depolarizing_error(0.0, 1), ["x"])    # ideal: not added
    assert nm.is_ideal()
    a, b = P.depolarizing_error(0.1, 1), P.amplitude_damping_error(0.2)
    nm.add_all_qubit_quantum_error(a, ["x", "sx"])
    nm.add_all_qubit_quantum_error(b, "x")                                   # composed after a
    np.testing.assert_allclose(nm.error_for("x", [3]).superop, b.superop @ a.superop, atol=1e-15)
    assert nm.error_for("sx", [0]) is a
    loc = P.thermal_relaxation_error(30.0, 20.0, 1.0)
    nm.add_quantum_error(loc, "x", [2])
    assert nm.error_for("x", [2]) is loc                                      # in place of the all-qubit error
    assert nm.error_for("x", [1]).superop is not loc.superop
    two = P.depolarizing_error(0.05, 2)
    nm.add_quantum_error(two, ["cx"], [0, 1])
    assert nm.error_for("cx", [0, 1]) is two and nm.error_for("cx", [1, 0]) is None
    assert nm.noise_instructions == ["cx", "sx", "x"] and nm.noise_qubits == [0, 1, 2]
    with pytest.raises(ValueError, match="does not match"):
        nm.add_quantum_error(two, "cx", [0])


def test_expand_is_tensor_swapped():
    P = pkg()
    a, b = P.amplitude_damping_error(0.3), P.phase_damping_error(0.2)
    np.testing.assert_allclose(a.expand(b).superop, b.tensor(a).superop, atol=0)


def roerror_reference(creg: str, memory_bits, probs, u, P):
    """ClassicalRegister::apply_roerror restated on the reference's string
    register (creg[size - 1 - bit] holds bit `bit`)."""
    creg = list(creg)
    mem_str = "".join(creg[len(creg) - 1 - b] for b in reversed(memory_bits))
    outcome = P.simulator.discrete_draw(probs[int(mem_str, 2)], u)
    noise = format(outcome, f"0{len(memory_bits)}b")
    for pos, b in enumerate(memory_bits):
        creg[len(creg) - 1 - b] = noise[len(noise) - 1 - pos]
    return "".join(creg)


def test_readout_error_checks_and_lookup():
    P = pkg()
    with pytest.raises(ValueError, match="is not 1"):
        P.ReadoutError([[0.9, 0.2], [0.1, 0.9]])
    with pytest.raises(ValueError, match="2\\*\\*"):
        P.ReadoutError([[0.5, 0.3, 0.2], [0.5, 0.3, 0.2], [0.5, 0.3, 0.2]])
    assert P.ReadoutError([[1, 0], [0, 1]]).ideal()
    nm = P.NoiseModel()
    nm.add_all_qubit_readout_error(P.ReadoutError([[1, 0], [0, 1]]))   # ideal: not added
    assert nm.is_ideal()
    d = P.ReadoutError([[0.9, 0.1], [0.2, 0.8]])
    loc = P.ReadoutError([[0.7, 0.3], [0.4, 0.6]])
    two = P.ReadoutError(np.eye(4)[[1, 0, 3, 2]])
    nm.add_all_qubit_readout_error(d)
    nm.add_readout_error(loc, [2])
    nm.add_readout_error(two, [0, 1])
    assert nm.has_readout_errors() and not nm.has_quantum_errors() and not nm.is_ideal()
    ops = nm.readout_ops([0, 1], [5, 6])                 # exactly the 2-qubit error's qubits
    assert len(ops) == 1 and ops[0][0] == [5, 6] and ops[0][1] is two.probabilities
    ops = nm.readout_ops([1, 2, 3], [0, 1, 2])           # per qubit: default, local, default
    assert [b for b, _ in ops] == [[0], [1], [2]]
    assert ops[1][1] is loc.probabilities and ops[0][1] is d.probabilities
    with pytest.raises(ValueError, match="single-qubit"):
        nm.add_all_qubit_readout_error(two)
    assert nm.noise_instructions == ["measure"]


def test_apply_readout_matches_string_register():
    P = pkg()
    rng = np.random.default_rng(7)
    probs2 = rng.random((4, 4))
    probs2 /= probs2.sum(axis=1, keepdims=True)
    for _ in range(200):
        mem = int(rng.integers(0, 1 << 6))
        bits = [int(x) for x in rng.choice(6, 2, replace=False)]
        u = float(rng.random())
        got = P.noise.apply_readout(mem, bits, probs2, u)
        want = roerror_reference(format(mem, "06b"), bits, probs2, u, P)
        assert format(got, "06b") == want


def test_sampled_readout_walks_samples_backwards():
    """measure_sampler: samples take the stream's first draws, then the
    readout draws go from the last sample to the first."""
    P = pkg()
    rng = np.random.default_rng(8)
    probs = np.array([[0.6, 0.4], [0.3, 0.7]])
    ro = [([0], probs), ([2], probs)]
    mem = rng.integers(0, 8, size=5).astype(np.uint64)
    u = rng.random(10)
    got = P.AerSimulator._readout_sampled(mem, ro, u)
    want, k = [], 0
    for i in reversed(range(5)):
        m = int(mem[i])
        for bits, p in ro:
            m = int(roerror_reference(format(m, "03b"), bits, p, u[k], P), 2)
            k += 1
        want.append(m)
    assert got == want


def test_basis_gates_reset_and_error_sizes():
    """NoiseModel.basis_gates / add_basis_gates / reset and the size check of
    errors on standard instructions (qiskit_aer/noise/noise_model.py:193-199,
    648-667, 1082-1107)."""
    P = pkg()
    nm = P.NoiseModel()
    assert nm.basis_gates == ["cx", "id", "rz", "sx"]
    nm.add_all_qubit_quantum_error(P.depolarizing_error(0.1, 1), ["u3", "measure"])
    nm.add_quantum_error(P.depolarizing_error(0.1, 2), "ecr", [0, 1])
    nm.add_quantum_error(P.depolarizing_error(0.1, 1), "my_label", [0])
    assert nm.basis_gates == ["cx", "ecr", "id", "rz", "sx", "u3"]
    assert nm.noise_instructions == ["ecr", "measure", "my_label", "u3"]
    with pytest.raises(ValueError, match='1 qubit QuantumError cannot be applied to 2 qubit instruction "cx"'):
        nm.add_all_qubit_quantum_error(P.depolarizing_error(0.1, 1), "cx")
    with pytest.raises(ValueError, match='2 qubit QuantumError cannot be applied to 1 qubit instruction "x"'):
        nm.add_quantum_error(P.depolarizing_error(0.1, 2), "x", [0, 1])
    nm.reset()
    assert nm.is_ideal() and nm.basis_gates == ["cx", "id", "rz", "sx"]
    assert P.NoiseModel(basis_gates=["u", "cz"]).basis_gates == ["cz", "u"]


def test_readout_error_algebra():
    """ReadoutError compose / dot / power / tensor / expand / to_dict as the
    reference's (qiskit_aer/noise/errors/readout_error.py:156-330): compose
    multiplies other * self, dot self * other, tensor self (x) other."""
    P = pkg()
    a = P.ReadoutError([[0.9, 0.1], [0.3, 0.7]])
    b = P.ReadoutError([[0.8, 0.2], [0.4, 0.6]])
    np.testing.assert_allclose(a.compose(b).probabilities, b.probabilities @ a.probabilities)
    np.testing.assert_allclose(a.compose(b, front=True).probabilities, a.probabilities @ b.probabilities)
    np.testing.assert_allclose(a.dot(b).probabilities, a.probabilities @ b.probabilities)
    np.testing.assert_allclose((a @ b).probabilities, a.compose(b).probabilities)
    np.testing.assert_allclose(a.power(3).probabilities, np.linalg.matrix_power(a.probabilities, 3))
    ab = a.tensor(b)
    assert ab.number_of_qubits == 2
    np.testing.assert_allclose(ab.probabilities, np.kron(a.probabilities, b.probabilities))
    np.testing.assert_allclose(a.expand(b).probabilities, np.kron(b.probabilities, a.probabilities))
    assert a.to_dict() == {"type": "roerror", "operations": ["measure"], "probabilities": [[0.9, 0.1], [0.3, 0.7]]}
    assert a.copy() == a and a != b
    with pytest.raises(ValueError, match="same number of qubits"):
        a.compose(ab)
    with pytest.raises(ValueError, match="positive integer"):
        a.power(0)
    # a tensor-product error on a 2-qubit measurement acts like the two
    # single-qubit errors: b on the first measured bit, a on the second
    nm2, nm1 = P.NoiseModel(), P.NoiseModel()
    nm2.add_readout_error(ab, [0, 1])
    nm1.add_readout_error(b, [0])
    nm1.add_readout_error(a, [1])
    (bits, probs), = nm2.readout_ops([0, 1], [0, 1])
    ops1 = nm1.readout_ops([0, 1], [0, 1])
    for actual in range(4):
        for read in range(4):
            p1 = np.prod([ops1[j][1][(actual >> j) & 1][(read >> j) & 1] for j in range(2)])
            assert abs(probs[actual][read] - p1) < 1e-15
