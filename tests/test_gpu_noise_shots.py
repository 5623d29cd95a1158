"""Sampled Kraus noise on the statevector method: the reference's Kraus noise
method (circuit_executor.hpp:648-657) turns every error into a Kraus
channel, and each shot applies one operator per channel drawn with its own
RNG stream (State::apply_kraus, statevector_state.hpp:1112-1156).  The
stacked shots equal the oracle's one-shot loop shot for shot, the one-state
path equals the stacked one, and the counts follow the density matrix."""
import ctypes as C

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def haar(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def oracle_apply_kraus(o, qubits, mats, r):
    """State::apply_kraus on the oracle, in the reference's order: the
    probability of each operator but the last from QubitVector::norm(qubits,
    mat), the first whose running sum exceeds r applied with its matrix
    scaled by 1/sqrt(p), else the last scaled by 1/sqrt(1 - sum)."""
    accum = 0.0
    for K in mats[:-1]:
        p = o.norm_matrix(qubits, K)
        accum += p
        if accum > r:
            o.apply_matrix(qubits, K * (1 / np.sqrt(p)))
            return
    o.apply_matrix(qubits, mats[-1] * (1 / np.sqrt(1.0 - accum)))


def noisy_ops(sim, ins):
    """(before, after): the Kraus channels the noise model puts around one
    instruction (before a measure, after a gate or reset)."""
    errs = sim._error_kraus(ins)
    return (errs, []) if ins.kind == "measure" else ([], errs)


def oracle_memory(P, sim, qc, shots, seed, sums=None):
    """The per-shot loop on the oracle: shot i from |0...0> with the stream
    seed + i, one uniform per Kraus channel and per measure / reset; saves
    add each shot's value to `sums` (expectation values of Pauli sums,
    probabilities)."""
    out = []
    for shot in range(shots):
        o = O.OracleQV(qc.num_qubits)
        u = P.uniforms(seed + shot, 512)
        used, mem = 0, 0
        for ins in qc.data:
            if ins.condition is not None:
                cb, val = ins.condition
                if any(((mem >> c) & 1) != ((val >> i) & 1) for i, c in enumerate(cb)):
                    continue
            if ins.kind == "save":
                if ins.name == "probabilities":
                    label, val = ins.data, o.probabilities(ins.qubits)
                else:
                    label, terms = ins.data
                    val = sum(c * o.expval_pauli(q, lab) for c, lab, q in terms)
                    if ins.name == "expval_var":   # a single Pauli: <P^2> = 1
                        val = np.array([val, 1.0 - val * val])
                sums[label] = sums.get(label, 0) + val
                continue
            before, after = noisy_ops(sim, ins)
            for op in before:
                oracle_apply_kraus(o, op.qubits, list(op.mats), u[used])
                used += 1
            if ins.kind == "unitary":
                o.apply_matrix(ins.qubits, ins.data)
            elif ins.name == "u3":
                o.apply_matrix(ins.qubits, O.u3(*ins.params))
            elif ins.name == "cx":
                o.apply_mcx(ins.qubits)
            elif ins.kind == "kraus":
                oracle_apply_kraus(o, ins.qubits, ins.data, u[used])
                used += 1
            elif ins.kind in ("measure", "reset"):
                probs = o.probabilities(ins.qubits)
                k = P.simulator.discrete_draw(probs, u[used])
                used += 1
                diag = np.zeros(1 << len(ins.qubits), dtype=complex)
                diag[k] = 1 / np.sqrt(probs[k])
                o.apply_diagonal_matrix(ins.qubits, diag)
                if ins.kind == "reset" and k:
                    perm = np.eye(1 << len(ins.qubits), dtype=complex)
                    perm[[0, k]] = perm[[k, 0]]
                    o.apply_matrix(ins.qubits, perm)
                if ins.kind == "measure":
                    for i, c in enumerate(ins.clbits):
                        mem = (mem & ~(1 << c)) | (((k >> i) & 1) << c)
                    for bits, rp in sim._readout_ops([ins]):   # readout errors draw after the outcome
                        mem = P.noise.apply_readout(mem, bits, rp, u[used])
                        used += 1
            for op in after:
                oracle_apply_kraus(o, op.qubits, list(op.mats), u[used])
                used += 1
        out.append(hex(mem))
    return out


def noise_model(P, measure=True):
    """Amplitude damping (Kraus, state-dependent probabilities) composed
    with depolarizing noise on 1-qubit gates, their tensor product on CX,
    pure depolarizing on resets (a mixture of unitaries) and damping before
    measurements."""
    e1 = P.depolarizing_error(0.04, 1).compose(P.amplitude_damping_error(0.12))
    nm = P.NoiseModel()
    nm.add_all_qubit_quantum_error(e1, ["u3"])
    nm.add_all_qubit_quantum_error(e1.tensor(P.amplitude_damping_error(0.05)), ["cx"])
    nm.add_all_qubit_quantum_error(P.depolarizing_error(0.1, 1), ["reset"])
    if measure:
        nm.add_all_qubit_quantum_error(P.amplitude_damping_error(0.2), ["measure"])
    return nm


def feedback_circuit(P, n, rng):
    qc = P.QuantumCircuit(n, 2 * n)
    for r in range(3):
        for q in range(n):
            qc.u3(*rng.uniform(0, 2 * np.pi, 3), q)
        for q in range(r % 2, n - 1, 2):
            qc.cx(q, q + 1)
        qc.measure([r % n], [2 * r])
        qc.u3(*rng.uniform(0, 2 * np.pi, 3), (r + 1) % n).c_if([2 * r], 1)
        qc.reset([(r + 2) % n])
    qc.measure(list(range(n)), list(range(n, 2 * n)))
    return qc


def test_rdm_and_kraus_segments_match_numpy():
    """The two stack entry points against numpy: reduced density matrices of
    1..3 qubits in a scrambled order, and each state's chosen operator
    times its scale (255 leaves a state untouched)."""
    P = pkg()
    A = P._capi
    L = P.lib()
    rng = np.random.default_rng(21)
    n, b, cnt = 7, 3, 7
    for precision, tol in (("double", 1e-14), ("single", 2e-6)):
        for qubits in ([3], [5, 0], [2, 6, 4]):
            k, D = len(qubits), 1 << len(qubits)
            psi = rng.normal(size=(1 << b, 1 << n)) + 1j * rng.normal(size=(1 << b, 1 << n))
            psi /= np.linalg.norm(psi, axis=1, keepdims=True)
            q = (C.c_uint64 * k)(*qubits)
            idx = np.arange(1 << n)
            val = np.zeros(idx.size, dtype=np.int64)
            for j, x in enumerate(qubits):
                val |= ((idx >> x) & 1) << j
            with P.QubitVector(n + b, precision) as st:
                st.initialize_from_vector(psi.reshape(-1))
                rho = np.empty((cnt, D, D), dtype=np.complex128)
                A.check(L.gbqv_rdm_segments(st.handle, n, cnt, q, k, rho.ctypes.data_as(A.vp)), st.handle)
                for s in range(cnt):
                    amp = np.zeros((D, (1 << n) // D), dtype=complex)
                    for a in range(D):
                        amp[a] = psi[s][val == a]
                    np.testing.assert_allclose(rho[s], amp @ amp.conj().T, rtol=0, atol=tol)
                mats = np.stack([haar(rng, D) * 0.5 for _ in range(3)])
                colmajor = np.ascontiguousarray(mats.transpose(0, 2, 1)).reshape(-1)
                branch = np.array([2, 0, 255, 1, 1, 0, 2, 255], dtype=np.uint8)
                scale = rng.uniform(0.5, 2.0, 1 << b)
                A.check(L.gbqv_kraus_segments(st.handle, n, cnt, q, k, colmajor.ctypes.data_as(A.vp), 3,
                                              branch.ctypes.data_as(A.vp), scale.ctypes.data_as(A.dp)), st.handle)
                got = st.copy_to_vector().reshape(1 << b, 1 << n)
            for s in range(1 << b):
                if s >= cnt or branch[s] == 255:
                    np.testing.assert_allclose(got[s], psi[s], rtol=0, atol=tol)
                    continue
                o = O.OracleQV(n, psi[s])
                o.apply_matrix(qubits, mats[branch[s]] * scale[s])
                np.testing.assert_allclose(got[s], o.data, rtol=0, atol=4 * tol)


def test_kraus_segments_reject_bad_arguments():
    P = pkg()
    A = P._capi
    L = P.lib()
    with P.QubitVector(6) as st:
        q = (C.c_uint64 * 1)(0)
        mats = np.eye(2, dtype=complex).reshape(-1)
        branch = np.array([1, 0], dtype=np.uint8)   # operator 1 of 1
        scale = np.ones(2)
        rc = L.gbqv_kraus_segments(st.handle, 5, 2, q, 1, mats.ctypes.data_as(A.vp), 1,
                                   branch.ctypes.data_as(A.vp), scale.ctypes.data_as(A.dp))
        assert rc != 0
        q4 = (C.c_uint64 * 4)(0, 1, 2, 3)
        rho = np.empty((2, 16, 16), dtype=complex)
        assert L.gbqv_rdm_segments(st.handle, 5, 2, q4, 4, rho.ctypes.data_as(A.vp)) != 0


@pytest.mark.parametrize("n", [3, 5])
def test_noisy_statevector_shots_match_oracle(n):
    """Every shot's memory equals the oracle loop's: Kraus channels with
    state-dependent probabilities (amplitude damping), mixtures of unitaries
    (depolarizing, no probability pass), a conditioned gate whose noise is
    conditioned with it, resets and mid-circuit measurements."""
    P = pkg()
    qc = feedback_circuit(P, n, np.random.default_rng(30 + n))
    sim = P.AerSimulator(noise_model=noise_model(P))
    sim.SHOT_GROUP_BITS = 4                       # 40 shots over three groups, the last partial
    res = sim.run(qc, shots=40, seed_simulator=55, memory=True)
    assert res.metadata()["noise"] == "kraus"
    assert res.get_memory() == oracle_memory(P, sim, qc, 40, 55)


def test_kraus_instruction_and_one_state_path():
    """A circuit's own Kraus instruction (2-qubit, four operators), and the
    one-state path (a conditioned 5-qubit gate keeps a circuit off the
    stack) equal to the stacked one in both precisions."""
    P = pkg()
    rng = np.random.default_rng(8)
    g1, g2 = 0.3, 0.15
    ad = lambda g: [np.array([[1, 0], [0, np.sqrt(1 - g)]]), np.array([[0, np.sqrt(g)], [0, 0]])]
    two = [np.kron(a, b) for a in ad(g1) for b in ad(g2)]
    qc = P.QuantumCircuit(5, 6)
    for q in range(5):
        qc.unitary(haar(rng, 2), [q])
    qc.kraus(two, [1, 3])
    qc.unitary(haar(rng, 4), [0, 3])
    qc.measure([3], [0])
    qc.kraus(ad(0.4), [2]).c_if(0, 1)
    qc.unitary(haar(rng, 4), [2, 4])
    qc.measure(list(range(5)), list(range(1, 6)))
    sim = P.AerSimulator()
    got = sim.run(qc, shots=48, seed_simulator=9, memory=True).get_memory()
    assert got == oracle_memory(P, sim, qc, 48, 9)
    for precision in ("double", "single"):
        stacked = P.AerSimulator(precision=precision).run(qc, shots=30, seed_simulator=3, memory=True)
        serial_sim = P.AerSimulator(precision=precision)
        serial_sim._conditioned_matrices = lambda items: None
        serial = serial_sim.run(qc, shots=30, seed_simulator=3, memory=True)
        assert stacked.metadata()["batched_shots_optimization"] is True
        assert stacked.get_memory() == serial.get_memory()


def test_noisy_statevector_counts_follow_the_density_matrix():
    """4096 trajectories of a noisy 4-qubit circuit measured at the end: every
    outcome's count lies within five standard deviations of the density
    matrix method's probability of it (same noise, superoperators)."""
    P = pkg()
    rng = np.random.default_rng(4)
    qc = P.QuantumCircuit(4, 4)
    for r in range(3):
        for q in range(4):
            qc.u3(*rng.uniform(0, 2 * np.pi, 3), q)
        for q in range(r % 2, 3, 2):
            qc.cx(q, q + 1)
    qd = P.QuantumCircuit(4, 4)
    qd.data = list(qc.data)
    qd.save_probabilities(list(range(4)), label="p")
    qc.measure(range(4), range(4))
    nm = noise_model(P, measure=False)
    shots = 4096
    counts = P.AerSimulator(noise_model=nm).run(qc, shots=shots, seed_simulator=17).get_counts()
    assert sum(counts.values()) == shots
    probs = np.asarray(P.AerSimulator(method="density_matrix", noise_model=nm).run(qd, shots=1).data()["p"])
    assert probs.shape == (16,)
    for v in range(16):
        p = probs[v]
        c = counts.get(format(v, "04b"), 0)
        assert abs(c - shots * p) <= 5 * np.sqrt(shots * p * (1 - p)) + 2, (v, c, shots * p)


def test_saves_average_over_noisy_shots():
    """save_expval, save_expval_var and save_probabilities in a circuit run
    shot by shot: the average over the shots (the reference's default
    `average` subtype), mid-circuit and at the end, against the oracle loop,
    stacked and one state at a time."""
    P = pkg()
    n = 4
    qc = feedback_circuit(P, n, np.random.default_rng(61))
    final = qc.data.pop()                        # the final measurement goes last again below
    qc.save_expectation_value([(0.7, "ZZ", [0, 2]), (-0.4, "X", [1])], label="mid")
    qc.u3(0.3, 0.2, 0.1, 3)
    qc.save_expectation_value_variance([(1.0, "Y", [3])], label="var")
    qc.save_probabilities([2, 0], label="p")
    qc.data.append(final)
    nm = noise_model(P)
    want = {}
    sim = P.AerSimulator(noise_model=nm)
    oracle_memory(P, sim, qc, 24, 5, want)
    for serial in (False, True):
        s2 = P.AerSimulator(noise_model=nm)
        s2.SHOT_GROUP_BITS = 3
        if serial:
            s2._conditioned_matrices = lambda items: None
        got = s2.run(qc, shots=24, seed_simulator=5).data()
        assert isinstance(got["mid"], float)
        assert abs(got["mid"] - want["mid"] / 24) < 1e-12
        np.testing.assert_allclose(got["var"], want["var"] / 24, rtol=0, atol=1e-12)
        np.testing.assert_allclose(got["p"], want["p"] / 24, rtol=0, atol=1e-12)


def test_kraus_noise_with_readout_errors():
    """Kraus channels and readout errors on the same shots: each shot's
    stream serves the channels, the outcome and then the readout errors in
    circuit order, stacked as in the oracle loop."""
    P = pkg()
    n = 4
    qc = feedback_circuit(P, n, np.random.default_rng(90))
    nm = noise_model(P)
    nm.add_all_qubit_readout_error(P.ReadoutError([[0.9, 0.1], [0.2, 0.8]]))
    nm.add_readout_error(P.ReadoutError([[0.7, 0.3], [0.05, 0.95]]), [1])
    sim = P.AerSimulator(noise_model=nm)
    sim.SHOT_GROUP_BITS = 4
    got = sim.run(qc, shots=40, seed_simulator=71, memory=True).get_memory()
    assert got == oracle_memory(P, sim, qc, 40, 71)
