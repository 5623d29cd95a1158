"""Circuits that cannot be measure-sampled, run shot by shot
(CircuitExecutor::run_circuit_shots): mid-circuit measurements, resets and
classically conditioned ops.  Counts equal, bit for bit, the same per-shot
algorithm run on the oracle (the reference's QubitVector arithmetic) with the
same per-shot seeds seed + i; deterministic circuits (teleportation with
conditioned corrections, reset) give their one outcome."""
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


def oracle_counts(P, qc, shots, seed):
    """The executor's per-shot loop on the oracle."""
    ndraw = sum(1 for i in qc.data if i.kind in ("measure", "reset"))
    counts = {}
    for shot in range(shots):
        o = O.OracleQV(qc.num_qubits)
        u = P.uniforms(seed + shot, ndraw) if ndraw else []
        used, mem = 0, 0
        for ins in qc.data:
            if ins.condition is not None:
                cb, val = ins.condition
                if any(((mem >> c) & 1) != ((val >> i) & 1) for i, c in enumerate(cb)):
                    continue
            if ins.kind == "unitary":
                o.apply_matrix(ins.qubits, ins.data)
            elif ins.kind == "diagonal":
                o.apply_diagonal_matrix(ins.qubits, ins.data)
            elif ins.name == "x":
                o.apply_mcx(ins.qubits)
            elif ins.kind in ("measure", "reset"):
                probs = o.probabilities(ins.qubits)
                k = P.simulator.discrete_draw(probs, u[used])
                used += 1
                dim = 1 << len(ins.qubits)
                final = k if ins.kind == "measure" else 0
                if len(ins.qubits) > 10:
                    # wider than the oracle's matrices: the same projection,
                    # scaling and move on its amplitudes
                    idx = np.arange(o.data.size)
                    val = np.zeros(idx.size, dtype=np.int64)
                    for j, q in enumerate(ins.qubits):
                        val |= ((idx >> q) & 1) << j
                    keep = o.data[val == k] * (1 / np.sqrt(probs[k]))
                    dst = idx[val == k]
                    for j, q in enumerate(ins.qubits):
                        dst = dst ^ ((((k ^ final) >> j) & 1) << q)
                    o.data[:] = 0
                    o.data[dst] = keep
                else:
                    diag = np.zeros(dim, dtype=complex)
                    diag[k] = 1 / np.sqrt(probs[k])
                    o.apply_diagonal_matrix(ins.qubits, diag)
                if final != k and len(ins.qubits) <= 10:
                    if len(ins.qubits) == 1:
                        o.apply_mcx(ins.qubits)
                    else:
                        perm = np.eye(dim, dtype=complex)
                        perm[[final, k]] = perm[[k, final]]
                        o.apply_matrix(ins.qubits, perm)
                if ins.kind == "measure":
                    for i, c in enumerate(ins.clbits):
                        mem = (mem & ~(1 << c)) | (((k >> i) & 1) << c)
        key = format(mem, f"0{qc.num_clbits}b")
        counts[key] = counts.get(key, 0) + 1
    return counts


@pytest.mark.parametrize("n", [3, 6, 12])
@pytest.mark.parametrize("precision", ["double", "single"])
def test_mid_circuit_measure_reset_conditionals_match_oracle(n, precision):
    P = pkg()
    rng = np.random.default_rng(40 + n)
    qc = P.QuantumCircuit(n, 4)
    for layer in range(3):
        for q in range(0, n - 1, 2):
            qc.unitary(haar(rng, 4), [q, q + 1])
        qc.measure(layer % n, layer)
        qc.unitary(haar(rng, 2), [(layer + 1) % n]).c_if(layer, 1)
        qc.reset([(layer + 2) % n])
    qc.reset([0, 1])
    qc.unitary(haar(rng, 4), [0, 1])
    qc.measure([0, 1], [2, 3])
    shots, seed = 64, 1234
    got = P.AerSimulator(precision=precision).run(qc, shots=shots, seed_simulator=seed).get_counts()
    assert sum(got.values()) == shots
    if precision == "double":
        assert got == oracle_counts(P, qc, shots, seed)


def test_teleportation_with_conditioned_corrections():
    P = pkg()
    rng = np.random.default_rng(3)
    u = haar(rng, 2)
    qc = P.QuantumCircuit(3, 3)
    qc.unitary(u, [0])
    qc.h(1).cx(1, 2)
    qc.cx(0, 1).h(0)
    qc.measure(0, 0).measure(1, 1)
    qc.x(2).c_if(1, 1)
    qc.z(2).c_if(0, 1)
    qc.unitary(u.conj().T, [2])
    qc.measure(2, 2)
    counts = P.AerSimulator().run(qc, shots=200, seed_simulator=11).get_counts()
    assert sum(counts.values()) == 200
    assert all(k[0] == "0" for k in counts)          # clbit 2 (leftmost) always 0
    assert len(counts) == 4                           # the Bell outcomes all occur


def test_reset_returns_to_zero():
    P = pkg()
    qc = P.QuantumCircuit(2, 2).h(0).cx(0, 1).reset([0, 1]).measure([0, 1], [0, 1])
    counts = P.AerSimulator().run(qc, shots=50, seed_simulator=5).get_counts()
    assert counts == {"00": 50}
    qc = P.QuantumCircuit(1, 1).h(0).reset(0).x(0).measure(0, 0)
    assert P.AerSimulator().run(qc, shots=20, seed_simulator=5).get_counts() == {"1": 20}


def test_sampleable_circuit_still_sampled():
    """Final measurements only: the one-sample path, same counts as before."""
    P = pkg()
    qc = P.QuantumCircuit(3, 3).h(0).cx(0, 1).cx(1, 2).measure([0, 1, 2], [0, 1, 2])
    res = P.AerSimulator().run(qc, shots=1000, seed_simulator=9)
    assert set(res.get_counts()) == {"000", "111"}
    assert "shot_branching" not in res.metadata()


def _mixed_circuit(P, n, rng):
    qc = P.QuantumCircuit(n, 6)
    for q in range(n):
        qc.unitary(haar(rng, 2), [q])
    qc.unitary(haar(rng, 4), [0, n - 1])
    qc.measure([0, 1, 2], [0, 1, 2])                          # a 3-qubit register
    qc.unitary(haar(rng, 4), [1, 2]).c_if([0, 1], 2)         # conditioned 2-qubit matrix
    qc.diagonal(np.exp(1j * rng.uniform(-3, 3, 4)), [0, 2]).c_if(2, 1)
    qc.x(n - 1).c_if(0, 1)
    qc.reset([1, n - 1])                                      # a 2-qubit reset
    qc.unitary(haar(rng, 4), [0, 1])
    qc.measure(0, 3).c_if(1, 0)                               # a conditioned measurement
    qc.unitary(haar(rng, 2), [2])
    qc.measure([2, 1], [4, 5])
    return qc


def _wide_registers(P, n, rng):
    """Registers measured and reset in one op wider than the register-sum
    kernel (k > 5), in a scrambled qubit order."""
    qc = P.QuantumCircuit(n, 2 * n)
    for layer in range(2):
        for q in range(n):
            qc.unitary(haar(rng, 2), [q])
        for q in range(layer, n - 1, 2):
            qc.unitary(haar(rng, 4), [q, q + 1])
    order = [int(x) for x in rng.permutation(n)[: n - 1]]
    qc.measure(order, list(range(n - 1)))
    qc.x(order[0]).c_if(0, 1)
    qc.reset(order[1:7])
    for q in range(n):
        qc.unitary(haar(rng, 2), [q])
    qc.unitary(haar(rng, 4), [0, n - 1]).c_if([1, 2], 3)
    qc.measure(list(range(n)), list(range(n, 2 * n)))
    return qc


@pytest.mark.parametrize("make,n", [(_mixed_circuit, 5), (_wide_registers, 8)])
@pytest.mark.parametrize("precision", ["double", "single"])
def test_stacked_shots_equal_one_shot_at_a_time(make, n, precision):
    """The stacked path (groups of 8 shots here, so that 50 shots span seven
    groups, the last one partial) gives every shot the memory the one-state
    loop gives it."""
    P = pkg()
    qc = make(P, n, np.random.default_rng(77))
    stacked = P.AerSimulator(precision=precision)
    stacked.SHOT_GROUP_BITS = 3
    res = stacked.run(qc, shots=50, seed_simulator=321, memory=True)
    assert res.metadata()["batched_shots_optimization"] is True
    serial = P.AerSimulator(precision=precision)
    serial._conditioned_matrices = lambda items: None
    ref = serial.run(qc, shots=50, seed_simulator=321, memory=True)
    assert "batched_shots_optimization" not in ref.metadata()
    assert res.get_memory() == ref.get_memory()
    assert res.get_counts() == ref.get_counts()
    if precision == "double":
        assert res.get_counts() == oracle_counts(P, qc, 50, 321)


def test_segment_probabilities_and_collapse_on_the_stack():
    P = pkg()
    A = P._capi
    rng = np.random.default_rng(5)
    n, b = 6, 3
    psi = rng.normal(size=(1 << b, 1 << n)) + 1j * rng.normal(size=(1 << b, 1 << n))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    qubits = [4, 1]
    with P.QubitVector(n + b) as st:
        st.initialize_from_vector(psi.reshape(-1))
        q = (C.c_uint64 * 2)(*qubits)
        probs = np.empty((6, 4))
        A.check(P.lib().gbqv_probabilities_segments(st.handle, n, 6, q, 2, probs.ctypes.data_as(A.dp)), st.handle)
        for s in range(6):
            o = O.OracleQV(n)
            o.data[:] = psi[s]
            np.testing.assert_allclose(probs[s], o.probabilities(qubits), rtol=0, atol=1e-14)
        meas = np.array([1, 3, 0xFFFFFFFF, 2, 0, 3, 1, 1], dtype=np.uint32)
        final = np.array([1, 0, 0, 2, 0, 1, 0, 0], dtype=np.uint32)
        scale = np.where(meas[:6] != 0xFFFFFFFF, 1 / np.sqrt(probs[np.arange(6), meas[:6] % 4]), 0.0)
        A.check(P.lib().gbqv_collapse_segments(st.handle, n, 6, q, 2, meas.ctypes.data_as(A.vp),
                                               final.ctypes.data_as(A.vp), scale.ctypes.data_as(A.dp)), st.handle)
        got = st.copy_to_vector().reshape(1 << b, 1 << n)
    idx = np.arange(1 << n)
    val = ((idx >> 4) & 1) | (((idx >> 1) & 1) << 1)
    for s in range(1 << b):
        if s >= 6 or meas[s] == 0xFFFFFFFF:
            np.testing.assert_array_equal(got[s], psi[s])     # skipped and padding states untouched
            continue
        want = np.zeros(1 << n, dtype=complex)
        src = idx[val == meas[s]]
        dst = src ^ ((((meas[s] ^ final[s]) >> 0) & 1) << 4) ^ ((((meas[s] ^ final[s]) >> 1) & 1) << 1)
        want[dst] = psi[s][src] * scale[s]
        np.testing.assert_allclose(got[s], want, rtol=0, atol=1e-15)
        assert abs(np.linalg.norm(got[s]) - 1) < 1e-12


def test_device_draws_for_wide_registers():
    """Registers of more than 10 qubits are drawn on the device: the
    outcome of each state equals the sequential draw on its probabilities
    (the uniforms here sit nowhere near a cumulative boundary), and the
    probability returned is the outcome's."""
    P = pkg()
    A = P._capi
    rng = np.random.default_rng(8)
    n, b = 12, 2
    psi = rng.normal(size=(1 << b, 1 << n)) + 1j * rng.normal(size=(1 << b, 1 << n))
    psi /= np.linalg.norm(psi, axis=1, keepdims=True)
    qubits = [int(x) for x in rng.permutation(n)[:11]]
    with P.QubitVector(n + b) as st:
        st.initialize_from_vector(psi.reshape(-1))
        q = (C.c_uint64 * 11)(*qubits)
        probs = np.empty((4, 1 << 11))
        A.check(P.lib().gbqv_probabilities_segments(st.handle, n, 4, q, 11, probs.ctypes.data_as(A.dp)), st.handle)
        for trial in range(8):
            u = rng.random(4)
            u[trial % 4] = -1.0  # no draw for one state
            out = np.empty(4, dtype=np.uint32)
            pr = np.empty(4)
            A.check(P.lib().gbqv_draw_segments(st.handle, n, 4, q, 11, u.ctypes.data_as(A.dp),
                                               out.ctypes.data_as(A.vp), pr.ctypes.data_as(A.dp)), st.handle)
            for s in range(4):
                if u[s] < 0:
                    assert out[s] == 0xFFFFFFFF
                    continue
                assert out[s] == P.simulator.discrete_draw(probs[s], u[s])
                assert pr[s] == probs[s, out[s]]


def test_wide_mid_circuit_register_matches_oracle():
    P = pkg()
    rng = np.random.default_rng(21)
    n = 12
    qc = P.QuantumCircuit(n, 2 * n)
    for q in range(n):
        qc.unitary(haar(rng, 2), [q])
    for q in range(0, n - 1, 2):
        qc.unitary(haar(rng, 4), [q, q + 1])
    order = [int(x) for x in rng.permutation(n)]
    qc.measure(order, list(range(n)))
    qc.reset(order[:11])
    for q in range(n):
        qc.unitary(haar(rng, 2), [q])
    qc.measure(list(range(n)), list(range(n, 2 * n)))
    got = P.AerSimulator().run(qc, shots=40, seed_simulator=99).get_counts()
    assert got == oracle_counts(P, qc, 40, 99)


def _measured_feedback(P, n, rng, gate_set="unitary"):
    """Mid-circuit measurements and conditioned gates, no reset."""
    qc = P.QuantumCircuit(n, 2 * n)
    for r in range(3):
        for q in range(n):
            qc.u3(*rng.uniform(0, 2 * np.pi, 3), q)
        for q in range(r % 2, n - 1, 2):
            qc.cx(q, q + 1)
        qc.measure([r % n, (r + 2) % n], [2 * r, 2 * r + 1])
        qc.u3(*rng.uniform(0, 2 * np.pi, 3), (r + 1) % n).c_if([2 * r], 1)
        qc.cx((r + 1) % n, (r + 3) % n).c_if([2 * r, 2 * r + 1], 2)
    qc.measure(list(range(n)), list(range(n, 2 * n)))
    return qc


def test_density_matrix_shots_equal_statevector_shots_when_ideal():
    """Without noise the density-matrix method's shots draw from the same
    probabilities with the same per-shot uniforms: identical counts."""
    P = pkg()
    qc = _measured_feedback(P, 4, np.random.default_rng(12))
    dm = P.AerSimulator(method="density_matrix").run(qc, shots=60, seed_simulator=8, memory=True)
    sv = P.AerSimulator().run(qc, shots=60, seed_simulator=8, memory=True)
    assert dm.get_memory() == sv.get_memory()


def test_noisy_density_matrix_shots_match_oracle():
    P = pkg()
    n = 4
    e1 = P.depolarizing_error(0.05, 1).compose(P.amplitude_damping_error(0.1))
    nm = P.NoiseModel()
    nm.add_all_qubit_quantum_error(e1, ["u3"])
    nm.add_all_qubit_quantum_error(e1.tensor(e1), ["cx"])
    qc = _measured_feedback(P, n, np.random.default_rng(13))
    sim = P.AerSimulator(method="density_matrix", noise_model=nm)
    got = sim.run(qc, shots=40, seed_simulator=4).get_counts()
    ndraw = sum(1 for ins in qc.data if ins.kind == "measure")
    want = {}
    for shot in range(40):
        o = O.OracleDM(n)
        u = P.uniforms(4 + shot, ndraw)
        used, mem = 0, 0
        for ins in qc.data:
            if ins.condition is not None:
                cb, val = ins.condition
                if any(((mem >> c) & 1) != ((val >> i) & 1) for i, c in enumerate(cb)):
                    continue
            if ins.kind == "measure":
                probs = o.probabilities(ins.qubits)
                k = P.simulator.discrete_draw(probs, u[used])
                used += 1
                diag = np.zeros(1 << len(ins.qubits), dtype=complex)
                diag[k] = 1 / np.sqrt(probs[k])
                o.apply_diagonal_unitary_matrix(ins.qubits, diag)
                for i, c in enumerate(ins.clbits):
                    mem = (mem & ~(1 << c)) | (((k >> i) & 1) << c)
                continue
            plain = P.circuit.Instruction(ins.kind, ins.name, ins.qubits, ins.params, ins.data, ins.clbits)
            for op in sim._with_noise([plain]):
                if op.kind == "superop":
                    o.apply_superop_matrix(op.qubits, op.data)
                elif op.name == "u3":
                    o.apply_unitary_matrix(op.qubits, O.u3(*op.params))
                else:
                    o.apply_cnot(*op.qubits)
        key = format(mem, f"0{2 * n}b")
        want[key] = want.get(key, 0) + 1
    assert got == want


@pytest.mark.parametrize("method", ["statevector", "density_matrix"])
def test_readout_errors_deterministic(method):
    """Readout errors with 0/1 probabilities: sampled final measurements, a
    two-qubit error on exactly the measured qubits, and a readout error
    ahead of a classical condition in a circuit run shot by shot."""
    P = pkg()
    always0 = P.ReadoutError([[1, 0], [1, 0]])
    flip = P.ReadoutError([[0, 1], [1, 0]])
    nm = P.NoiseModel()
    nm.add_all_qubit_readout_error(flip)
    nm.add_readout_error(always0, [0])
    qc = P.QuantumCircuit(3, 3).x(0).measure([0, 1, 2], [0, 1, 2])
    res = P.AerSimulator(method=method, noise_model=nm).run(qc, shots=50, seed_simulator=1, memory=True)
    assert res.get_counts() == {"110": 50}           # qubit 0 reads 0, qubits 1 and 2 read 1
    assert res.get_memory() == ["0x6"] * 50
    nm2 = P.NoiseModel()
    nm2.add_readout_error(P.ReadoutError(np.eye(4)[[3, 2, 1, 0]]), [0, 1])   # reads a ^ 3
    qc2 = P.QuantumCircuit(2, 2).x(0).measure([0, 1], [0, 1])
    assert P.AerSimulator(method=method, noise_model=nm2).run(qc2, shots=20, seed_simulator=2).get_counts() == {"10": 20}
    nm3 = P.NoiseModel()
    nm3.add_readout_error(always0, [0])
    qc3 = P.QuantumCircuit(2, 2).x(0).measure(0, 0)
    qc3.x(1).c_if(0, 1)
    qc3.measure(1, 1)
    assert P.AerSimulator(method=method).run(qc3, shots=30, seed_simulator=3).get_counts() == {"11": 30}
    assert P.AerSimulator(method=method, noise_model=nm3).run(qc3, shots=30, seed_simulator=3).get_counts() == {"00": 30}
