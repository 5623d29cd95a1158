"""Circuits that cannot be measure-sampled, run shot by shot
(CircuitExecutor::run_circuit_shots): mid-circuit measurements, resets and
classically conditioned ops.  Counts equal, bit for bit, the same per-shot
algorithm run on the oracle (the reference's QubitVector arithmetic) with the
same per-shot seeds seed + i; deterministic circuits (teleportation with
conditioned corrections, reset) give their one outcome."""
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
            elif ins.kind in ("measure", "reset"):
                probs = o.probabilities(ins.qubits)
                k = P.simulator.discrete_draw(probs, u[used])
                used += 1
                dim = 1 << len(ins.qubits)
                diag = np.zeros(dim, dtype=complex)
                diag[k] = 1 / np.sqrt(probs[k])
                o.apply_diagonal_matrix(ins.qubits, diag)
                final = k if ins.kind == "measure" else 0
                if final != k:
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
