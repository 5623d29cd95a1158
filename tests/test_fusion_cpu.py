"""Fusion pass (Fusion::optimize_circuit, src/transpile/fusion.hpp) checks on
the host: thresholds and metadata, the fusers' structural behaviour, and that
every fused op equals the product of the ops it replaced (composed with the
oracle).  Mirrors test/terra/backends/aer_simulator/test_fusion.py."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O


def haar(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def qv_circuit(n, depth, seed):
    """Quantum-volume-style: per layer a seeded permutation into pairs, Haar SU(4) each."""
    P = pkg()
    rng = np.random.default_rng(seed)
    qc = P.QuantumCircuit(n)
    for _ in range(depth):
        perm = rng.permutation(n)
        for a, b in zip(perm[0::2], perm[1::2]):
            u = haar(rng, 4)
            u = u / np.linalg.det(u) ** 0.25
            qc.unitary(u, [int(a), int(b)])
    return qc


def full_unitary_of(ops_list, n):
    """Compose [(qubits, matrix)] into a full 2^n unitary with the oracle."""
    u = O.OracleQV(2 * n, np.eye(1 << n, dtype=complex).reshape(-1, order="F"))
    for q, m in ops_list:
        u.apply_matrix(q, m)
    return u.data.reshape(1 << n, 1 << n, order="F")


def native_ops(nc):
    out = []
    for i, (t, name, q) in enumerate(nc.ops()):
        m = nc.op_matrix(i)
        if t == 2:  # diagonal
            m = np.diag(m).reshape(-1, order="F")
        out.append((q, m))
    return out


def test_threshold_and_metadata():
    P = pkg()
    sim = P.AerSimulator()
    qc = qv_circuit(6, 3, 1)
    segs, _, _, meta = sim.compile(qc)
    assert meta["fusion"]["enabled"] is True
    assert meta["fusion"]["applied"] is False          # 6 <= threshold 14
    assert meta["fusion"]["threshold"] == 14 and meta["fusion"]["max_fused_qubits"] == 5
    sim2 = P.AerSimulator(fusion_threshold=5)
    segs, _, _, meta = sim2.compile(qc)
    assert meta["fusion"]["applied"] is True and meta["fusion"]["method"] == "unitary"
    dm = P.AerSimulator(method="density_matrix")
    cfg = dm.fusion_config()
    assert cfg.threshold == 7 and cfg.max_qubit == 2
    off = P.AerSimulator(fusion_enable=False)
    _, _, _, meta = off.compile(qc)
    assert meta["fusion"] == {"enabled": False}


@pytest.mark.parametrize("n,depth,maxq", [(6, 4, 5), (7, 5, 3), (5, 6, 4), (8, 3, 2)])
def test_fused_circuit_equals_unfused(n, depth, maxq):
    P = pkg()
    qc = qv_circuit(n, depth, 100 + n)
    sim = P.AerSimulator(fusion_threshold=1, fusion_max_qubit=maxq)
    segs, _, _, meta = sim.compile(qc)
    nc = segs[0][1]
    fused = native_ops(nc)
    assert meta["fusion"]["applied"]
    assert len(fused) < len(qc.data)
    assert all(len(q) <= maxq for q, _ in fused)
    ref = full_unitary_of([(i.qubits, i.data) for i in qc.data], n)
    got = full_unitary_of(fused, n)
    np.testing.assert_allclose(got, ref, atol=1e-12)


def test_gate_fusion_random_ops():
    """test_fusion_operations: random named gates, fused == unfused."""
    P = pkg()
    rng = np.random.default_rng(5)
    n = 6
    qc = P.QuantumCircuit(n)
    one = ["h", "x", "y", "z", "s", "sdg", "t", "tdg", "sx", "sxdg"]
    for _ in range(60):
        r = rng.integers(0, 5)
        if r == 0:
            qc.append_gate(str(rng.choice(one)), [int(rng.integers(n))])
        elif r == 1:
            qc.append_gate(str(rng.choice(["rx", "ry", "rz", "p"])), [int(rng.integers(n))], [rng.uniform(-3, 3)])
        elif r == 2:
            a, b = rng.choice(n, 2, replace=False)
            qc.append_gate(str(rng.choice(["cx", "cz", "cy", "swap"])), [int(a), int(b)])
        elif r == 3:
            a, b = rng.choice(n, 2, replace=False)
            qc.append_gate(str(rng.choice(["cp", "rzz", "rxx", "crx"])), [int(a), int(b)], [rng.uniform(-3, 3)])
        else:
            qc.append_gate("u3", [int(rng.integers(n))], list(rng.uniform(-3, 3, 3)))
    sim = P.AerSimulator(fusion_threshold=1)
    segs, _, _, meta = sim.compile(qc)
    fused = native_ops(segs[0][1])
    unf = P.NativeCircuit(n, qc.data)
    ref = full_unitary_of(native_ops(unf), n)
    np.testing.assert_allclose(full_unitary_of(fused, n), ref, atol=1e-12)


def test_diagonal_fusion_cx_u1_cx():
    """test_fusion_diagonal (test_fusion.py:514): cx - p - cx chains fuse to a diagonal."""
    P = pkg()
    n = 4
    qc = P.QuantumCircuit(n)
    for i in range(3):
        qc.cx(i, i + 1).p(0.1 * (i + 1), i + 1).cx(i, i + 1)
    qc.h(0)
    sim = P.AerSimulator(fusion_threshold=1)
    segs, _, _, meta = sim.compile(qc)
    ops = segs[0][1].ops()
    assert ops[0][0] == 2, ops      # a diagonal op first
    unf = P.NativeCircuit(n, qc.data)
    np.testing.assert_allclose(full_unitary_of(native_ops(segs[0][1]), n),
                               full_unitary_of(native_ops(unf), n), atol=1e-12)


def test_superop_fusion_dm():
    P = pkg()
    n = 4
    nm = P.NoiseModel()
    err = P.depolarizing_error(0.01, 1).compose(P.amplitude_damping_error(0.02))
    nm.add_all_qubit_quantum_error(err, ["u3", "h"])
    nm.add_all_qubit_quantum_error(err.tensor(err), ["cx"])
    qc = P.QuantumCircuit(n)
    rng = np.random.default_rng(3)
    for _ in range(4):
        for q in range(n):
            qc.u3(*rng.uniform(0, 2 * np.pi, 3), q)
        qc.cx(0, 1).cx(2, 3)
    sim = P.AerSimulator(method="density_matrix", noise_model=nm, fusion_threshold=1)
    segs, _, _, meta = sim.compile(qc)
    assert meta["fusion"]["method"] == "superop"
    ops = segs[0][1].ops()
    assert all(len(q) <= 2 for _, _, q in ops)
    assert any(t == 3 for t, _, _ in ops)


def test_noise_tensor_matches_kraus_of_kron():
    P = pkg()
    rng = np.random.default_rng(0)
    ua, ub = haar(rng, 2), haar(rng, 2)
    ea = P.QuantumError.from_kraus([ua])
    eb = P.QuantumError.from_kraus([ub])
    want = O.kraus_superop([np.kron(ub, ua)])
    np.testing.assert_allclose(eb.tensor(ea).superop, want, atol=1e-14)
    np.testing.assert_allclose(P.depolarizing_error(1e-3, 1).superop, O.depolarizing_superop(1e-3), atol=1e-15)
    np.testing.assert_allclose(P.amplitude_damping_error(2e-3).superop, O.amplitude_damping_superop(2e-3), atol=1e-15)
