"""End-to-end circuits through AerSimulator on the GPU against the oracle:
a quantum-volume circuit (fused) vs the oracle applying every unfused gate,
counts identical for the same RngEngine seed, fusion on == fusion off, and
the noisy density-matrix workload with Pauli expectation values."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O
from test_fusion_cpu import haar, qv_circuit

pytestmark = pytest.mark.gpu


def oracle_run(qc):
    o = O.OracleQV(qc.num_qubits)
    for ins in qc.data:
        if ins.kind == "unitary":
            o.apply_matrix(ins.qubits, ins.data)
    return o


@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("single", 2e-5)])
def test_qv_circuit_fused_vs_oracle(precision, tol):
    P = pkg()
    n = 16
    qc = qv_circuit(n, 16, 2024)
    qc.save_statevector()
    qc.measure_all()
    sim = P.AerSimulator(precision=precision)
    res = sim.run(qc, shots=1024, seed_simulator=42)
    assert res.metadata()["fusion"]["applied"]
    o = oracle_run(qc)
    np.testing.assert_allclose(res.get_statevector(), o.data, atol=tol)
    if precision == "double":
        samples = o.sample_measure(P.uniforms(42, 1024))
        want = {}
        for s in samples:
            key = format(int(s), f"0{n}b")
            want[key] = want.get(key, 0) + 1
        assert res.get_counts() == want


def test_fusion_on_off_identical_counts():
    P = pkg()
    qc = qv_circuit(15, 10, 7)
    qc.measure_all()
    a = P.AerSimulator().run(qc, shots=2000, seed_simulator=5).get_counts()
    b = P.AerSimulator(fusion_enable=False).run(qc, shots=2000, seed_simulator=5).get_counts()
    c = P.AerSimulator(blocking_enable=False).run(qc, shots=2000, seed_simulator=5).get_counts()
    assert a == b == c


def test_noisy_density_matrix_vs_oracle():
    P = pkg()
    n = 6
    rng = np.random.default_rng(31)
    e1 = P.depolarizing_error(1e-3, 1).compose(P.amplitude_damping_error(2e-3))
    nm = P.NoiseModel()
    nm.add_all_qubit_quantum_error(e1, ["u3"])
    nm.add_all_qubit_quantum_error(e1.tensor(e1), ["cx"])
    qc = P.QuantumCircuit(n)
    for _ in range(5):
        for q in range(n):
            qc.u3(*rng.uniform(0, 2 * np.pi, 3), q)
        perm = rng.permutation(n)
        for a, b in zip(perm[0::2], perm[1::2]):
            qc.cx(int(a), int(b))
    terms = []
    for _ in range(20):
        k = int(rng.integers(1, 4))
        q = [int(x) for x in rng.choice(n, k, replace=False)]
        terms.append((float(rng.normal()), "".join(rng.choice(list("IXYZ"), k)), q))
    qc.save_density_matrix()
    qc.save_expectation_value(terms)
    sim = P.AerSimulator(method="density_matrix", noise_model=nm, fusion_threshold=2)
    res = sim.run(qc)
    assert res.metadata()["fusion"]["method"] == "superop"
    # oracle: unfused gates + superops
    o = O.OracleDM(n)
    for ins in sim._with_noise(qc.split_final()[0]):
        if ins.kind == "gate" and ins.name == "u3":
            o.apply_unitary_matrix(ins.qubits, O.u3(*ins.params))
        elif ins.kind == "gate" and ins.name == "cx":
            o.apply_cnot(*ins.qubits)
        elif ins.kind == "superop":
            o.apply_superop_matrix(ins.qubits, ins.data)
    rho = res.data()["density_matrix"]
    np.testing.assert_allclose(rho.reshape(-1, order="F"), o.data, atol=1e-12)
    want = sum(c * o.expval_pauli(q, lab) for c, lab, q in terms)
    assert abs(res.data()["expectation_value"] - want) < 1e-12


def test_density_matrix_with_relaxation_and_local_errors_vs_oracle():
    """Thermal relaxation on every u3, a Pauli + reset error on the u3 of
    qubit 2 in its place, a two-qubit error on cx(0, 1) only and relaxation
    on both qubits of every other cx: the density matrix after fusion of
    gates and superoperators equals the oracle applying each gate and its
    error in turn."""
    P = pkg()
    n = 5
    rng = np.random.default_rng(44)
    t = P.thermal_relaxation_error(50.0, 70.0, 1.5, 0.05)
    nm = P.NoiseModel()
    nm.add_all_qubit_quantum_error(t, ["u3"])
    nm.add_quantum_error(P.pauli_error([("X", 0.02), ("Z", 0.03), ("I", 0.95)]).compose(P.reset_error(0.01, 0.02)),
                         "u3", [2])
    nm.add_all_qubit_quantum_error(t.tensor(P.thermal_relaxation_error(40.0, 30.0, 3.0)), ["cx"])
    nm.add_quantum_error(P.depolarizing_error(0.04, 2), "cx", [0, 1])
    qc = P.QuantumCircuit(n)
    for _ in range(4):
        for q in range(n):
            qc.u3(*rng.uniform(0, 2 * np.pi, 3), q)
        qc.cx(0, 1).cx(2, 3).cx(1, 4).cx(4, 0)
    qc.save_density_matrix()
    sim = P.AerSimulator(method="density_matrix", noise_model=nm, fusion_threshold=2)
    rho = sim.run(qc).data()["density_matrix"]
    o = O.OracleDM(n)
    for ins in sim._with_noise(qc.split_final()[0]):
        if ins.kind == "gate" and ins.name == "u3":
            o.apply_unitary_matrix(ins.qubits, O.u3(*ins.params))
        elif ins.kind == "gate" and ins.name == "cx":
            o.apply_cnot(*ins.qubits)
        elif ins.kind == "superop":
            o.apply_superop_matrix(ins.qubits, ins.data)
    np.testing.assert_allclose(rho.reshape(-1, order="F"), o.data, atol=1e-12)
    assert abs(np.trace(rho) - 1) < 1e-12
