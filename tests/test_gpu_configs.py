"""The four single-instance workloads at (or near) their stated sizes, through
the engine's public API on the GPU, against the oracle (the C restatement of
Aer's QubitVector / DensityMatrix, OpenMP on every host core).

* 20-qubit quantum-volume circuit, 20 layers, complex128: the statevector
  within 1e-12 of the oracle applying every unfused SU(4), and the counts of
  1024 shots identical for the same seed (the reference's uniforms).
* The same family at 28 qubits x 30 layers (4.3 GB complex128 state): Aer's
  Fusion emits dense 4-qubit ops, which run on the tcgen05 digit-slice kernel;
  statevector within 1e-12 of the oracle applying every unfused gate; counts
  identical.  (30 qubits needs 17 GB twice on the host and ~3 min of oracle
  time; 28 qubits runs the same kernel and fusion on every op.)
* 14-qubit noisy density matrix (2^28-entry rho, 4.3 GB): U3 layers + CX
  pairing, depolarizing p=1e-3 then amplitude damping gamma=2e-3 after every
  gate, fused to superoperators on the GPU; rho within 1e-12 of the oracle
  applying every unfused gate and superoperator, and 50 random Pauli strings
  within 1e-12.  8 of the 40 layers: the oracle needs ~5 s per layer of this
  size on 16 cores.
* 26-qubit hardware-efficient ansatz, 12 layers (624 parameters), 200 Pauli
  terms: the energy within 1e-11 of the oracle (complex128) and within
  1e-5 x sum|c_k| (complex64, float32 state); the adjoint gradient within 1e-8 relative of
  parameter shift on a subset of parameters (complex128), and within 1e-7
  absolute of central finite differences.
"""
import os

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O
from test_fusion_cpu import qv_circuit

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _oracle_threads():
    O.build()
    O.set_threads(os.cpu_count() or 1, 14)


def _oracle_qv(qc):
    o = O.OracleQV(qc.num_qubits)
    for ins in qc.data:
        if ins.kind == "unitary":
            o.apply_matrix(ins.qubits, ins.data)
    return o


def _counts(samples, n):
    out = {}
    for s in samples:
        k = format(int(s), f"0{n}b")
        out[k] = out.get(k, 0) + 1
    return out


@pytest.mark.parametrize("n,layers", [(20, 20), (28, 30)])
def test_quantum_volume_statevector_and_counts(n, layers):
    P = pkg()
    qc = qv_circuit(n, layers, 2024 + n)
    qc.save_statevector()
    qc.measure_all()
    sim = P.AerSimulator(precision="double")
    res = sim.run(qc, shots=1024, seed_simulator=17)
    meta = res.metadata()["fusion"]
    assert meta["applied"]
    sv = res.get_statevector()
    o = _oracle_qv(qc)
    err = float(np.max(np.abs(sv - o.data)))
    print(f"QV {n}q x {layers}: max |amp - oracle| = {err:.3e}")
    assert err <= 1e-12, err
    del sv
    want = _counts(o.sample_measure(P.uniforms(17, 1024)), n)
    assert res.get_counts() == want


def test_quantum_volume_complex64_tolerance():
    """complex64 on the 20-qubit circuit: stated tolerance 2e-5 absolute per
    amplitude (float32 state, 3xTF32 dense products)."""
    P = pkg()
    qc = qv_circuit(20, 20, 2044)
    qc.save_statevector()
    res = P.AerSimulator(precision="single").run(qc)
    err = float(np.max(np.abs(res.get_statevector() - _oracle_qv(qc).data)))
    print(f"QV 20q complex64: max |amp - oracle| = {err:.3e}")
    assert err <= 2e-5, err


def test_noisy_density_matrix_14q():
    P = pkg()
    n, layers = 14, 8
    rng = np.random.default_rng(2031)
    e1 = P.depolarizing_error(1e-3, 1).compose(P.amplitude_damping_error(2e-3))
    nm = P.NoiseModel()
    nm.add_all_qubit_quantum_error(e1, ["u3"])
    nm.add_all_qubit_quantum_error(e1.tensor(e1), ["cx"])
    qc = P.QuantumCircuit(n)
    for _ in range(layers):
        for q in range(n):
            qc.u3(*rng.uniform(0, 2 * np.pi, 3), q)
        perm = rng.permutation(n)
        for a, b in zip(perm[0::2], perm[1::2]):
            qc.cx(int(a), int(b))
    terms = []
    for _ in range(50):
        k = int(rng.integers(1, 5))
        q = [int(x) for x in rng.choice(n, k, replace=False)]
        terms.append(("".join(rng.choice(list("IXYZ"), k)), q))
    for i, (lab, q) in enumerate(terms):
        qc.save_expectation_value([(1.0, lab, q)], label=f"p{i}")
    qc.save_density_matrix()
    sim = P.AerSimulator(method="density_matrix", noise_model=nm, precision="double")
    res = sim.run(qc)
    assert res.metadata()["fusion"]["method"] == "superop"
    data = res.data()
    o = O.OracleDM(n)
    for ins in sim._with_noise(qc.split_final()[0]):
        if ins.kind == "gate" and ins.name == "u3":
            o.apply_unitary_matrix(ins.qubits, O.u3(*ins.params))
        elif ins.kind == "gate" and ins.name == "cx":
            o.apply_cnot(*ins.qubits)
        elif ins.kind == "superop":
            o.apply_superop_matrix(ins.qubits, ins.data)
    rho = data["density_matrix"]
    err = float(np.max(np.abs(rho.reshape(-1, order="F") - o.data)))
    print(f"DM 14q x {layers} layers: max |rho - oracle| = {err:.3e}")
    assert err <= 1e-12, err
    del rho
    for i, (lab, q) in enumerate(terms):
        assert abs(data[f"p{i}"] - o.expval_pauli(q, lab)) <= 1e-12, (i, lab, q)


def _oracle_energy(ans, theta, ham):
    o = O.OracleQV(ans.num_qubits)
    axis = {"rx": 0, "ry": 1, "rz": 2}
    for ins in ans.instructions(theta):
        if ins.name in axis:
            o.apply_rotation(ins.qubits, axis[ins.name], ins.params[0])
        elif ins.name == "cx":
            o.apply_mcx(ins.qubits)
        else:
            raise AssertionError(ins.name)
    return sum(c * o.expval_pauli(q, lab) for (q, lab), c in zip(ham.terms, ham.coeffs))


def test_adjoint_26q_624_params():
    P = pkg()
    adj = P.adjoint
    rng = np.random.default_rng(2024)
    n, layers = 26, 12
    ans = adj.hardware_efficient_ansatz(n, layers)
    assert ans.num_params == 624
    ham = adj.random_hamiltonian(n, 200, rng)
    theta = rng.uniform(-np.pi, np.pi, ans.num_params)
    e_or = _oracle_energy(ans, theta, ham)

    eng = adj.Engine(n, "double")
    e, g = eng.energy_and_grad(ans, theta, ham)
    print(f"HEA 26q c128: |E - oracle| = {abs(e - e_or):.3e}")
    assert abs(e - e_or) <= 1e-11
    idx = [0, 1, 25, 311, 312, 600, 623]
    ps = eng.param_shift_grad(ans, theta, ham, idx)
    ps_v = np.array([ps[i] for i in idx])
    rel = float(np.linalg.norm(g[idx] - ps_v) / np.linalg.norm(ps_v))
    print(f"HEA 26q c128: adjoint vs parameter shift, relative error {rel:.3e} over {len(idx)} parameters")
    assert rel <= 1e-8, rel
    fd = eng.finite_diff_grad(ans, theta, ham, [3, 400], h=1e-5)
    for i, v in fd.items():
        assert abs(v - g[i]) <= 1e-7, (i, v, g[i])
    eng.close()

    eng = adj.Engine(n, "single")
    e32, g32 = eng.energy_and_grad(ans, theta, ham)
    scale = float(np.sum(np.abs(ham.coeffs)))
    print(f"HEA 26q c64: |E - oracle| = {abs(e32 - e_or):.3e} (sum |c| = {scale:.1f})")
    assert abs(e32 - e_or) <= 1e-5 * scale
    rel32 = float(np.linalg.norm(g32[idx] - ps_v) / np.linalg.norm(ps_v))
    print(f"HEA 26q c64: adjoint vs complex128 parameter shift, relative error {rel32:.3e}")
    assert rel32 <= 2e-3, rel32
    eng.close()
