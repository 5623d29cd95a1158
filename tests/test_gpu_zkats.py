"""The reference's own known-answer tests through AerSimulator on the GPU.
Gates (tests/golden/ref_kats.json, from test/terra/reference/
ref_1q_clifford.py, ref_2q_clifford.py, ref_non_clifford.py and
ref_rotation.py): the statevector method's final state and outcome
probabilities, and the unitary method's matrix, against the reference's
targets including the global phase.  Noise (tests/golden/
ref_noise_kats.json, from ref_pauli_noise.py, ref_reset_noise.py,
ref_kraus_noise.py, and ref_reset.py's noiseless resets): the density-matrix
method's sampled counts equal the oracle's density matrix sampled with the
same uniforms, and that matrix gives the reference's target distribution
(tests/test_ref_noise_kats_cpu.py)."""
import numpy as np
import pytest

from _pkg import pkg
from test_ref_kats_cpu import KATS, cplx
from test_ref_noise_kats_cpu import (NOISE_KATS, RESET_KATS, circuit_of as noisy_circuit_of, kat_id, noise_model_of,
                                     oracle_state)

pytestmark = pytest.mark.gpu


def circuit_of(P, case):
    qc = P.QuantumCircuit(case["num_qubits"])
    for name, qubits, params in case["ops"]:
        qc.append_gate(name, qubits, params)
    return qc


def test_statevector_method_reference_kats():
    P = pkg()
    sim = P.AerSimulator(method="statevector")
    for case in KATS:
        n = case["num_qubits"]
        qc = circuit_of(P, case)
        qc.save_statevector()
        psi = np.asarray(sim.run(qc).get_statevector())
        where = f"{case['source']}[{case['index']}]"
        if "statevector" in case:
            np.testing.assert_allclose(psi, cplx(case["statevector"]), atol=1e-12, err_msg=where)
        want = np.zeros(1 << n)
        for k, p in case["probabilities"].items():
            want[int(k)] = p
        np.testing.assert_allclose(np.abs(psi) ** 2, want, atol=1e-12, err_msg=where)


def test_unitary_method_reference_kats():
    P = pkg()
    sim = P.AerSimulator(method="unitary")
    checked = 0
    for case in KATS:
        if "unitary" not in case:
            continue
        n = case["num_qubits"]
        qc = circuit_of(P, case)
        qc.save_unitary()
        U = np.asarray(sim.run(qc).get_unitary())
        want = cplx(case["unitary"]).reshape(1 << n, 1 << n, order="F")
        np.testing.assert_allclose(U, want, atol=1e-12, err_msg=f"{case['source']}[{case['index']}]")
        checked += 1
    assert checked >= 90


@pytest.mark.parametrize("case", NOISE_KATS + RESET_KATS, ids=kat_id)
def test_density_matrix_reference_noise_kats(case):
    P = pkg()
    sim = P.AerSimulator(method="density_matrix", noise_model=noise_model_of(P, case["noise"]))
    qc = noisy_circuit_of(P, case)
    shots, seed = 2000, 11
    got = sim.run(qc, shots=shots, seed_simulator=seed).get_counts()
    o, meas = oracle_state(sim, qc)
    qubits = [q for m in meas for q in m.qubits]
    clbits = [c for m in meas for c in m.clbits]
    want = sim._counts(o.sample_measure(P.uniforms(seed, shots)), qubits, clbits, case["num_clbits"])
    assert got == want
