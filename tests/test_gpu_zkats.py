"""The reference's own known-answer tests for gates (tests/golden/ref_kats.json,
from test/terra/reference/ref_1q_clifford.py, ref_2q_clifford.py,
ref_non_clifford.py and ref_rotation.py) through AerSimulator on the GPU:
the statevector method's final state and outcome probabilities, and the
unitary method's matrix, against the reference's targets including the
global phase."""
import numpy as np
import pytest

from _pkg import pkg
from test_ref_kats_cpu import KATS, cplx

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
