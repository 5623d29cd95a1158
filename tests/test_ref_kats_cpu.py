"""The reference's own known-answer tests for gates (test/terra/reference/
ref_1q_clifford.py, ref_2q_clifford.py, ref_non_clifford.py, ref_rotation.py;
recorded in tests/golden/ref_kats.json by gen_ref_kats.py), on the host.

Each circuit is assembled by the engine (gbqv_circuit_gate: the gate names,
parameter order and qubit order of the reference's gate dispatch) and every
op's matrix, as the engine defines it (gbqv_circuit_op_matrix), is applied by
the oracle.  The final statevector, the circuit unitary and the outcome
probabilities must equal the reference's targets exactly, including the
global phase (the reference compares with ignore_phase=False)."""
import json
from pathlib import Path

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

KATS = json.loads((Path(__file__).parent / "golden" / "ref_kats.json").read_text())["cases"]


def cplx(pairs):
    a = np.asarray(pairs, dtype=float)
    return a[:, 0] + 1j * a[:, 1]


def engine_ops(case):
    P = pkg()
    qc = P.QuantumCircuit(case["num_qubits"])
    for name, qubits, params in case["ops"]:
        qc.append_gate(name, qubits, params)
    nc = P.NativeCircuit(case["num_qubits"], qc.data)
    return [(q, nc.op_matrix(i)) for i, (_, _, q) in enumerate(nc.ops())]


def case_id(case):
    return f"{case['source'].split(':')[1]}[{case['index']}]"


def test_fixture_covers_the_reference_gate_set():
    names = {op[0] for c in KATS for op in c["ops"]}
    assert {"h", "x", "y", "z", "s", "sdg", "t", "tdg", "cx", "cz", "swap", "ecr", "ccx", "cswap", "cp", "cu",
            "rx", "ry", "rz", "id", "delay"} <= names
    assert len(KATS) >= 100


@pytest.mark.parametrize("case", KATS, ids=case_id)
def test_reference_kat(case):
    n = case["num_qubits"]
    ops = engine_ops(case)
    o = O.OracleQV(n)
    for q, m in ops:
        o.apply_matrix(q, m)
    if "statevector" in case:
        np.testing.assert_allclose(o.data, cplx(case["statevector"]), atol=1e-12)
    probs = o.probabilities()
    want = np.zeros(1 << n)
    for k, p in case["probabilities"].items():
        want[int(k)] = p
    np.testing.assert_allclose(probs, want, atol=1e-12)
    if "unitary" in case:
        u = O.OracleQV(2 * n, np.eye(1 << n, dtype=complex).reshape(-1, order="F"))
        for q, m in ops:
            u.apply_matrix(q, m)
        np.testing.assert_allclose(u.data, cplx(case["unitary"]), atol=1e-12)
