"""Cache-blocked runs (one HBM pass for a run of small ops) in both forms:
the register-tile kernel (blocking mode 1, gbqv_runreg.cu) and the
shared-memory kernel (mode 2), against one kernel per op (mode 0) and the
oracle applying every gate: random circuits of 1-2 qubit unitaries, real
rotations, diagonals on 1-3 qubits and multi-controlled X gates, on states
whose tiles use every register width (11-16 qubits), both precisions."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def haar(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def random_small_ops(P, n, count, rng):
    qc = P.QuantumCircuit(n)
    for _ in range(count):
        r = rng.random()
        if r < 0.25:
            qc.unitary(haar(rng, 2), [int(rng.integers(n))])
        elif r < 0.45:
            qc.unitary(haar(rng, 4), [int(x) for x in rng.choice(n, 2, replace=False)])
        elif r < 0.6:
            qc.ry(float(rng.uniform(-3, 3)), int(rng.integers(n)))
        elif r < 0.75:
            k = int(rng.integers(1, 4))
            qc.diagonal(np.exp(1j * rng.uniform(-3, 3, 1 << k)), [int(x) for x in rng.choice(n, k, replace=False)])
        else:
            k = int(rng.integers(1, 4))
            qc.append_gate({1: "x", 2: "cx", 3: "ccx"}[k], [int(x) for x in rng.choice(n, k, replace=False)])
    return qc


def oracle_of(qc):
    o = O.OracleQV(qc.num_qubits)
    for ins in qc.data:
        if ins.kind == "unitary":
            o.apply_matrix(ins.qubits, ins.data)
        elif ins.kind == "diagonal":
            o.apply_diagonal_matrix(ins.qubits, ins.data)
        elif ins.name == "ry":
            o.apply_mcu(ins.qubits, O.rotation_matrix(1, ins.params[0]))
        else:
            o.apply_mcx(ins.qubits)
    return o.data


def run_mode(P, qc, precision, mode):
    with P.QubitVector(qc.num_qubits, precision) as st:
        P._capi.check(P.lib().gbqv_set_blocking(st.handle, mode), st.handle)
        st.initialize()
        nc = P.NativeCircuit(qc.num_qubits, qc.data)
        P._capi.check(P.lib().gbqv_execute(st.handle, nc.handle), st.handle)
        return st.copy_to_vector()


@pytest.mark.parametrize("n", [11, 12, 13, 14, 16])
@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("single", 2e-5)])
def test_run_forms_agree_with_oracle(n, precision, tol):
    P = pkg()
    rng = np.random.default_rng(600 + n)
    qc = P.QuantumCircuit(n)
    for q in range(n):
        qc.unitary(haar(rng, 2), [q])  # spread the amplitude over the whole state
    qc.data += random_small_ops(P, n, 120, rng).data
    want = oracle_of(qc)
    got = {m: run_mode(P, qc, precision, m) for m in (0, 1, 2)}
    for m in (0, 1, 2):
        np.testing.assert_allclose(got[m], want, rtol=0, atol=tol)
    if precision == "double":
        # the same products in both run forms (summation order may differ in lane ops)
        assert np.max(np.abs(got[1] - got[2])) < 1e-13
