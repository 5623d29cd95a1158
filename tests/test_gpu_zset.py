"""set_statevector / set_density_matrix / set_unitary through AerSimulator
on the GPU: each method starts from the given state, then applies the
circuit; against the oracle started from the same state."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O
from test_gpu_runs import haar

pytestmark = pytest.mark.gpu


def gate_ops(P, n, build):
    qc = P.QuantumCircuit(n)
    build(qc)
    nc = P.NativeCircuit(n, qc.data)
    return qc, [(q, nc.op_matrix(i)) for i, (_, _, q) in enumerate(nc.ops())]


def build(qc):
    qc.h(0).cx(0, 1).ry(0.3, 2).cz(1, 2).u3(0.1, 0.2, 0.3, 0)


def test_set_statevector_then_gates():
    P = pkg()
    n = 3
    rng = np.random.default_rng(31)
    v = rng.normal(size=8) + 1j * rng.normal(size=8)
    v /= np.linalg.norm(v)
    body, ops = gate_ops(P, n, build)
    qc = P.QuantumCircuit(n).x(0)
    qc.set_statevector(v)
    qc.data += body.data
    qc.save_statevector()
    o = O.OracleQV(n, v)
    for q, m in ops:
        o.apply_matrix(q, m)
    np.testing.assert_allclose(P.AerSimulator().run(qc).get_statevector(), o.data, atol=1e-12)


def test_set_density_matrix_and_pure_state():
    P = pkg()
    n = 3
    rng = np.random.default_rng(32)
    a = rng.normal(size=(8, 8)) + 1j * rng.normal(size=(8, 8))
    rho = a @ a.conj().T
    rho /= np.trace(rho)
    v = rng.normal(size=8) + 1j * rng.normal(size=8)
    v /= np.linalg.norm(v)
    body, ops = gate_ops(P, n, build)
    for start in (rho, np.outer(v, v.conj())):
        qc = P.QuantumCircuit(n)
        if start is rho:
            qc.set_density_matrix(rho)
        else:
            qc.set_statevector(v)
        qc.data += body.data
        qc.save_density_matrix()
        o = O.OracleDM(n, start.reshape(-1, order="F"))
        for q, m in ops:
            o.apply_unitary_matrix(q, m.reshape(-1))
        got = P.AerSimulator(method="density_matrix").run(qc).data()["density_matrix"]
        np.testing.assert_allclose(got.reshape(-1, order="F"), o.data, atol=1e-12)


def test_set_unitary_then_gates():
    P = pkg()
    n = 3
    U0 = haar(np.random.default_rng(33), 8)
    body, ops = gate_ops(P, n, build)
    qc = P.QuantumCircuit(n)
    qc.set_unitary(U0)
    qc.data += body.data
    qc.save_unitary()
    o = O.OracleQV(2 * n, U0.reshape(-1, order="F"))
    for q, m in ops:
        o.apply_matrix(q, m)
    got = P.AerSimulator(method="unitary").run(qc).get_unitary()
    np.testing.assert_allclose(got, o.data.reshape(8, 8, order="F"), atol=1e-12)
