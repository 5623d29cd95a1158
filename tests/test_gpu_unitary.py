"""The unitary method (QubitUnitary::State over QV::UnitaryMatrix,
src/simulators/unitary/): a 2^n x 2^n matrix stored column-major over 2n
vector qubits, starting as the identity; every gate multiplies it from the
left.  Against the oracle doing what the reference's UnitaryMatrix does
(the QubitVector operations on the 2n-qubit vec(I), gate qubits below n),
with and without Fusion (threshold halved for the unitary method), both
precisions; and the unitary method's op-set errors."""
import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O
from test_gpu_bind import FIXED_GATES, PARAM_GATES, haar, oracle_gate

pytestmark = pytest.mark.gpu


def random_circuit(P, n, count, rng):
    qc = P.QuantumCircuit(n)
    for _ in range(count):
        r = rng.random()
        if r < 0.45:
            name, k, npar = PARAM_GATES[rng.integers(len(PARAM_GATES))]
            if k > n:
                continue
            qc.append_gate(name, [int(x) for x in rng.choice(n, k, replace=False)],
                           [float(x) for x in rng.uniform(-np.pi, np.pi, npar)])
        elif r < 0.85:
            name, k = FIXED_GATES[rng.integers(len(FIXED_GATES))]
            if k > n:
                continue
            qc.append_gate(name, [int(x) for x in rng.choice(n, k, replace=False)])
        else:
            k = min(n, int(rng.integers(1, 4)))
            qc.unitary(haar(rng, 1 << k), [int(x) for x in rng.choice(n, k, replace=False)])
    return qc


def oracle_unitary(qc):
    n = qc.num_qubits
    o = O.OracleQV(2 * n, np.eye(1 << n, dtype=complex).reshape(-1, order="F"))
    for ins in qc.data:
        if ins.kind == "unitary":
            o.apply_matrix(ins.qubits, ins.data)
        elif ins.kind == "gate":
            oracle_gate(o, ins.name, ins.qubits, ins.params)
    return o.data.reshape(1 << n, 1 << n, order="F")


@pytest.mark.parametrize("n", [1, 3, 6, 9])
@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("single", 5e-5)])
def test_unitary_method_matches_oracle(n, precision, tol):
    P = pkg()
    rng = np.random.default_rng(900 + n)
    qc = random_circuit(P, n, 60, rng)
    qc.save_unitary()
    res = P.AerSimulator(method="unitary", precision=precision).run(qc)
    U = res.get_unitary()
    assert U.shape == (1 << n, 1 << n)
    want = oracle_unitary(qc)
    np.testing.assert_allclose(U, want, rtol=0, atol=tol)
    np.testing.assert_allclose(U.conj().T @ U, np.eye(1 << n), atol=tol * 10)
    if n >= 8:
        assert res.metadata()["fusion"]["applied"]
        unfused = P.AerSimulator(method="unitary", precision=precision, fusion_enable=False).run(qc).get_unitary()
        np.testing.assert_allclose(unfused, want, rtol=0, atol=tol)


def test_unitary_matrix_handle():
    P = pkg()
    with P.UnitaryMatrix(3) as u:
        np.testing.assert_array_equal(u.copy_to_matrix(), np.eye(8))
        m = haar(np.random.default_rng(1), 8)
        u.initialize_from_matrix(m)
        u.apply_matrix([1], np.array([[0, 1], [1, 0]]))
        x1 = np.kron(np.eye(2), np.kron([[0, 1], [1, 0]], np.eye(2)))
        np.testing.assert_allclose(u.copy_to_matrix(), x1 @ m, atol=1e-15)
        u.initialize()
        np.testing.assert_array_equal(u.copy_to_matrix(), np.eye(8))


def test_unitary_method_rejects_measurement():
    P = pkg()
    qc = P.QuantumCircuit(2).h(0).measure_all()
    with pytest.raises(ValueError, match="invalid instruction"):
        P.AerSimulator(method="unitary").run(qc)
