"""set_statevector / set_density_matrix / set_unitary (the reference's
SetStatevector, SetDensityMatrix and SetUnitary instructions,
qiskit_aer/library/set_instructions/; applied by
Statevector::State / DensityMatrix::State as initialize_from_vector /
initialize_from_matrix, statevector_state.hpp:538-540,
densitymatrix_state.hpp:456-461) on the host: size checks, where they
split the op list, and what each method does with them."""
import numpy as np
import pytest

from _pkg import pkg


class FakeState:
    def __init__(self):
        self.calls = []

    def initialize_from_vector(self, v):
        self.calls.append(("vector", np.asarray(v)))

    def initialize_from_matrix(self, m):
        self.calls.append(("matrix", np.asarray(m)))


def test_sizes_are_checked():
    P = pkg()
    qc = P.QuantumCircuit(2)
    with pytest.raises(ValueError, match="statevector"):
        qc.set_statevector(np.ones(8) / np.sqrt(8))
    with pytest.raises(ValueError, match="density matrix"):
        qc.set_density_matrix(np.eye(2) / 2)
    with pytest.raises(ValueError, match="unitary"):
        qc.set_unitary(np.eye(8))


def test_set_splits_the_op_list_in_circuit_order():
    P = pkg()
    v = np.array([0, 1, 1j, 0]) / np.sqrt(2)
    qc = P.QuantumCircuit(2).h(0)
    qc.save_statevector("before")
    qc.set_statevector(v)
    qc.cx(0, 1)
    qc.save_statevector("after")
    sim = P.AerSimulator(fusion_enable=False)
    segments, meas, saves, _ = sim.compile(qc)
    assert [nc.num_ops() for _, nc in segments] == [1, 1]
    assert [(p, ins.kind, ins.name) for p, ins in saves] == [(1, "save", "statevector"), (1, "set", "statevector"),
                                                            (2, "save", "statevector")]
    # a circuit with a set instruction is not run on the stack of bindings
    assert not sim._bound_batchable(qc)
    # the shot-by-shot paths refuse it
    qc2 = P.QuantumCircuit(1, 1).measure(0, 0).x(0)
    qc2.set_statevector([1, 0])
    with pytest.raises(NotImplementedError, match="set instructions"):
        sim._run_shots(qc2, 4, 1)


def test_each_method_initialises_its_state():
    P = pkg()
    v = np.array([0.6, 0.8j])
    qc = P.QuantumCircuit(1)
    qc.set_statevector(v)
    ins = qc.data[0]
    st = FakeState()
    P.AerSimulator()._save(st, ins, {})
    assert st.calls[0][0] == "vector" and np.allclose(st.calls[0][1], v)
    st = FakeState()
    P.AerSimulator(method="density_matrix")._save(st, ins, {})
    assert st.calls[0][0] == "matrix" and np.allclose(st.calls[0][1], np.outer(v, v.conj()))
    rho = np.array([[0.5, 0.1], [0.1, 0.5]])
    qc.set_density_matrix(rho)
    st = FakeState()
    P.AerSimulator(method="density_matrix")._save(st, qc.data[1], {})
    assert st.calls[0][0] == "matrix" and np.allclose(st.calls[0][1], rho)
    with pytest.raises(ValueError, match="not supported by the statevector method"):
        P.AerSimulator()._save(FakeState(), qc.data[1], {})
    qc.set_unitary(np.array([[0, 1], [1, 0]]))
    st = FakeState()
    sim = P.AerSimulator(method="unitary")
    sim._check_unitary_circuit(qc.copy().__class__(1).set_unitary(np.eye(2)))
    sim._save(st, qc.data[2], {})
    assert st.calls[0][0] == "matrix"
    with pytest.raises(ValueError, match="not supported by the unitary method"):
        sim._save(FakeState(), ins, {})


class FakeCopies:
    def copy_to_vector(self):
        return "vector"

    def copy_to_matrix(self):
        return "matrix"


def test_save_state_key_and_form_per_method():
    """save_state saves the method's own state under the method's name
    (statevector_state.hpp:597-615, densitymatrix_state.hpp:562), or under
    its label."""
    P = pkg()
    qc = P.QuantumCircuit(1).save_state().save_state("mine")
    for method, form in (("statevector", "vector"), ("density_matrix", "matrix"), ("unitary", "matrix")):
        sim, data = P.AerSimulator(method=method), {}
        for ins in qc.data:
            sim._save(FakeCopies(), ins, data)
        assert data == {method: form, "mine": form}
    P.AerSimulator(method="unitary")._check_unitary_circuit(qc)
