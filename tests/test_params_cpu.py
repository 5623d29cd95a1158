"""Parameter binding host logic (no GPU): parameter expressions, circuit
parameters and assignment, the binding table of the C ABI with the
reference's validation messages (controller_execute.hpp:104-155,
aerbackend.py:96-144), Fusion leaving bound gates alone, and EstimatorV2's
pub coercion and broadcasting (estimator_v2.py:112-160)."""
import ctypes as C

import numpy as np
import pytest

from _pkg import pkg


def test_parameter_expressions():
    P = pkg()
    a, b = P.Parameter("a"), P.Parameter("b")
    e = 2 * a - b / 2 + 1.0
    assert e.parameters == {a, b}
    assert e.bind({a: 1.0, b: 2.0}) == 2.0
    np.testing.assert_allclose(e.evaluate({a: np.array([1.0, 2.0]), b: np.array([2.0, 0.0])}), [2.0, 5.0])
    partial = e.bind({a: 0.5})
    assert isinstance(partial, P.ParameterExpression) and partial.parameters == {b}
    assert (a - a).bind({}) == 0.0
    assert float(-(a * 0) + 3) == 3.0
    with pytest.raises(TypeError):
        a * b
    with pytest.raises(TypeError):
        float(a)


def test_circuit_parameters_sorted_and_assigned():
    P = pkg()
    b, a = P.Parameter("b"), P.Parameter("a")
    qc = P.QuantumCircuit(2).ry(b, 0).rz(a + 1, 1).cx(0, 1).rx(0.5, 0)
    assert [p.name for p in qc.parameters] == ["a", "b"]
    bound = qc.assign_parameters([0.25, -1.0])
    assert bound.parameters == []
    assert bound.data[0].params == [-1.0] and bound.data[1].params == [1.25]
    assert qc.parameters  # the original keeps its parameters
    with pytest.raises(ValueError):
        qc.assign_parameters([1.0])


def test_bind_table_and_reference_errors():
    P = pkg()
    A = P._capi
    a = P.Parameter("a")
    qc = P.QuantumCircuit(3).h(0).ry(a, 1).u(a, 0.2, 2 * a, 2)
    nc = P.NativeCircuit(3, qc.data)
    assert [(i, pos) for i, pos, _ in nc.param_slots] == [(1, 0), (2, 0), (2, 2)]
    nc.bind({a: np.array([0.1, 0.2, 0.3])}, 3)
    n = C.c_int()
    A.check(P.lib().gbqv_circuit_num_bindings(nc.handle, C.byref(n)))
    assert n.value == 3
    v = np.zeros(3)
    with pytest.raises(P.GBQVError, match="instruction position out of range"):
        A.check(P.lib().gbqv_circuit_bind_param(nc.handle, 9, 0, 3, v.ctypes.data_as(A.dp)))
    with pytest.raises(P.GBQVError, match="param position out of range"):
        A.check(P.lib().gbqv_circuit_bind_param(nc.handle, 1, 1, 3, v.ctypes.data_as(A.dp)))
    with pytest.raises(P.GBQVError, match="same number of values"):
        A.check(P.lib().gbqv_circuit_bind_param(nc.handle, 1, 0, 2, v.ctypes.data_as(A.dp)))
    with pytest.raises(P.GBQVError, match="only gate parameters"):
        nc2 = P.NativeCircuit(2, P.QuantumCircuit(2).unitary(np.eye(2), [0]).data)
        A.check(P.lib().gbqv_circuit_bind_param(nc2.handle, 0, 0, 3, v.ctypes.data_as(A.dp)))


def test_fusion_keeps_bound_gates():
    P = pkg()
    a = P.Parameter("a")
    qc = P.QuantumCircuit(4)
    for layer in range(3):
        for q in range(4):
            qc.ry(a * (q + 1), q)
        for q in range(3):
            qc.cx(q, q + 1)
    nc = P.NativeCircuit(4, qc.data)
    nc.bind({a: np.linspace(0, 1, 5)}, 5)
    sim = P.AerSimulator(fusion_threshold=1)
    nc.fuse(sim.fusion_config())
    names = [name for _, name, _ in nc.ops()]
    assert names.count("ry") == 12  # every bound gate survives as itself


def test_run_binds_validation():
    P = pkg()
    a = P.Parameter("a")
    qc = P.QuantumCircuit(1).rx(a, 0)
    check = P.AerSimulator._check_binds
    with pytest.raises(ValueError, match="parameter_binds is not specified"):
        check([qc], None, True)
    with pytest.raises(ValueError, match="More than 1 parameter table"):
        check([qc], [{a: [1]}, {a: [2]}], True)
    with pytest.raises(ValueError, match="does not match"):
        check([qc, qc], [{a: [1]}], False)
    with pytest.raises(ValueError, match="same number of values"):
        b = P.Parameter("b")
        check([P.QuantumCircuit(1).rx(a, 0).ry(b, 0)], [{a: [1, 2], b: [1]}], True)
    out = check([qc, P.QuantumCircuit(1).h(0)], [{a: [1, 2, 3]}, {}], False)
    assert out[1] == {} and list(out[0][a]) == [1, 2, 3]


def test_estimator_pub_coercion_and_broadcast_shapes():
    P = pkg()
    import importlib
    pr = importlib.import_module(P.__name__ + ".primitives")
    a, b = P.Parameter("a"), P.Parameter("b")
    qc = P.QuantumCircuit(2).ry(a, 0).rz(b, 1)
    obs = pr.coerce_observables(["XZ", {"ZZ": 0.5, "XI": 1.0}, [("YY", 2.0), ("YY", 1.0)]], 2)
    assert obs.shape == (3,) and obs[2] == {"YY": 3.0}
    assert pr.coerce_observables([["ZZ"], ["XX"]], 2).shape == (2, 1)
    with pytest.raises(ValueError):
        pr.coerce_observables("ZZZ", 2)
    pv = pr.coerce_parameter_values({(a, b): np.zeros((4, 2))}, qc)
    assert pv.shape == (4, 2)
    pv = pr.coerce_parameter_values({a: [1.0, 2.0], b: 0.5}, qc)
    np.testing.assert_array_equal(pv, [[1.0, 0.5], [2.0, 0.5]])
    with pytest.raises(ValueError):
        pr.coerce_parameter_values(np.zeros((3, 3)), qc)
    with pytest.raises(ValueError):
        pr.coerce_parameter_values(None, qc)


def test_unitary_method_host_rules():
    """The unitary method halves the fusion threshold
    (Executor::transpile_fusion, circuit_executor.hpp:1259-1262) and accepts
    only its op set (unitary_state.hpp:35-54)."""
    P = pkg()
    sv = P.AerSimulator().fusion_config()
    un = P.AerSimulator(method="unitary").fusion_config()
    assert (sv.threshold, un.threshold, un.max_qubit) == (14, 7, 5)
    sim = P.AerSimulator(method="unitary")
    sim._check_unitary_circuit(P.QuantumCircuit(2).h(0).cx(0, 1).unitary(np.eye(2), [1]).save_unitary())
    for bad in (P.QuantumCircuit(2).measure(0, 0), P.QuantumCircuit(2).reset(0),
                P.QuantumCircuit(2).h(0).save_statevector()):
        with pytest.raises(ValueError, match="invalid instruction"):
            sim._check_unitary_circuit(bad)


def test_bit_array_packing_and_counts():
    P = pkg()
    import importlib
    pr = importlib.import_module(P.__name__ + ".primitives")
    vals = np.array([[0b1011, 0b0001, 0b1011], [0x1FF, 0, 1]], dtype=np.uint64)
    b = pr.BitArray(vals, 9)
    assert b.shape == (2,) and b.num_shots == 3
    np.testing.assert_array_equal(b.array[0, 0], [0x00, 0x0B])      # big-endian bytes
    np.testing.assert_array_equal(b.array[1, 0], [0x01, 0xFF])
    assert b.get_counts(0) == {"000001011": 2, "000000001": 1}
    assert b.get_bitstrings(1) == ["111111111", "000000000", "000000001"]
    assert sum(b.get_int_counts().values()) == 6
