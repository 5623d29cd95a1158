"""Runtime parameter binding on the GPU against the oracle: a parameterised
circuit with B bindings runs once on a stack of B states
(gbqv_execute_bound, the reference's batched parameter-bind execution,
batch_shots_executor.hpp:152-314), and every binding's final statevector and
Pauli expectation values equal the oracle applying that binding's gates one
by one (QubitVector arithmetic): complex128 to 1e-12, complex64 to the
engine's single-precision tolerance.  Also: chunked stacks (bindings split
over several launches), zero padding states, the per-binding loop used for
circuits with measurements, and EstimatorV2 broadcasting."""
import ctypes

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu

PARAM_GATES = [("rx", 1, 1), ("ry", 1, 1), ("rz", 1, 1), ("p", 1, 1), ("u", 1, 3), ("r", 1, 2),
               ("rxx", 2, 1), ("ryy", 2, 1), ("rzz", 2, 1), ("rzx", 2, 1), ("cp", 2, 1), ("crx", 2, 1),
               ("cry", 2, 1), ("crz", 2, 1)]
FIXED_GATES = [("h", 1), ("x", 1), ("y", 1), ("s", 1), ("t", 1), ("sx", 1), ("cx", 2), ("cz", 2), ("cy", 2),
               ("swap", 2), ("ccx", 3)]


def haar(rng, d):
    z = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def oracle_gate(o, name, q, p):
    """Statevector::State::apply_gate (statevector_state.hpp:733-865) on the oracle."""
    rot = {"rx": 0, "ry": 1, "rz": 2, "crx": 0, "cry": 1, "crz": 2}
    if name in rot:
        o.apply_mcu(q, O.rotation_matrix(rot[name], p[0]))
    elif name in ("p", "cp"):
        o.apply_mcphase(q, np.exp(1j * p[0]))
    elif name == "u":
        o.apply_mcu(q, O.u4(p[0], p[1], p[2], 0.0))
    elif name == "r":
        th, ph = p
        c, s = np.cos(th / 2), np.sin(th / 2)
        o.apply_mcu(q, np.array([[c, -1j * np.exp(-1j * ph) * s], [-1j * np.exp(1j * ph) * s, c]]))
    elif name in ("rxx", "ryy", "rzx"):
        o.apply_matrix(q, O.rotation_matrix({"rxx": 3, "ryy": 4, "rzx": 6}[name], p[0]))
    elif name == "rzz":
        o.apply_diagonal_matrix(q, O.rzz_diag(p[0]))
    elif name == "h":
        o.apply_mcu(q, O.u4(np.pi / 2, 0.0, np.pi, 0.0))
    elif name in ("x", "cx", "ccx"):
        o.apply_mcx(q)
    elif name in ("y", "cy"):
        o.apply_mcy(q)
    elif name == "s":
        o.apply_diagonal_matrix(q, [1, 1j])
    elif name == "t":
        o.apply_diagonal_matrix(q, [1, np.exp(0.25j * np.pi)])
    elif name == "sx":
        o.apply_matrix(q, 0.5 * np.array([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]))
    elif name == "cz":
        o.apply_mcphase(q, -1.0)
    elif name == "swap":
        o.apply_mcswap(q)
    else:
        raise KeyError(name)


def random_bound_circuit(P, n, ngates, nparams, rng):
    params = [P.Parameter(f"t{i}") for i in range(nparams)]
    qc = P.QuantumCircuit(n)
    for _ in range(ngates):
        r = rng.random()
        if r < 0.55:
            name, k, npar = PARAM_GATES[rng.integers(len(PARAM_GATES))]
            if k > n:
                continue
            ps = []
            for _ in range(npar):
                a = params[rng.integers(nparams)]
                ps.append(a if rng.random() < 0.5 else 1.5 * a - 0.25)
            q = [int(x) for x in rng.choice(n, k, replace=False)]
            qc.append_gate(name, q, ps)
        elif r < 0.9:
            name, k = FIXED_GATES[rng.integers(len(FIXED_GATES))]
            if k > n:
                continue
            qc.append_gate(name, [int(x) for x in rng.choice(n, k, replace=False)])
        else:
            k = min(n, int(rng.integers(1, 4)))
            qc.unitary(haar(rng, 1 << k), [int(x) for x in rng.choice(n, k, replace=False)])
    return qc, params


def oracle_binding(qc, values: dict):
    o = O.OracleQV(qc.num_qubits)
    for ins in qc.data:
        if ins.kind == "unitary":
            o.apply_matrix(ins.qubits, ins.data)
        elif ins.kind == "gate":
            p = [x.bind(values) if hasattr(x, "bind") else x for x in ins.params]
            oracle_gate(o, ins.name, ins.qubits, [float(x) for x in p])
    return o


def pauli_terms(rng, n, count):
    out = []
    for _ in range(count):
        k = int(rng.integers(1, min(n, 4) + 1))
        q = [int(x) for x in rng.choice(n, k, replace=False)]
        out.append((float(rng.normal()), "".join(rng.choice(list("IXYZ"), k)), q))
    return out


@pytest.mark.parametrize("n,nbind", [(1, 3), (3, 5), (7, 17), (13, 2), (15, 9)])
@pytest.mark.parametrize("precision", ["double", "single"])
def test_bound_circuit_matches_oracle_per_binding(n, nbind, precision):
    P = pkg()
    rng = np.random.default_rng(100 * n + nbind)
    qc, params = random_bound_circuit(P, n, 60, 5, rng)
    terms = pauli_terms(rng, n, 12)
    qc.save_statevector()
    qc.save_expectation_value(terms, label="H")
    values = {p: rng.uniform(-np.pi, np.pi, nbind) for p in params}
    binds = {p: v for p, v in values.items() if p in qc.parameters}
    res = P.AerSimulator(precision=precision).run(qc, parameter_binds=[binds], seed_simulator=3)
    assert len(res.results) == nbind
    assert res.metadata(0)["parameter_binding"]["batched"]
    tol = 1e-12 if precision == "double" else 3e-6 * 60
    for j in range(nbind):
        o = oracle_binding(qc, {p: v[j] for p, v in binds.items()})
        np.testing.assert_allclose(res.get_statevector(j), o.data, rtol=0, atol=tol)
        want = sum(c * o.expval_pauli(q, lab) for c, lab, q in terms)
        assert abs(res.data(j)["H"] - want) < tol * 10
        assert res.results[j]["seed_simulator"] == 3 + 2113 * j


def test_chunked_stack_and_seeds_match_one_stack():
    P = pkg()
    rng = np.random.default_rng(8)
    n, nbind = 9, 11
    qc, params = random_bound_circuit(P, n, 40, 3, rng)
    terms = pauli_terms(rng, n, 6)
    qc.save_expectation_value(terms, label="E")
    binds = {p: rng.uniform(-3, 3, nbind) for p in qc.parameters}
    whole = P.AerSimulator().run(qc, parameter_binds=[binds], seed_simulator=1)
    sim = P.AerSimulator()
    sim.MAX_STACK_QUBITS = n + 2  # 4 bindings per stack: chunks of 4, 4, 3
    parts = sim.run(qc, parameter_binds=[binds], seed_simulator=1)
    for j in range(nbind):
        assert abs(whole.data(j)["E"] - parts.data(j)["E"]) < 1e-13
        o = oracle_binding(qc, {p: v[j] for p, v in binds.items()})
        assert abs(parts.data(j)["E"] - sum(c * o.expval_pauli(q, lab) for c, lab, q in terms)) < 1e-11


def test_padding_states_stay_zero_and_binding_offset():
    P = pkg()
    n = 4
    a = P.Parameter("a")
    qc = P.QuantumCircuit(n).h(0).ry(a, 1).cx(1, 2).rz(2 * a, 3)
    vals = np.array([0.1, 0.7, -1.2, 2.5, 0.4])
    nc = P.NativeCircuit(n, qc.data)
    nc.bind({a: vals}, len(vals))
    with P.QubitVector(n + 2) as st:
        P._capi.check(P.lib().gbqv_execute_bound(st.handle, nc.handle, 2, 3), st.handle)
        stack = st.copy_to_vector()
    assert np.all(stack[3 << n:] == 0)
    for j in range(3):
        o = oracle_binding(qc, {a: vals[2 + j]})
        np.testing.assert_allclose(stack[j << n:(j + 1) << n], o.data, atol=1e-13)


@pytest.mark.parametrize("n", [3, 12])
def test_measured_bound_circuit_samples_each_state_as_its_own(n):
    """Shots of a bound circuit come from each binding's own state of the
    stack with its own seed: counts and per-shot memory equal the circuit
    bound and run alone."""
    P = pkg()
    a, b = P.Parameter("a"), P.Parameter("b")
    qc = P.QuantumCircuit(n).ry(a, 0).cx(0, 1).rx(b, n - 1)
    for q in range(2, n, 3):
        qc.h(q)
    qc.measure_all()
    binds = {a: [0.3, 1.9, -2.2], b: [2.2, -0.4, 0.9]}
    res = P.AerSimulator().run(qc, shots=500, parameter_binds=[binds], seed_simulator=21, memory=True)
    assert res.metadata(0)["parameter_binding"]["batched"]
    for j in range(3):
        one = P.AerSimulator().run(qc.assign_parameters({a: binds[a][j], b: binds[b][j]}), shots=500,
                                   seed_simulator=21 + 2113 * j, memory=True)
        assert res.get_counts(j) == one.get_counts()
        assert res.get_memory(j) == one.get_memory()
        assert len(res.get_memory(j)) == 500


def test_sampler_v2_shapes_and_counts():
    P = pkg()
    a = P.Parameter("a")
    qc = P.QuantumCircuit(2).ry(a, 0).cx(0, 1).measure_all()
    vals = np.linspace(0.2, 2.8, 6).reshape(2, 3, 1)
    res = P.SamplerV2(seed=7).run([(qc, vals), (P.QuantumCircuit(1).h(0).measure_all(),)], shots=300).result()
    bits = res[0].data.meas
    assert bits.shape == (2, 3) and bits.num_shots == 300 and bits.num_bits == 2
    assert bits.array.shape == (2, 3, 300, 1)
    for k, idx in enumerate(np.ndindex(2, 3)):
        want = P.AerSimulator().run(qc.assign_parameters([vals[idx][0]]), shots=300,
                                    seed_simulator=7 + 2113 * k).get_counts()
        assert bits.get_counts(idx) == want
        assert set(bits.get_counts(idx)) <= {"00", "11"}
    assert sum(res[1].data.meas.get_counts().values()) == 300


def test_unbound_parameters_are_an_error():
    P = pkg()
    a = P.Parameter("a")
    qc = P.QuantumCircuit(2).rx(a, 0)
    with pytest.raises(ValueError, match="parameter_binds is not specified"):
        P.AerSimulator().run(qc)


@pytest.mark.parametrize("precision", ["double", "single"])
def test_estimator_v2_broadcasting_against_oracle(precision):
    P = pkg()
    rng = np.random.default_rng(77)
    n = 6
    qc, _ = random_bound_circuit(P, n, 50, 3, rng)
    params = qc.parameters
    values = rng.uniform(-np.pi, np.pi, size=(3, 1, len(params)))
    labels = ["".join(rng.choice(list("IXYZ"), n)) for _ in range(4)]
    # shape (4,): a dict, a label, a (label, coeff) list, a label
    observables = [{labels[0]: 0.5, labels[1]: -1.25}, labels[2], [(labels[3], 2.0), (labels[0], 1.0)], labels[1]]
    est = P.EstimatorV2(options={"backend_options": {"precision": precision}})
    res = est.run([(qc, observables, values)]).result()
    evs = res[0].data.evs
    assert evs.shape == (3, 4)
    assert np.all(res[0].data.stds == 0.0)
    tol = 1e-11 if precision == "double" else 2e-4
    for i in range(3):
        o = oracle_binding(qc, dict(zip(params, values[i, 0])))
        ev = lambda lab: o.expval_pauli(list(range(n)), lab)
        want = [0.5 * ev(labels[0]) - 1.25 * ev(labels[1]), ev(labels[2]), 2.0 * ev(labels[3]) + ev(labels[0]),
                ev(labels[1])]
        np.testing.assert_allclose(evs[i], want, atol=tol)


def test_estimator_v2_precision_and_no_parameters():
    P = pkg()
    qc = P.QuantumCircuit(2).h(0).cx(0, 1)
    est = P.EstimatorV2(options={"run_options": {"seed_simulator": 5}})
    exact = est.run([(qc, ["ZZ", "XX", "ZI"])]).result()[0].data.evs
    np.testing.assert_allclose(exact, [1.0, 1.0, 0.0], atol=1e-14)
    noisy = est.run([(qc, ["ZZ", "XX", "ZI"])], precision=0.1).result()[0]
    assert np.all(noisy.data.stds == 0.1)
    again = est.run([(qc, ["ZZ", "XX", "ZI"])], precision=0.1).result()[0]
    np.testing.assert_array_equal(noisy.data.evs, again.data.evs)
    assert not np.allclose(noisy.data.evs, exact)
    with pytest.raises(ValueError, match="precision less than 0"):
        est.run([(qc, "ZZ", None, -1.0)])


@pytest.mark.parametrize("precision,tol", [("double", 1e-12), ("single", 2e-6)])
def test_stacked_expvals_against_oracle(precision, tol):
    """expval_pauli_segments on a stack of 8 random 16-qubit states (the
    EstimatorV2 reduction: complex64 sums in float with compensation, one
    conversion per thread) against the oracle's expval_pauli per state, for
    Z-only terms and terms with X/Y on low and high qubits."""
    P = pkg()
    n, nseg = 16, 8
    rng = np.random.default_rng(61)
    states = []
    for _ in range(nseg):
        v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
        states.append(v / np.linalg.norm(v))
    st = P.QubitVector(n + 3, precision)
    st.initialize_from_vector(np.concatenate(states))
    labels = ["Z" * n, "I" * (n - 1) + "X", "Y" + "I" * (n - 1), "XZ" + "I" * (n - 4) + "YZ",
              "I" * 5 + "ZZ" + "I" * (n - 8) + "X", "Y" * n, "I" * (n - 3) + "XXX", "Z" + "I" * (n - 2) + "Z"]
    terms = [(list(range(n)), lab) for lab in labels]
    got = st.expval_pauli_segments(n, nseg, terms)
    for j, v in enumerate(states):
        o = O.OracleQV(n, v.astype(np.complex64) if precision == "single" else v)
        for t, lab in enumerate(labels):
            assert abs(got[t, j] - o.expval_pauli(list(range(n)), lab)) < tol, (lab, j)


@pytest.mark.parametrize("precision,tol", [("double", 1e-13), ("single", 2e-6)])
def test_specialised_runs_match_interpreting_runs(precision, tol):
    """Bound runs compiled for their op sequence (runtime_compile=2) give the
    interpreting kernel's states (runtime_compile=0) and the oracle's, for a
    circuit of every gate kind over 9 bindings of a 15-qubit state (runs of
    the register-tile kernel with register, lane and thread bits); a repeat
    with the default tiering (1) compiles on the second execution."""
    P = pkg()
    rng = np.random.default_rng(812)
    n, nbind = 15, 9
    qc, params = random_bound_circuit(P, n, 80, 6, rng)
    qc.save_statevector()
    values = {p: rng.uniform(-np.pi, np.pi, nbind) for p in params}
    binds = [{p: v for p, v in values.items() if p in qc.parameters}]
    L = P.lib()

    def launched():
        compiled, launches = ctypes.c_uint64(), ctypes.c_uint64()
        P._capi.check(L.gbqv_run_jit_counts(ctypes.byref(compiled), ctypes.byref(launches)))
        return launches.value

    res, used = {}, {}
    for mode in (0, 2, 1):
        sim = P.AerSimulator(precision=precision, runtime_compile=mode)
        before = launched()
        for _ in range(2 if mode == 1 else 1):
            res[mode] = sim.run(qc, parameter_binds=binds, seed_simulator=5)
        used[mode] = launched() - before
    assert used[0] == 0 and used[2] > 0 and used[1] > 0, used
    for j in range(nbind):
        a, b, c = (np.asarray(res[m].get_statevector(j)) for m in (0, 2, 1))
        assert np.max(np.abs(a - b)) <= tol
        assert np.max(np.abs(a - c)) <= tol
        o = oracle_binding(qc, {p: v[j] for p, v in binds[0].items()})
        np.testing.assert_allclose(b, o.data, rtol=0, atol=1e-12 if precision == "double" else 3e-6 * 80)
