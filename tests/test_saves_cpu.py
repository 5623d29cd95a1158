"""Save instructions' host logic without a GPU: the reference's
expectation-value parameters (_expval_params, save_expectation_value.py:
139-168, including O.O for the variance), Base::apply_save_expval
(state.hpp:416-447) and the amplitude / ket-dict saves, evaluated through
AerSimulator._save on a CPU stand-in for the state (the oracle)."""
import itertools

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

PM = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]), "Y": np.array([[0, -1j], [1j, 0]]), "Z": np.diag([1, -1])}


def full_matrix(n, label, qubits):
    ops = [PM["I"]] * n
    for j, q in enumerate(qubits):
        ops[n - 1 - q] = PM[label[len(label) - 1 - j]]
    out = np.array([[1.0 + 0j]])
    for m in ops:
        out = np.kron(out, m)
    return out


class OracleState:
    """The methods _save calls, on the oracle's statevector."""

    def __init__(self, vec):
        self.o = O.OracleQV(int(np.log2(vec.size)), vec)

    def expval_pauli_many(self, pairs, coeffs=None):
        vals = np.array([self.o.expval_pauli(q, lab) for q, lab in pairs])
        return vals, float(vals.sum())

    def copy_to_vector(self):
        return self.o.data.copy()

    def probabilities(self, qubits=()):
        return self.o.probabilities(list(qubits))


def random_terms(rng, n, count):
    terms = []
    for _ in range(count):
        k = int(rng.integers(1, 4))
        q = [int(x) for x in rng.choice(n, k, replace=False)]
        terms.append((float(rng.normal()), "".join(rng.choice(list("IXYZ"), k)), q))
    return terms


def test_expval_params_match_matrix_algebra():
    P = pkg()
    rng = np.random.default_rng(3)
    n = 3
    terms = random_terms(rng, n, 6) + [(0.5 + 0.25j, "XY", [0, 2]), (0.5 - 0.25j, "YX", [2, 0])]
    params = P.circuit.expval_params(terms, variance=True)
    Om = sum(complex(c).real * full_matrix(n, lab, q) for c, lab, q in terms)
    O2 = sum(complex(ca) * complex(cb) * full_matrix(n, la, qa) @ full_matrix(n, lb, qb)
             for ca, la, qa in terms for cb, lb, qb in terms)
    got1 = sum(c1 * full_matrix(n, lab, q) for (q, lab), c1, _ in params)
    got2 = sum(c2 * full_matrix(n, lab, q) for (q, lab), _, c2 in params)
    np.testing.assert_allclose(got1, Om, atol=1e-12)
    np.testing.assert_allclose(got2, _real_part_decomp(O2, n), atol=1e-12)
    keys = [tuple(q) + (lab,) for (q, lab), _, _ in params]
    assert len(keys) == len(set(keys))                      # one entry per distinct Pauli


def _real_part_decomp(M, n):
    """sum_P Re(tr(P M) / 2^n) P: the real parts of M's Pauli coefficients."""
    out = np.zeros_like(M)
    for labs in itertools.product("IXYZ", repeat=n):
        lab = "".join(labs)
        Pm = full_matrix(n, lab, list(range(n)))
        out = out + (np.trace(Pm @ M) / 2 ** n).real * Pm
    return out


def test_save_expval_variance_amplitudes_and_dicts():
    P = pkg()
    rng = np.random.default_rng(9)
    n = 4
    vec = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    vec /= np.linalg.norm(vec)
    vec[3] = 1e-9                                           # chopped out of the dicts
    vec /= np.linalg.norm(vec)
    st = OracleState(vec)
    sim = P.AerSimulator()
    terms = random_terms(rng, n, 5)
    qc = (P.QuantumCircuit(n).save_expectation_value(terms, "E").save_expectation_value_variance(terms, "V")
          .save_amplitudes([0, 5, 9], "A").save_amplitudes_squared([5, 3], "A2")
          .save_probabilities_dict([2, 0], "PD").save_statevector_dict("SD"))
    data = {}
    for ins in qc.data:
        sim._save(st, ins, data)
    Om = sum(c * full_matrix(n, lab, q) for c, lab, q in terms)
    mean = float(np.real(vec.conj() @ Om @ vec))
    var = float(np.real(vec.conj() @ Om @ Om @ vec)) - mean * mean
    assert abs(data["E"] - mean) < 1e-12
    assert abs(data["V"][0] - mean) < 1e-12 and abs(data["V"][1] - var) < 1e-12
    np.testing.assert_array_equal(data["A"], vec[[0, 5, 9]])
    np.testing.assert_allclose(data["A2"], np.abs(vec[[5, 3]]) ** 2, atol=1e-15)
    probs = st.probabilities([2, 0])
    assert data["PD"] == {hex(k): probs[k] for k in range(4)}
    assert "0x3" not in data["SD"] and data["SD"]["0x0"] == vec[0]
    assert len(data["SD"]) == (1 << n) - 1
    with pytest.raises(ValueError, match="empty"):
        sim._save(st, P.QuantumCircuit(n).save_amplitudes([]).data[0], {})


def test_ket_dict_chops_parts():
    P = pkg()
    d = P.simulator.ket_dict(np.array([1e-9 + 0.5j, 0.0, 1e-9, 0.3 + 1e-12j]), 1e-8)
    assert d == {"0x0": 0.5j, "0x3": 0.3 + 0j}
