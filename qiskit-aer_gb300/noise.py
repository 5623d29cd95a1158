"""Noise channels as superoperators, in the vec(rho) layout the engine uses.

``depolarizing_error`` and ``amplitude_damping_error`` follow
qiskit_aer/noise/errors/standard_errors.py:170-219 and 351-462; a
``QuantumError`` is carried as its superoperator S (4^k x 4^k,
S = sum conj(K) (x) K over its Kraus / Pauli terms), which is how the
reference applies errors under the density-matrix method
(src/noise/quantum_error.hpp:177-183, 493-509).  ``NoiseModel`` inserts the
error after every gate of the listed names, as
``NoiseModel::sample_noise(..., Method::superop)`` does
(src/noise/noise_model.hpp:274, 434-450).
"""
from __future__ import annotations

import itertools

import numpy as np

_P = {
    "I": np.eye(2, dtype=complex),
    "X": np.array([[0, 1], [1, 0]], dtype=complex),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=complex),
    "Z": np.array([[1, 0], [0, -1]], dtype=complex),
}


def _kron_all(mats):
    out = np.array([[1.0 + 0j]])
    for m in mats:
        out = np.kron(out, m)
    return out


def kraus_superop(kraus) -> np.ndarray:
    """sum_i conj(K_i) (x) K_i (Utils::kraus_superop)."""
    return sum(np.kron(np.conj(k), k) for k in kraus)


class QuantumError:
    """A k-qubit channel held as its superoperator (column-major meaning:
    vec(rho') = S vec(rho), vec index = row + 2^k col)."""

    def __init__(self, superop: np.ndarray, num_qubits: int):
        self.superop = np.asarray(superop, dtype=complex)
        self.num_qubits = num_qubits

    @classmethod
    def from_kraus(cls, kraus):
        k = int(np.log2(np.asarray(kraus[0]).shape[0]))
        return cls(kraus_superop(kraus), k)

    def compose(self, other: "QuantumError") -> "QuantumError":
        """self then other (qiskit QuantumError.compose semantics)."""
        return QuantumError(other.superop @ self.superop, self.num_qubits)

    def tensor(self, other: "QuantumError") -> "QuantumError":
        """self (x) other with `other` on the lower qubit (qiskit ordering):
        the result acts on [q_other..., q_self...]."""
        ka, kb = other.num_qubits, self.num_qubits
        da, db = 1 << ka, 1 << kb
        D = da * db
        # S[v_out, v_in] with v = r + d*c; reshape gives [c_out, r_out, c_in, r_in]
        sa = other.superop.reshape(da, da, da, da)
        sb = self.superop.reshape(db, db, db, db)
        # combined v = ra + da*rb + D*(ca + da*cb): axis order (cb, ca, rb, ra)
        out = np.einsum("pqrs,tuvw->tpuqvrws", sa, sb).reshape(D * D, D * D)
        return QuantumError(out, ka + kb)

    def to_instruction_args(self):
        return self.superop


def depolarizing_error(param: float, num_qubits: int) -> QuantumError:
    terms = 4 ** num_qubits
    max_param = terms / (terms - 1)
    if param < 0 or param > max_param:
        raise ValueError(f"Depolarizing parameter must be in between 0 and {max_param}.")
    probs = [1 - param / max_param] + (terms - 1) * [param / terms]
    sup = 0
    for p, labels in zip(probs, itertools.product("IXYZ", repeat=num_qubits)):
        m = _kron_all([_P[c] for c in labels])
        sup = sup + p * np.kron(m.conj(), m)
    return QuantumError(sup, num_qubits)


def amplitude_damping_error(param_amp: float, excited_state_population: float = 0.0) -> QuantumError:
    return phase_amplitude_damping_error(param_amp, 0.0, excited_state_population)


def phase_amplitude_damping_error(param_amp, param_phase, excited_state_population=0.0) -> QuantumError:
    if param_amp < 0 or param_phase < 0 or param_amp + param_phase > 1:
        raise ValueError("Invalid amplitude and phase damping parameters")
    c0 = np.sqrt(1 - excited_state_population)
    c1 = np.sqrt(excited_state_population)
    par = 1 - param_amp - param_phase
    ops = [
        c0 * np.array([[1, 0], [0, np.sqrt(par)]], dtype=complex),
        c0 * np.array([[0, np.sqrt(param_amp)], [0, 0]], dtype=complex),
        c0 * np.array([[0, 0], [0, np.sqrt(param_phase)]], dtype=complex),
        c1 * np.array([[np.sqrt(par), 0], [0, 1]], dtype=complex),
        c1 * np.array([[0, 0], [np.sqrt(param_amp), 0]], dtype=complex),
        c1 * np.array([[np.sqrt(param_phase), 0], [0, 0]], dtype=complex),
    ]
    ops = [k for k in ops if np.linalg.norm(k) > 1e-10]
    return QuantumError.from_kraus(ops)


class NoiseModel:
    def __init__(self):
        self._all_qubit = {}   # gate name -> QuantumError

    def add_all_qubit_quantum_error(self, error: QuantumError, instructions):
        for name in ([instructions] if isinstance(instructions, str) else instructions):
            self._all_qubit[name] = error

    def error_for(self, name: str):
        return self._all_qubit.get(name)

    def is_ideal(self) -> bool:
        return not self._all_qubit
