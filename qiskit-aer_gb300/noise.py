"""Noise channels as superoperators, in the vec(rho) layout the engine uses.

The standard errors follow qiskit_aer/noise/errors/standard_errors.py
(kraus_error :32, mixed_unitary_error :59, coherent_unitary_error :110,
pauli_error :123, depolarizing_error :170-219, reset_error :222,
thermal_relaxation_error :257, phase_amplitude_damping_error /
amplitude_damping_error / phase_damping_error :351-520); a ``QuantumError``
is carried as its superoperator S (4^k x 4^k, S = sum conj(K) (x) K over its
Kraus / Pauli / unitary terms), which is how the reference applies errors
under the density-matrix method (src/noise/quantum_error.hpp:177-183,
493-509).  ``NoiseModel`` inserts the error after every gate of the listed
names, as ``NoiseModel::sample_noise(..., Method::superop)`` does
(src/noise/noise_model.hpp:274, 434-450): an error given for the gate's
exact qubits (``add_quantum_error``) in place of the all-qubit one
(``NoiseModel::sample_local_quantum_noise``, noise_model.hpp:710-780);
errors added twice for the same key are composed (noise_model.py:669-806).
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


ATOL = 1e-8  # the reference's QuantumError tolerance (TolerancesMixin)


class QuantumError:
    """A k-qubit channel held as its superoperator (column-major meaning:
    vec(rho') = S vec(rho), vec index = row + 2^k col)."""

    def __init__(self, superop: np.ndarray, num_qubits: int):
        self.superop = np.asarray(superop, dtype=complex)
        self.num_qubits = num_qubits

    def ideal(self) -> bool:
        """The identity channel (a global phase included), which a noise
        model does not add (noise_model.py:669-700)."""
        return bool(np.max(np.abs(self.superop - np.eye(self.superop.shape[0]))) <= 1e-12)

    def expand(self, other: "QuantumError") -> "QuantumError":
        """other (x) self, with self on the lower qubits (QuantumError.expand)."""
        return other.tensor(self)

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

    def kraus(self) -> list:
        """The channel's canonical Kraus operators (QuantumError::kraus,
        src/noise/quantum_error.hpp:405-430), computed once."""
        if getattr(self, "_kraus", None) is None:
            self._kraus = superop_kraus(self.superop, self.num_qubits)
        return self._kraus


def superop_kraus(superop: np.ndarray, num_qubits: int, threshold: float = 1e-10) -> list:
    """Canonical Kraus operators of a superoperator (Utils::superop2kraus,
    src/framework/noise_utils.hpp:33-87): the Choi matrix
    C = sum vec(K) vec(K)^dag (vec column-major) rearranged from S =
    sum conj(K) (x) K, its eigenvectors largest eigenvalue first, and
    K = sqrt(lambda) unvec(v) for every eigenvalue above the threshold."""
    d = 1 << num_qubits
    s4 = np.asarray(superop, dtype=complex).reshape(d, d, d, d)  # [c', r, c'', r'']: conj(K)[c', c''] K[r, r'']
    choi = np.einsum("ebca->abce", s4).reshape(d * d, d * d)
    choi = 0.5 * (choi + choi.conj().T)
    w, v = np.linalg.eigh(choi)
    keep = [idx for idx in range(d * d - 1, -1, -1) if w[idx] > threshold]
    # Within an eigenspace of equal eigenvalues any orthonormal basis gives
    # canonical operators (the eigensolver returns one of them); where Pauli
    # matrices span the eigenspace they are taken, so that a Pauli channel's
    # operators are its Paulis, each a multiple of a unitary.
    pv = _pauli_vectors(num_qubits)
    start = 0
    while start < len(keep):
        end = start + 1
        while end < len(keep) and w[keep[start]] - w[keep[end]] <= 1e-12:
            end += 1
        if end - start > 1:
            cols = keep[start:end]
            weight = np.sum(np.abs(v[:, cols].conj().T @ pv) ** 2, axis=0)
            sel = np.nonzero(weight > 1 - 1e-9)[0]
            if sel.size == len(cols):
                v[:, cols] = pv[:, sel]
        start = end
    return [np.sqrt(w[idx]) * v[:, idx].reshape((d, d), order="F") for idx in keep]


def _pauli_vectors(num_qubits: int) -> np.ndarray:
    """Columns: vec (column-major) of every num_qubits-qubit Pauli matrix
    divided by sqrt(2^num_qubits), orthonormal."""
    one = [np.eye(2), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.diag([1.0, -1.0])]
    mats = [np.eye(1, dtype=complex)]
    for _ in range(num_qubits):
        mats = [np.kron(p, m) for p in one for m in mats]
    return np.stack([m.reshape(-1, order="F") for m in mats], axis=1) / np.sqrt(1 << num_qubits)


def _check_probs(probs) -> None:
    probs = [float(p) for p in probs]
    if any(p < -ATOL for p in probs):
        raise ValueError("Probabilities are invalid.")
    if not np.isclose(sum(probs) - 1, 0, atol=ATOL):
        raise ValueError(f"Probabilities are not normalized: {sum(probs)} != 1")


def _as_square(m) -> tuple[np.ndarray, int]:
    m = np.asarray(m, dtype=complex)
    k = int(round(np.log2(m.shape[0]))) if m.ndim == 2 and m.shape[0] else -1
    if m.ndim != 2 or m.shape[0] != m.shape[1] or k < 1 or m.shape[0] != 1 << k:
        raise ValueError("A matrix in the error is not a square matrix of qubits.")
    return m, k


def kraus_error(noise_ops, canonical_kraus: bool = False) -> QuantumError:
    """A channel from Kraus matrices (trace preserving within ATOL)."""
    if not isinstance(noise_ops, (list, tuple)) or not noise_ops:
        raise ValueError("Invalid Kraus error input.")
    mats = [_as_square(k) for k in noise_ops]
    if len({k for _, k in mats}) != 1:
        raise ValueError("Kraus matrices of different sizes.")
    ks = [m for m, _ in mats]
    if not np.allclose(sum(m.conj().T @ m for m in ks), np.eye(ks[0].shape[0]), atol=ATOL):
        raise ValueError("Input Kraus matrices are not a CPTP channel.")
    return QuantumError(kraus_superop(ks), mats[0][1])


def mixed_unitary_error(noise_ops) -> QuantumError:
    """sum_j p_j U_j rho U_j^dag from pairs (U_j, p_j)."""
    ops = list(noise_ops) if isinstance(noise_ops, (list, tuple, zip)) else None
    if not ops:
        raise ValueError("Input noise ops is not a list." if ops is None else "Input noise list is empty.")
    mats = [(_as_square(u), p) for u, p in ops]
    k = mats[0][0][1]
    for (u, ku), _ in mats:
        if ku != k:
            raise ValueError("Input matrices different size.")
        if not np.allclose(u.conj().T @ u, np.eye(u.shape[0]), atol=ATOL):
            raise ValueError("Input matrix is not unitary.")
    _check_probs([p for _, p in mats])
    return QuantumError(sum(float(p) * np.kron(u.conj(), u) for (u, _), p in mats), k)


def coherent_unitary_error(unitary) -> QuantumError:
    return mixed_unitary_error([(unitary, 1)])


def pauli_error(noise_ops) -> QuantumError:
    """A Pauli mixture from pairs (label, p); labels read as qiskit's Pauli
    strings (the rightmost character on qubit 0)."""
    ops = list(noise_ops) if isinstance(noise_ops, (list, tuple, zip)) else None
    if not ops:
        raise ValueError("Input noise ops is not a list." if ops is None else "Input noise list is empty.")
    labels = [str(lab).upper() for lab, _ in ops]
    if any(not lab or set(lab) - set("IXYZ") for lab in labels):
        raise ValueError(f"Invalid Pauli input operator: {labels}")
    if len({len(lab) for lab in labels}) != 1:
        raise ValueError("Pauli's are not all of the same length.")
    probs = [float(p) for _, p in ops]
    _check_probs(probs)
    sup = 0
    for lab, p in zip(labels, probs):
        m = _kron_all([_P[c] for c in lab])
        sup = sup + p * np.kron(m.conj(), m)
    return QuantumError(sup, len(labels[0]))


_RESET0 = kraus_superop([np.array([[1, 0], [0, 0]], dtype=complex), np.array([[0, 1], [0, 0]], dtype=complex)])
_X = np.kron(_P["X"].conj(), _P["X"])
_Z = np.kron(_P["Z"].conj(), _P["Z"])


def reset_error(prob0: float, prob1: float = 0.0) -> QuantumError:
    """E(rho) = (1 - p0 - p1) rho + Tr[rho] (p0 |0><0| + p1 |1><1|)."""
    if prob0 < 0 or prob1 < 0 or prob0 > 1 or prob1 > 1 or prob0 + prob1 > 1:
        raise ValueError("Invalid reset probabilities.")
    return QuantumError((1 - prob0 - prob1) * np.eye(4) + prob0 * _RESET0 + prob1 * (_X @ _RESET0), 1)


def thermal_relaxation_error(t1: float, t2: float, time: float, excited_state_population: float = 0.0) -> QuantumError:
    """T1 relaxation towards the equilibrium populations (p0, p1) and T2
    dephasing over `time`.  For T2 <= T1 the reference builds it as a mixture
    of I, Z, reset to |0> and reset to |1>; for T1 < T2 <= 2 T1 from its Choi
    matrix; both are the channel rho00' = (1 - p1 r) rho00 + p0 r rho11,
    rho11' = p1 r rho00 + (1 - p0 r) rho11, rho01' = e^(-time/T2) rho01 with
    r = 1 - e^(-time/T1).  The mixture is built here for T2 <= T1, the Choi
    matrix's superoperator otherwise."""
    if excited_state_population < 0:
        raise ValueError(f"Invalid excited state population ({excited_state_population} < 0).")
    if excited_state_population > 1:
        raise ValueError(f"Invalid excited state population ({excited_state_population} > 1).")
    if time < 0:
        raise ValueError(f"Invalid gate_time ({time} < 0)")
    if t1 <= 0:
        raise ValueError("Invalid T_1 relaxation time parameter: T_1 <= 0.")
    if t2 <= 0:
        raise ValueError("Invalid T_2 relaxation time parameter: T_2 <= 0.")
    if t2 - 2 * t1 > 0:
        raise ValueError("Invalid T_2 relaxation time parameter: T_2 greater than 2 * T_1.")
    rate1, p_reset = (0.0, 0.0) if t1 == np.inf else (1 / t1, 1 - np.exp(-time / t1))
    rate2, exp_t2 = (0.0, 1.0) if t2 == np.inf else (1 / t2, np.exp(-time / t2))
    p1 = excited_state_population
    p0 = 1 - p1
    if t2 > t1:
        sup = np.zeros((4, 4), dtype=complex)  # vec index row + 2 col
        sup[0, 0], sup[0, 3] = 1 - p1 * p_reset, p0 * p_reset
        sup[3, 0], sup[3, 3] = p1 * p_reset, 1 - p0 * p_reset
        sup[1, 1] = sup[2, 2] = exp_t2
        return QuantumError(sup, 1)
    p_reset0, p_reset1 = p_reset * p0, p_reset * p1
    p_z = (1 - p_reset) * (1 - np.exp(-time * (rate2 - rate1))) / 2
    p_id = 1 - p_z - p_reset0 - p_reset1
    return QuantumError(p_id * np.eye(4) + p_z * _Z + p_reset0 * _RESET0 + p_reset1 * (_X @ _RESET0), 1)


def phase_damping_error(param_phase: float, canonical_kraus: bool = True) -> QuantumError:
    return phase_amplitude_damping_error(0.0, param_phase, 0.0)


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


def amplitude_damping_error(param_amp: float, excited_state_population: float = 0.0,
                            canonical_kraus: bool = True) -> QuantumError:
    return phase_amplitude_damping_error(param_amp, 0.0, excited_state_population)


def phase_amplitude_damping_error(param_amp, param_phase, excited_state_population=0.0,
                                  canonical_kraus: bool = True) -> QuantumError:
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


class ReadoutError:
    """Classical readout error of k qubits: probabilities[a][m] = P(read m |
    actual a), outcome index bit j on the error's qubit j
    (qiskit_aer/noise/errors/readout_error.py:36-110, checks :254-282)."""

    def __init__(self, probabilities, atol: float = ATOL):
        if probabilities is None or len(probabilities) == 0:
            raise ValueError("Input probabilities: empty.")
        rows = [np.asarray(r, dtype=np.float64) for r in probabilities]
        n_out = len(rows[0])
        k = int(np.log2(n_out)) if n_out else 0
        if n_out == 0 or 2 ** k != n_out:
            raise ValueError(f"Invalid probabilities: length {n_out} != 2**{k}")
        if len(rows) != n_out:
            raise ValueError("Invalid probabilities.")
        for r in rows:
            if len(r) != n_out:
                raise ValueError("Invalid probabilities: vectors are different lengths.")
            if abs(r.sum() - 1) > atol:
                raise ValueError(f"Invalid probabilities: sum({list(r)})= {r.sum()} is not 1.")
            if np.any(r < 0):
                raise ValueError(f"Invalid probabilities: {list(r)} contains a negative probability.")
        self.probabilities = np.array(rows)
        self.number_of_qubits = k

    def ideal(self) -> bool:
        return round(float(np.linalg.norm(self.probabilities - np.eye(self.probabilities.shape[0]))), 12) == 0

    # ---- algebra, as the reference's ReadoutError (readout_error.py:156-330):
    # rows are the actual outcome, columns the value read ----
    def copy(self) -> "ReadoutError":
        return ReadoutError(self.probabilities.copy())

    def to_dict(self) -> dict:
        return {"type": "roerror", "operations": ["measure"], "probabilities": self.probabilities.tolist()}

    @staticmethod
    def _other(other) -> "ReadoutError":
        return other if isinstance(other, ReadoutError) else ReadoutError(other)

    def _matmul(self, other, left_multiply: bool = False) -> "ReadoutError":
        other = self._other(other)
        if self.number_of_qubits != other.number_of_qubits:
            raise ValueError("other must have same number of qubits.")
        a, b = (other, self) if left_multiply else (self, other)
        return ReadoutError(a.probabilities @ b.probabilities)

    def compose(self, other, front: bool = False) -> "ReadoutError":
        """other * self (the reference's order); front=True gives self * other."""
        return self._matmul(other) if front else self._matmul(other, left_multiply=True)

    def dot(self, other) -> "ReadoutError":
        return self._matmul(other)

    def power(self, n: int) -> "ReadoutError":
        if not isinstance(n, int) or n < 1:
            raise ValueError("Can only power with positive integer powers.")
        ret = self.copy()
        for _ in range(1, n):
            ret = ret.compose(self)
        return ret

    def tensor(self, other) -> "ReadoutError":
        """self (x) other: other acts on the lower bits of the outcome."""
        return ReadoutError(np.kron(self.probabilities, self._other(other).probabilities))

    def expand(self, other) -> "ReadoutError":
        return ReadoutError(np.kron(self._other(other).probabilities, self.probabilities))

    def __matmul__(self, other):
        return self.compose(other)

    def __eq__(self, other) -> bool:
        return (isinstance(other, ReadoutError) and self.probabilities.shape == other.probabilities.shape
                and np.allclose(self.probabilities, other.probabilities, atol=ATOL))


def apply_readout(memory: int, bits, probs: np.ndarray, u: float) -> int:
    """ClassicalRegister::apply_roerror (framework/creg.hpp:230-262) on an
    integer classical memory: the actual value of `bits` (bit j of the value
    on bits[j]) picks the row of probs, one draw with uniform u
    (RngEngine::rand_int) gives the value read, written back to `bits`."""
    from .simulator import discrete_draw
    actual = 0
    for j, b in enumerate(bits):
        actual |= ((memory >> b) & 1) << j
    read = discrete_draw(probs[actual], u)
    for j, b in enumerate(bits):
        memory = (memory & ~(1 << b)) | (((read >> j) & 1) << b)
    return memory


# Standard instructions of fixed size, for the error-size check of
# NoiseModel._check_number_of_qubits (qiskit_aer/noise/noise_model.py:128-173, 1082-1107)
_1Q_INSTRUCTIONS = frozenset(["u1", "u2", "u3", "u", "p", "r", "rx", "ry", "rz", "id", "x", "y", "z", "h", "s", "sdg",
                              "sx", "sxdg", "t", "tdg"])
_2Q_INSTRUCTIONS = frozenset(["swap", "cx", "cy", "cz", "csx", "cp", "cu", "cu1", "cu2", "cu3", "rxx", "ryy", "rzz",
                              "rzx", "ecr"])
_3Q_INSTRUCTIONS = frozenset(["ccx", "cswap"])
# gates the simulator takes as they are: a noisy one among them joins basis_gates
_SIMULATOR_GATES = _1Q_INSTRUCTIONS | _2Q_INSTRUCTIONS | _3Q_INSTRUCTIONS | frozenset(
    ["ccz", "crx", "cry", "crz", "csxdg", "mcx", "mcy", "mcz", "mcp", "mcphase", "mcr", "mcrx", "mcry", "mcrz",
     "mcu", "mcu1", "mcu2", "mcu3", "mcswap", "mcsx", "mcsxdg", "delay", "pauli", "unitary", "diagonal"])


class NoiseModel:
    def __init__(self, basis_gates=None):
        # basis gates for compiling to the noise model (noise_model.py:193-199)
        self._basis_gates = set(["id", "rz", "sx", "cx"] if basis_gates is None else basis_gates)
        self._all_qubit = {}   # gate name -> QuantumError
        self._local = {}       # gate name -> {qubit tuple: QuantumError}
        self._readout_default = None   # single-qubit ReadoutError for every measured qubit
        self._readout_local = {}       # qubit tuple -> ReadoutError

    def add_all_qubit_readout_error(self, error, warnings: bool = True):
        """A single-qubit readout error on every measured qubit without one of
        its own; a second call replaces the first (noise_model.py:808-856)."""
        error = error if isinstance(error, ReadoutError) else ReadoutError(error)
        if error.ideal():
            return
        if error.number_of_qubits != 1:
            raise ValueError("All-qubit readout errors must defined as single-qubit errors.")
        self._readout_default = error

    def add_readout_error(self, error, qubits, warnings: bool = True):
        """A readout error on exactly these qubits (noise_model.py:858-920)."""
        error = error if isinstance(error, ReadoutError) else ReadoutError(error)
        if error.ideal():
            return
        qubits = tuple(int(q) for q in qubits)
        if error.number_of_qubits != len(qubits):
            raise ValueError(f"Number of qubits ({len(qubits)}) does not match the readout error size "
                             f"({error.number_of_qubits})")
        self._readout_local[qubits] = error

    def readout_ops(self, qubits, clbits) -> list:
        """The readout errors after a measurement of qubits into clbits, as
        (clbits, probabilities) in the order they apply
        (NoiseModel::sample_readout_noise, noise_model.hpp): one error over
        the whole measurement when one is given for exactly its qubits, else
        per qubit its own error or the all-qubit one."""
        qubits = [int(q) for q in qubits]
        exact = self._readout_local.get(tuple(qubits))
        if exact is not None:
            return [(list(clbits), exact.probabilities)]
        out = []
        for q, c in zip(qubits, clbits):
            e = self._readout_local.get((q,), self._readout_default)
            if e is not None:
                out.append(([int(c)], e.probabilities))
        return out

    @property
    def basis_gates(self) -> list:
        return sorted(self._basis_gates)

    def add_basis_gates(self, instructions) -> None:
        """Add instructions to basis_gates: those the simulator takes as
        gates (not measure, reset, kraus, superop; noise_model.py:652-667)."""
        for name in self._names(instructions):
            if name in _SIMULATOR_GATES:
                self._basis_gates.add(name)

    def reset(self) -> None:
        """Remove every error and restore the default basis gates."""
        self.__init__()

    @staticmethod
    def _check_number_of_qubits(error, name: str) -> None:
        for size, names in ((1, _1Q_INSTRUCTIONS), (2, _2Q_INSTRUCTIONS), (3, _3Q_INSTRUCTIONS)):
            if name in names and error.num_qubits != size:
                raise ValueError(f"{error.num_qubits} qubit QuantumError cannot be applied to {size} qubit "
                                 f'instruction "{name}".')

    def has_readout_errors(self) -> bool:
        return self._readout_default is not None or bool(self._readout_local)

    def has_quantum_errors(self) -> bool:
        return bool(self._all_qubit) or bool(self._local)

    @staticmethod
    def _names(instructions):
        return [instructions] if isinstance(instructions, str) else list(instructions)

    def add_all_qubit_quantum_error(self, error: QuantumError, instructions, warnings: bool = True):
        """An error after every listed gate or reset, or before every
        measure; a second error for the same instruction is composed after
        the first; an ideal error is not added."""
        if error.ideal():
            return
        for name in self._names(instructions):
            self._check_number_of_qubits(error, name)
            old = self._all_qubit.get(name)
            self._all_qubit[name] = error if old is None else old.compose(error)
            self.add_basis_gates(name)

    def add_quantum_error(self, error: QuantumError, instructions, qubits, warnings: bool = True):
        """An error on the listed instructions on exactly these qubits (in
        this order), used there in place of the all-qubit error: after a gate
        or reset, before a measure."""
        if error.ideal():
            return
        qubits = tuple(int(q) for q in qubits)
        if error.num_qubits != len(qubits):
            raise ValueError(f"Number of qubits ({len(qubits)}) does not match  the error size ({error.num_qubits})")
        for name in self._names(instructions):
            self._check_number_of_qubits(error, name)
            table = self._local.setdefault(name, {})
            old = table.get(qubits)
            table[qubits] = error if old is None else old.compose(error)
            self.add_basis_gates(name)

    def error_for(self, name: str, qubits=None):
        if qubits is not None:
            local = self._local.get(name, {}).get(tuple(int(q) for q in qubits))
            if local is not None:
                return local
        return self._all_qubit.get(name)

    def op_errors(self, name: str, qubits) -> list:
        """[(qubits, QuantumError)] an instruction gets
        (NoiseModel::sample_local_quantum_noise, noise_model.hpp:726-781).
        A gate gets the error for exactly its qubits, else the all-qubit
        one.  A measure or reset without an error for exactly its qubits gets,
        per qubit, that qubit's own error or the all-qubit one, because
        measure and reset act on any number of qubits while their errors are
        usually single-qubit."""
        qubits = [int(q) for q in qubits]
        if name not in ("measure", "reset"):
            err = self.error_for(name, qubits)
            return [] if err is None else [(qubits, err)]
        exact = self._local.get(name, {}).get(tuple(qubits))
        if exact is not None:
            return [(qubits, exact)]
        out = []
        for q in qubits:
            err = self.error_for(name, [q])
            if err is not None:
                out.append(([q], err))
        return out

    @property
    def noise_instructions(self) -> list:
        names = set(self._all_qubit) | set(self._local)
        return sorted(names | ({"measure"} if self.has_readout_errors() else set()))

    @property
    def noise_qubits(self) -> list:
        qs = {q for table in self._local.values() for key in table for q in key}
        return sorted(qs | {q for key in self._readout_local for q in key})

    def is_ideal(self) -> bool:
        return not self.has_quantum_errors() and not self.has_readout_errors()
