"""Python mirror of the reference's qreg surface on the GB300 engine.

``QubitVector`` follows AER::QV::QubitVector<T> / QubitVectorThrust<T>
(src/simulators/statevector/qubitvector.hpp:61-651) and ``DensityMatrix``
follows AER::QV::DensityMatrix<T> (src/simulators/density_matrix/
densitymatrix.hpp:34-171): same member names, argument meaning (column-major
matrices, qubits[0] = least-significant matrix bit, target last, Pauli labels
read right to left) and errors (``GBQVError`` where the reference raises
std::runtime_error / std::invalid_argument).  Every call goes through the C
ABI of libgbqv.so; the amplitudes stay in HBM until ``copy_to_vector``.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi as A

PRECISIONS = {"double": A.C128, "single": A.C64, "complex128": A.C128, "complex64": A.C64}


class QubitVector:
    """A 2^n-amplitude statevector resident on the GPU."""

    _kind = A.STATEVECTOR

    def __init__(self, num_qubits: int, precision: str = "double"):
        if precision not in PRECISIONS:
            raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
        self._L = A.lib()
        h = C.c_void_p()
        A.check(self._L.gbqv_create(int(num_qubits), PRECISIONS[precision], self._kind, C.byref(h)))
        self._h = h
        self.precision = "double" if PRECISIONS[precision] == A.C128 else "single"
        self._nq = int(num_qubits)

    # ---- lifetime ----
    def close(self) -> None:
        if getattr(self, "_h", None):
            self._L.gbqv_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _c(self, rc: int) -> None:
        A.check(rc, self._h)

    @property
    def handle(self):
        return self._h

    def num_qubits(self) -> int:
        return self._nq

    def num_vector_qubits(self) -> int:
        v = C.c_int()
        self._c(self._L.gbqv_num_vector_qubits(self._h, C.byref(v)))
        return v.value

    def size(self) -> int:
        return 1 << self.num_vector_qubits()

    def synchronize(self) -> None:
        self._c(self._L.gbqv_synchronize(self._h))

    def stream(self) -> int:
        """The handle's cudaStream_t as an integer (for torch.cuda.ExternalStream)."""
        p = C.c_void_p()
        self._c(self._L.gbqv_get_stream(self._h, C.byref(p)))
        return p.value or 0

    def set_tensor_c128(self, mode) -> None:
        """complex128 dense 4/5-qubit gates: True / 1 tensor cores (tcgen05 for
        4 qubits, the default), 2 tensor cores through mma.sync only, False / 0
        FP64 FMAs."""
        self._c(self._L.gbqv_set_tensor_c128(self._h, int(mode)))

    def device_pointer(self) -> int:
        p = C.c_void_p()
        self._c(self._L.gbqv_device_data(self._h, C.byref(p)))
        return p.value

    # ---- state ----
    def zero(self) -> None:
        self._c(self._L.gbqv_zero(self._h))

    def initialize(self) -> None:
        self._c(self._L.gbqv_initialize(self._h))

    def initialize_from_vector(self, vec) -> None:
        v = np.ascontiguousarray(np.asarray(vec, dtype=np.complex128).reshape(-1))
        self._c(self._L.gbqv_initialize_from_vector(self._h, v.ctypes.data_as(A.vp), v.size))

    def copy_to_vector(self) -> np.ndarray:
        out = np.empty(self.size(), dtype=np.complex128)
        self._c(self._L.gbqv_copy_to_host(self._h, out.ctypes.data_as(A.vp), out.size))
        return out

    move_to_vector = copy_to_vector
    vector = copy_to_vector

    def checkpoint(self) -> None:
        self._c(self._L.gbqv_checkpoint(self._h))

    def revert(self, keep: bool) -> None:
        self._c(self._L.gbqv_revert(self._h, int(bool(keep))))

    def inner_product(self) -> complex:
        z = A.c128()
        self._c(self._L.gbqv_inner_product(self._h, C.byref(z)))
        return complex(z.re, z.im)

    # ---- gates ----
    def apply_matrix(self, qubits, mat) -> None:
        q, qp, k = A.qubits_arg(qubits)
        m, mp = A.cmat_arg(mat)
        if m.size != 1 << (2 * k):
            raise A.GBQVError(1, f"matrix has {m.size} entries, expected {1 << (2 * k)}")
        self._c(self._L.gbqv_apply_matrix(self._h, qp, k, mp))

    def apply_diagonal_matrix(self, qubits, diag) -> None:
        q, qp, k = A.qubits_arg(qubits)
        d, dp = A.cmat_arg(np.asarray(diag).reshape(-1))
        if d.size != 1 << k:
            raise A.GBQVError(1, f"diagonal has {d.size} entries, expected {1 << k}")
        self._c(self._L.gbqv_apply_diagonal_matrix(self._h, qp, k, dp))

    def apply_mcx(self, qubits) -> None:
        q, qp, k = A.qubits_arg(qubits)
        self._c(self._L.gbqv_apply_mcx(self._h, qp, k))

    def apply_mcy(self, qubits) -> None:
        q, qp, k = A.qubits_arg(qubits)
        self._c(self._L.gbqv_apply_mcy(self._h, qp, k))

    def apply_mcswap(self, qubits) -> None:
        q, qp, k = A.qubits_arg(qubits)
        self._c(self._L.gbqv_apply_mcswap(self._h, qp, k))

    def apply_mcphase(self, qubits, phase) -> None:
        q, qp, k = A.qubits_arg(qubits)
        self._c(self._L.gbqv_apply_mcphase(self._h, qp, k, A.cz(phase)))

    def apply_mcu(self, qubits, mat) -> None:
        q, qp, k = A.qubits_arg(qubits)
        m, mp = A.cmat_arg(mat)
        if m.size != 4:
            raise A.GBQVError(1, "apply_mcu takes a 2x2 matrix")
        self._c(self._L.gbqv_apply_mcu(self._h, qp, k, mp))

    def apply_rotation(self, qubits, axis: int, theta: float) -> None:
        q, qp, k = A.qubits_arg(qubits)
        self._c(self._L.gbqv_apply_rotation(self._h, qp, k, int(axis), float(theta)))

    def apply_pauli(self, qubits, pauli: str, coeff=1.0) -> None:
        q, qp, k = A.qubits_arg(qubits)
        self._c(self._L.gbqv_apply_pauli(self._h, qp, k, pauli.encode(), A.cz(coeff)))

    def apply_permutation_matrix(self, qubits, pairs) -> None:
        q, qp, k = A.qubits_arg(qubits)
        p = np.ascontiguousarray(np.asarray(pairs, dtype=np.uint64).reshape(-1))
        self._c(self._L.gbqv_apply_permutation_matrix(self._h, qp, k, p.ctypes.data_as(A.u64p), p.size // 2))

    def apply_multiplexer(self, control_qubits, target_qubits, mat) -> None:
        c, cp, nc = A.qubits_arg(control_qubits)
        t, tp, nt = A.qubits_arg(target_qubits)
        m, mp = A.cmat_arg(mat)
        self._c(self._L.gbqv_apply_multiplexer(self._h, cp, nc, tp, nt, mp))

    def apply_multi_swaps(self, qubits) -> None:
        q, qp, k = A.qubits_arg(qubits)
        self._c(self._L.gbqv_apply_multi_swaps(self._h, qp, k))

    # ---- reductions ----
    def norm(self, qubits=None, mat=None) -> float:
        out = C.c_double()
        if qubits is None:
            self._c(self._L.gbqv_norm(self._h, C.byref(out)))
        else:
            q, qp, k = A.qubits_arg(qubits)
            m, mp = A.cmat_arg(mat)
            self._c(self._L.gbqv_norm_matrix(self._h, qp, k, mp, C.byref(out)))
        return out.value

    def norm_matrix(self, qubits, mat) -> float:
        return self.norm(qubits, mat)

    def probabilities(self, qubits=()) -> np.ndarray:
        q, qp, k = A.qubits_arg(list(qubits))
        nbits = k if k else self._nq
        out = np.empty(1 << nbits, dtype=np.float64)
        self._c(self._L.gbqv_probabilities(self._h, qp, k, out.ctypes.data_as(A.dp)))
        return out

    def probability(self, outcome: int) -> float:
        """QubitVector::probability (qubitvector.hpp:302): the one entry read back."""
        v = C.c_double()
        self._c(self._L.gbqv_probability(self._h, int(outcome), C.byref(v)))
        return v.value

    def set_sample_measure_index_size(self, index_size: int) -> None:
        """QubitVector::set_sample_measure_index_size (qubitvector.hpp:457)."""
        self._c(self._L.gbqv_set_sample_measure_index_size(self._h, int(index_size)))

    def sample_measure(self, rnds) -> np.ndarray:
        r = np.ascontiguousarray(np.asarray(rnds, dtype=np.float64).reshape(-1))
        out = np.empty(r.size, dtype=np.uint64)
        self._c(self._L.gbqv_sample_measure(self._h, r.ctypes.data_as(A.dp), r.size, out.ctypes.data_as(A.u64p)))
        return out

    def expval_pauli(self, qubits, pauli: str, initial_phase=1.0) -> float:
        q, qp, k = A.qubits_arg(qubits)
        out = C.c_double()
        self._c(self._L.gbqv_expval_pauli(self._h, qp, k, pauli.encode(), A.cz(initial_phase), C.byref(out)))
        return out.value

    def expval_pauli_many(self, terms, coeffs=None):
        """terms: list of (qubits, label); returns (per-term values, weighted sum)."""
        qs, offs, labels = [], [0], []
        for q, lab in terms:
            qs.extend(int(x) for x in q)
            offs.append(len(qs))
            labels.append(lab.encode())
        qa = np.ascontiguousarray(np.asarray(qs, dtype=np.uint64))
        oa = (C.c_int * len(offs))(*offs)
        la = (C.c_char_p * max(1, len(labels)))(*labels)
        ca = np.ascontiguousarray(np.ones(len(labels)) if coeffs is None else np.asarray(coeffs, dtype=np.float64))
        out = np.empty(len(labels), dtype=np.float64)
        total = C.c_double()
        self._c(self._L.gbqv_expval_pauli_many(self._h, len(labels), qa.ctypes.data_as(A.u64p), oa, la,
                                               ca.ctypes.data_as(A.dp), out.ctypes.data_as(A.dp), C.byref(total)))
        return out, total.value


    def expval_pauli_segments(self, state_qubits: int, nseg: int, terms) -> np.ndarray:
        """<P_t> on each of the first nseg states of a stack of
        2^state_qubits-amplitude states: array [term, state]."""
        qs, offs, labels = [], [0], []
        for q, lab in terms:
            qs.extend(int(x) for x in q)
            offs.append(len(qs))
            labels.append(lab.encode())
        qa = np.ascontiguousarray(np.asarray(qs, dtype=np.uint64))
        oa = (C.c_int * len(offs))(*offs)
        la = (C.c_char_p * max(1, len(labels)))(*labels)
        out = np.empty((len(labels), int(nseg)), dtype=np.float64)
        if labels:
            self._c(self._L.gbqv_expval_pauli_segments(self._h, int(state_qubits), int(nseg), len(labels),
                                                       qa.ctypes.data_as(A.u64p), oa, la, out.ctypes.data_as(A.dp)))
        return out


class DensityMatrix(QubitVector):
    """vec(rho) of n qubits over 2n vector qubits, resident on the GPU."""

    _kind = A.DENSITY_MATRIX

    def initialize_from_vector(self, vec) -> None:
        """Length 4^n: an already vectorised rho; length 2^n: a pure state."""
        super().initialize_from_vector(vec)

    def initialize_from_matrix(self, mat) -> None:
        m = np.asarray(mat, dtype=np.complex128)
        super().initialize_from_vector(m.reshape(-1, order="F"))

    def copy_to_matrix(self) -> np.ndarray:
        d = 1 << self._nq
        return self.copy_to_vector().reshape(d, d, order="F")

    def _q(self, qubits):
        return A.qubits_arg(qubits)

    def apply_superop_matrix(self, qubits, mat) -> None:
        q, qp, k = self._q(qubits)
        m, mp = A.cmat_arg(mat)
        self._c(self._L.gbqv_dm_apply_superop_matrix(self._h, qp, k, mp))

    def apply_diagonal_superop_matrix(self, qubits, diag) -> None:
        q, qp, k = self._q(qubits)
        d, dp = A.cmat_arg(np.asarray(diag).reshape(-1))
        self._c(self._L.gbqv_dm_apply_diagonal_superop_matrix(self._h, qp, k, dp))

    def apply_unitary_matrix(self, qubits, mat) -> None:
        q, qp, k = self._q(qubits)
        m, mp = A.cmat_arg(mat)
        self._c(self._L.gbqv_dm_apply_unitary_matrix(self._h, qp, k, mp))

    def apply_diagonal_unitary_matrix(self, qubits, diag) -> None:
        q, qp, k = self._q(qubits)
        d, dp = A.cmat_arg(np.asarray(diag).reshape(-1))
        self._c(self._L.gbqv_dm_apply_diagonal_unitary_matrix(self._h, qp, k, dp))

    def apply_cnot(self, qctrl: int, qtrgt: int) -> None:
        self._c(self._L.gbqv_dm_apply_cnot(self._h, int(qctrl), int(qtrgt)))

    def apply_swap(self, q0: int, q1: int) -> None:
        self._c(self._L.gbqv_dm_apply_swap(self._h, int(q0), int(q1)))

    def apply_x(self, q: int) -> None:
        self._c(self._L.gbqv_dm_apply_x(self._h, int(q)))

    def apply_y(self, q: int) -> None:
        self._c(self._L.gbqv_dm_apply_y(self._h, int(q)))

    def apply_phase(self, q: int, phase) -> None:
        self._c(self._L.gbqv_dm_apply_phase(self._h, int(q), A.cz(phase)))

    def apply_cphase(self, q0: int, q1: int, phase) -> None:
        self._c(self._L.gbqv_dm_apply_cphase(self._h, int(q0), int(q1), A.cz(phase)))

    def apply_toffoli(self, c0: int, c1: int, t: int) -> None:
        self._c(self._L.gbqv_dm_apply_toffoli(self._h, int(c0), int(c1), int(t)))

    def apply_reset(self, qubits) -> None:
        q, qp, k = self._q(qubits)
        self._c(self._L.gbqv_dm_apply_reset(self._h, qp, k))

    def trace(self) -> complex:
        z = A.c128()
        self._c(self._L.gbqv_dm_trace(self._h, C.byref(z)))
        return complex(z.re, z.im)


class UnitaryMatrix(QubitVector):
    """QV::UnitaryMatrix (src/simulators/unitary/unitarymatrix.hpp): the
    2^n x 2^n matrix of the unitary method, stored column-major over 2n vector
    qubits and resident on the GPU; starts as the identity, and gates on
    qubits 0..n-1 multiply it from the left."""

    _kind = A.UNITARY

    def initialize_from_matrix(self, mat) -> None:
        m = np.asarray(mat, dtype=np.complex128)
        d = 1 << self._nq
        if m.shape != (d, d):
            raise ValueError("Unitary::State::initialize: initial state does not match qubit number")
        super().initialize_from_vector(m.reshape(-1, order="F"))

    def copy_to_matrix(self) -> np.ndarray:
        d = 1 << self._nq
        return self.copy_to_vector().reshape(d, d, order="F")

    move_to_matrix = copy_to_matrix
