"""TEST INFRASTRUCTURE ONLY — Python face of the oracle.

Loads ``oracle/liboracle.so`` (the plain-C restatement in ``oracle_qv.c``) and,
where it was built, ``oracle/_ref/libaerref.so`` (the reference's own
QubitVector<double> / DensityMatrix<double> / UnitaryMatrix<double> compiled
from the qiskit-aer sources).  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline legs import this module; the engine never does.

The numpy helpers at the bottom restate the small host-side algorithms the
reference runs around the hot path: the gate matrices of
``src/framework/linalg/matrix_utils/vmatrix_defs.hpp``, the superoperator
construction of ``DensityMatrix::vmat2vsuperop`` (densitymatrix.hpp:265-281)
and of ``Utils::kraus_superop`` (src/framework/utils.hpp), and the noise
channels of ``qiskit_aer/noise/errors/standard_errors.py``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "liboracle.so"
REF_PATH = HERE / "_ref" / "libaerref.so"

class CComplex(C.Structure):
    """Passes a C99 double complex by value (same ABI as {double, double})."""

    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def _cz(z) -> CComplex:
    z = complex(z)
    return CComplex(z.real, z.imag)


_u64p = C.POINTER(C.c_uint64)
_dp = C.POINTER(C.c_double)
_vp = C.c_void_p


def build(ref: bool = False) -> None:
    """Compile liboracle.so (and, when the reference tree exists, _ref)."""
    subprocess.check_call(["make", "-s", "-C", str(HERE), "all"])
    if ref and Path(os.environ.get("AER_SRC", "/root/reference/src")).is_dir():
        subprocess.check_call(["make", "-s", "-C", str(HERE), "ref"])


def _u64(a) -> C.Array:
    a = np.ascontiguousarray(a, dtype=np.uint64)
    return a, a.ctypes.data_as(_u64p)


def _c128(a):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a, a.ctypes.data_as(_vp)


class _Lib:
    _lib = None

    @classmethod
    def get(cls):
        if cls._lib is None:
            if not LIB_PATH.exists():
                build()
            lib = C.CDLL(str(LIB_PATH))
            lib.orc_norm.restype = C.c_double
            lib.orc_expval_pauli.restype = C.c_int
            lib.orc_dm_expval_pauli.restype = C.c_int
            lib.orc_apply_pauli.restype = C.c_int
            lib.orc_mt64_next.restype = C.c_uint64
            cls._lib = lib
        return cls._lib


def set_threads(threads: int, omp_threshold: int = 14) -> None:
    _Lib.get().orc_set_threads(C.c_int(threads), C.c_int(omp_threshold))


def uniforms(seed: int, count: int) -> np.ndarray:
    """std::uniform_real_distribution<double>(0,1) over std::mt19937_64(seed)."""
    out = np.empty(count, dtype=np.float64)
    _Lib.get().orc_uniforms(C.c_uint64(seed), C.c_uint64(count), out.ctypes.data_as(_dp))
    return out


def _narrow(qubits, limit: int = 10) -> None:
    """The C restatement keeps per-group index tables of 2^limit entries."""
    if len(qubits) > limit:
        raise ValueError(f"the oracle applies matrices of at most {limit} qubits")


class OracleQV:
    """QubitVector<double> restated in C, on a numpy complex128 buffer."""

    def __init__(self, num_qubits: int, data: np.ndarray | None = None):
        self.n = num_qubits
        if data is None:
            self.data = np.zeros(1 << num_qubits, dtype=np.complex128)
            self.data[0] = 1.0
        else:
            self.data = np.ascontiguousarray(data, dtype=np.complex128).copy()
            assert self.data.size == 1 << num_qubits
        self.lib = _Lib.get()

    @property
    def _p(self):
        return self.data.ctypes.data_as(_vp)

    def apply_matrix(self, qubits, mat):
        _narrow(qubits, 13)
        q, qp = _u64(qubits)
        m, mp = _c128(np.asarray(mat).reshape(-1, order="F") if np.ndim(mat) == 2 else mat)
        self.lib.orc_apply_matrix(self._p, C.c_int(self.n), qp, C.c_int(len(q)), mp)

    def apply_diagonal_matrix(self, qubits, diag):
        _narrow(qubits)
        q, qp = _u64(qubits)
        d, dp = _c128(diag)
        self.lib.orc_apply_diagonal(self._p, C.c_int(self.n), qp, C.c_int(len(q)), dp)

    def apply_mcx(self, qubits):
        q, qp = _u64(qubits)
        self.lib.orc_apply_mcx(self._p, C.c_int(self.n), qp, C.c_int(len(q)))

    def apply_mcy(self, qubits):
        q, qp = _u64(qubits)
        self.lib.orc_apply_mcy(self._p, C.c_int(self.n), qp, C.c_int(len(q)))

    def apply_mcswap(self, qubits):
        q, qp = _u64(qubits)
        self.lib.orc_apply_mcswap(self._p, C.c_int(self.n), qp, C.c_int(len(q)))

    def apply_mcphase(self, qubits, phase):
        q, qp = _u64(qubits)
        ph = np.complex128(phase)
        self.lib.orc_apply_mcphase.argtypes = [_vp, C.c_int, _u64p, C.c_int, CComplex]
        self.lib.orc_apply_mcphase(self._p, self.n, qp, len(q), _cz(ph))

    def apply_mcu(self, qubits, mat):
        q, qp = _u64(qubits)
        m, mp = _c128(np.asarray(mat).reshape(-1, order="F") if np.ndim(mat) == 2 else mat)
        self.lib.orc_apply_mcu(self._p, C.c_int(self.n), qp, C.c_int(len(q)), mp)

    def apply_rotation(self, qubits, axis: int, theta: float):
        """QubitVector::apply_rotation (qubitvector.hpp:1722-1750)."""
        if axis in (0, 1, 2):
            self.apply_mcu(qubits, rotation_matrix(axis, theta))
        elif axis == 5:
            self.apply_diagonal_matrix(qubits, rzz_diag(theta))
        elif axis in (3, 4, 6):
            self.apply_matrix(qubits, rotation_matrix(axis, theta))
        else:
            raise ValueError("invalid rotation axis")

    def apply_pauli(self, qubits, label: str, coeff=1.0):
        q, qp = _u64(qubits)
        c = np.complex128(coeff)
        self.lib.orc_apply_pauli.argtypes = [_vp, C.c_int, _u64p, C.c_int, C.c_char_p, CComplex]
        rc = self.lib.orc_apply_pauli(self._p, self.n, qp, len(q), label.encode(), _cz(c))
        if rc:
            raise ValueError(f"invalid Pauli {label!r}")

    def apply_permutation_matrix(self, qubits, pairs):
        _narrow(qubits)
        q, qp = _u64(qubits)
        p, pp = _u64(np.asarray(pairs).reshape(-1))
        self.lib.orc_apply_permutation(self._p, C.c_int(self.n), qp, C.c_int(len(q)), pp,
                                       C.c_int(len(p) // 2))

    def apply_multiplexer(self, controls, targets, mat):
        c, cp = _u64(controls)
        t, tp = _u64(targets)
        m, mp = _c128(np.asarray(mat).reshape(-1, order="F") if np.ndim(mat) == 2 else mat)
        self.lib.orc_apply_multiplexer(self._p, C.c_int(self.n), cp, C.c_int(len(c)), tp,
                                       C.c_int(len(t)), mp)

    def apply_multi_swaps(self, qubits):
        q, qp = _u64(qubits)
        self.lib.orc_apply_multi_swaps(self._p, C.c_int(self.n), qp, C.c_int(len(q)))

    def norm(self) -> float:
        return float(self.lib.orc_norm(self._p, C.c_int(self.n)))

    def norm_matrix(self, qubits, mat) -> float:
        """QubitVector::norm(qubits, mat) = ||M psi||^2 (qubitvector.hpp:1888-2082)."""
        tmp = OracleQV(self.n, self.data)
        tmp.apply_matrix(qubits, mat)
        return tmp.norm()

    def expval_pauli(self, qubits, label: str, initial_phase=1.0) -> float:
        q, qp = _u64(qubits)
        ph = np.complex128(initial_phase)
        out = C.c_double()
        self.lib.orc_expval_pauli.argtypes = [_vp, C.c_int, _u64p, C.c_int, C.c_char_p,
                                              CComplex, _dp]
        rc = self.lib.orc_expval_pauli(self._p, self.n, qp, len(q), label.encode(), _cz(ph),
                                       C.byref(out))
        if rc:
            raise ValueError(f"invalid Pauli {label!r}")
        return out.value

    def probabilities(self, qubits=()) -> np.ndarray:
        q, qp = _u64(list(qubits))
        k = len(q)
        out = np.empty(1 << (k if k else self.n), dtype=np.float64)
        self.lib.orc_probabilities(self._p, C.c_int(self.n), qp, C.c_int(k), out.ctypes.data_as(_dp))
        return out

    def sample_measure(self, rnds, index_size: int = 10) -> np.ndarray:
        r = np.ascontiguousarray(rnds, dtype=np.float64)
        out = np.empty(r.size, dtype=np.uint64)
        self.lib.orc_sample_measure(self._p, C.c_int(self.n), r.ctypes.data_as(_dp),
                                    C.c_uint64(r.size), out.ctypes.data_as(_u64p), C.c_int(index_size))
        return out

    def inner_product(self, other: np.ndarray) -> complex:
        o = np.ascontiguousarray(other, dtype=np.complex128)
        re, im = C.c_double(), C.c_double()
        self.lib.orc_inner_product(self._p, o.ctypes.data_as(_vp), C.c_int(self.n), C.byref(re),
                                   C.byref(im))
        return complex(re.value, im.value)


class OracleDM(OracleQV):
    """DensityMatrix<double> restated: vec(rho) over 2n vector qubits."""

    def __init__(self, num_qubits: int, data: np.ndarray | None = None):
        self.nq = num_qubits
        if data is not None and np.asarray(data).size == 1 << num_qubits:
            psi = np.asarray(data, dtype=np.complex128)
            data = np.kron(psi.conj(), psi)
        super().__init__(2 * num_qubits, data)

    def superop_qubits(self, qubits):
        return list(qubits) + [q + self.nq for q in qubits]

    def apply_superop_matrix(self, qubits, mat):
        self.apply_matrix(self.superop_qubits(qubits), mat)

    def apply_diagonal_superop_matrix(self, qubits, diag):
        self.apply_diagonal_matrix(self.superop_qubits(qubits), diag)

    def apply_unitary_matrix(self, qubits, mat):
        """DensityMatrix::apply_unitary_matrix (densitymatrix.hpp:297-317)."""
        mat = np.asarray(mat, dtype=np.complex128)
        if mat.ndim == 1:
            d = int(round(np.sqrt(mat.size)))
            mat = mat.reshape(d, d, order="F")
        if len(qubits) > 4:
            self.apply_matrix(list(qubits), mat)
            self.apply_matrix([q + self.nq for q in qubits], mat.conj())
        else:
            self.apply_superop_matrix(qubits, vmat2vsuperop(mat))

    def apply_diagonal_unitary_matrix(self, qubits, diag):
        diag = np.asarray(diag, dtype=np.complex128)
        self.apply_diagonal_superop_matrix(qubits, np.kron(diag.conj(), diag))

    def apply_cnot(self, c, t):
        pairs = [(1, 3), (4, 12), (5, 15), (6, 14), (7, 13), (9, 11)]
        self.apply_permutation_matrix([c, t, c + self.nq, t + self.nq], pairs)

    def apply_swap(self, a, b):
        pairs = [(1, 2), (4, 8), (5, 10), (6, 9), (7, 11), (13, 14)]
        self.apply_permutation_matrix([a, b, a + self.nq, b + self.nq], pairs)

    def apply_toffoli(self, a, b, c):
        pairs = [(3, 7), (11, 15), (19, 23), (24, 56), (25, 57), (26, 58), (27, 63), (28, 60),
                 (29, 61), (30, 62), (31, 59), (35, 39), (43, 47), (51, 55)]
        nq = self.nq
        self.apply_permutation_matrix([a, b, c, a + nq, b + nq, c + nq], pairs)

    def apply_reset(self, qubits):
        """DensityMatrix::apply_reset via SMatrix::reset (densitymatrix.hpp:536-541)."""
        self.apply_superop_matrix(qubits, reset_superop(len(qubits)).reshape(-1, order="F"))

    def expval_pauli(self, qubits, label: str, initial_phase=1.0) -> float:
        q, qp = _u64(qubits)
        ph = np.complex128(initial_phase)
        out = C.c_double()
        self.lib.orc_dm_expval_pauli.argtypes = [_vp, C.c_int, _u64p, C.c_int, C.c_char_p,
                                                 CComplex, _dp]
        rc = self.lib.orc_dm_expval_pauli(self._p, self.nq, qp, len(q), label.encode(), _cz(ph),
                                          C.byref(out))
        if rc:
            raise ValueError(f"invalid Pauli {label!r}")
        return out.value

    def probabilities(self, qubits=()) -> np.ndarray:
        q, qp = _u64(list(qubits))
        k = len(q)
        out = np.empty(1 << (k if k else self.nq), dtype=np.float64)
        self.lib.orc_dm_probabilities(self._p, C.c_int(self.nq), qp, C.c_int(k), out.ctypes.data_as(_dp))
        return out

    def sample_measure(self, rnds, index_size: int = 10) -> np.ndarray:
        r = np.ascontiguousarray(rnds, dtype=np.float64)
        out = np.empty(r.size, dtype=np.uint64)
        self.lib.orc_dm_sample_measure(self._p, C.c_int(self.nq), r.ctypes.data_as(_dp),
                                       C.c_uint64(r.size), out.ctypes.data_as(_u64p), C.c_int(index_size))
        return out

    def trace(self) -> complex:
        d = 1 << self.nq
        return complex(self.data[:: d + 1].sum())


# --------------------------------------------------------------------------
# Gate matrices, vmatrix_defs.hpp (column-major flattening = mat.reshape(-1, order="F"))
# --------------------------------------------------------------------------
def u3(theta, phi, lam):
    """VMatrix::u3 (vmatrix_defs.hpp:217-225)."""
    c, s = np.cos(0.5 * theta), np.sin(0.5 * theta)
    return np.array([[c, -np.exp(1j * lam) * s], [np.exp(1j * phi) * s, np.exp(1j * (phi + lam)) * c]])


def u4(theta, phi, lam, gamma):
    """VMatrix::u4 (vmatrix_defs.hpp:227-235)."""
    c, s = np.cos(0.5 * theta), np.sin(0.5 * theta)
    return np.array([[np.exp(1j * gamma) * c, -np.exp(1j * (lam + gamma)) * s],
                     [np.exp(1j * (phi + gamma)) * s, np.exp(1j * (phi + lam + gamma)) * c]])


def rotation_matrix(axis: int, theta: float) -> np.ndarray:
    """VMatrix::rx/ry/rz/rxx/ryy/rzz/rzx (vmatrix_defs.hpp:247-320)."""
    c, s = np.cos(0.5 * theta), np.sin(0.5 * theta)
    if axis == 0:
        return np.array([[c, -1j * s], [-1j * s, c]])
    if axis == 1:
        return np.array([[c, -s], [s, c]], dtype=np.complex128)
    if axis == 2:
        return np.array([[np.exp(-0.5j * theta), 0], [0, np.exp(0.5j * theta)]])
    m = np.zeros((4, 4), dtype=np.complex128)
    if axis == 3:
        m[0, 0] = m[1, 1] = m[2, 2] = m[3, 3] = c
        m[0, 3] = m[1, 2] = m[2, 1] = m[3, 0] = -1j * s
    elif axis == 4:
        m[0, 0] = m[1, 1] = m[2, 2] = m[3, 3] = c
        m[0, 3] = m[3, 0] = 1j * s
        m[1, 2] = m[2, 1] = -1j * s
    elif axis == 5:
        m = np.diag(rzz_diag(theta))
    elif axis == 6:
        m[0, 0] = m[1, 1] = m[2, 2] = m[3, 3] = c
        m[0, 2] = m[2, 0] = -1j * s
        m[1, 3] = m[3, 1] = 1j * s
    return m


def rzz_diag(theta):
    ep, em = np.exp(0.5j * theta), np.exp(-0.5j * theta)
    return np.array([em, ep, ep, em])


def vmat2vsuperop(mat: np.ndarray) -> np.ndarray:
    """conj(U) (x) U in the reference's vectorised layout (densitymatrix.hpp:265-281).

    Returned as a 2-D (column-major meaning) superoperator matrix S with
    S[dim*i + k, dim*j + l] = conj(U[i, j]) * U[k, l]."""
    return np.kron(np.conj(mat), mat)


def kraus_superop(kraus) -> np.ndarray:
    """Sum of conj(K) (x) K (Utils::kraus_superop, src/framework/utils.hpp)."""
    return sum(np.kron(np.conj(k), k) for k in kraus)


def reset_superop(k: int) -> np.ndarray:
    """SMatrix::reset(dim) (smatrix_defs.hpp): every |i><j| -> delta_ij |0><0|."""
    dim = 1 << k
    s = np.zeros((dim * dim, dim * dim), dtype=np.complex128)
    for i in range(dim):
        s[0, i * (dim + 1)] = 1.0
    return s


PAULI = {
    "I": np.eye(2, dtype=np.complex128),
    "X": np.array([[0, 1], [1, 0]], dtype=np.complex128),
    "Y": np.array([[0, -1j], [1j, 0]], dtype=np.complex128),
    "Z": np.array([[1, 0], [0, -1]], dtype=np.complex128),
}


def depolarizing_superop(p: float, num_qubits: int = 1) -> np.ndarray:
    """depolarizing_error(p, n) as a superoperator (standard_errors.py:170-219):
    identity with 1 - p * (4^n - 1) / 4^n, every other Pauli with p / 4^n."""
    import itertools

    terms = 4 ** num_qubits
    max_param = terms / (terms - 1)
    probs = [1 - p / max_param] + (terms - 1) * [p / terms]
    total = 0
    for prob, labels in zip(probs, itertools.product("IXYZ", repeat=num_qubits)):
        m = np.array([[1.0 + 0j]])
        for lab in labels:
            m = np.kron(m, PAULI[lab])
        total = total + prob * np.kron(m.conj(), m)
    return total


def amplitude_damping_kraus(gamma: float):
    """amplitude_damping_error(gamma) Kraus set (standard_errors.py:351-462)."""
    a0 = np.array([[1, 0], [0, np.sqrt(1 - gamma)]], dtype=np.complex128)
    a1 = np.array([[0, np.sqrt(gamma)], [0, 0]], dtype=np.complex128)
    return [k for k in (a0, a1) if np.linalg.norm(k) > 1e-10]


def amplitude_damping_superop(gamma: float) -> np.ndarray:
    return kraus_superop(amplitude_damping_kraus(gamma))


def dense_pauli(label: str) -> np.ndarray:
    m = np.array([[1.0 + 0j]])
    for lab in label:
        m = np.kron(m, PAULI[lab])
    return m


class RefQV:
    """The reference's own QubitVector<double>, through oracle/_ref/libaerref.so."""

    _lib = None

    @classmethod
    def lib(cls):
        if cls._lib is None:
            lib = C.CDLL(str(REF_PATH))
            lib.ref_qv_create.restype = _vp
            lib.ref_dm_create.restype = _vp
            lib.ref_um_create.restype = _vp
            for f in ("ref_qv_norm", "ref_qv_expval_pauli", "ref_dm_expval_pauli", "ref_qv_norm_matrix"):
                getattr(lib, f).restype = C.c_double
            cls._lib = lib
        return cls._lib

    @staticmethod
    def available() -> bool:
        return REF_PATH.exists()
