"""The reference's C runtime API (aer_state / aer_apply_* / aer_apply_measure,
include/aer_runtime_gb300.h) on the GPU: a circuit driven gate by gate equals
the oracle, single amplitudes and probabilities agree with the released
vector, and measurement collapses and renormalises with seeded outcomes."""
import ctypes as C

import numpy as np
import pytest

from _pkg import pkg
from oracle import oracle as O

pytestmark = pytest.mark.gpu


class CC(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


def _lib():
    L = pkg().lib()
    L.aer_state.restype = C.c_void_p
    L.aer_allocate_qubits.restype = C.c_uint64
    L.aer_allocate_qubits.argtypes = [C.c_void_p, C.c_uint64]
    L.aer_apply_measure.restype = C.c_uint64
    L.aer_apply_measure.argtypes = [C.c_void_p, C.POINTER(C.c_uint64), C.c_size_t]
    L.aer_probability.restype = C.c_double
    L.aer_probability.argtypes = [C.c_void_p, C.c_uint64]
    L.aer_amplitude.restype = CC
    L.aer_amplitude.argtypes = [C.c_void_p, C.c_uint64]
    L.aer_release_statevector.restype = C.POINTER(CC)
    L.aer_release_statevector.argtypes = [C.c_void_p]
    for f in ("aer_state_initialize", "aer_state_finalize"):
        getattr(L, f).argtypes = [C.c_void_p]
    L.aer_state_configure.argtypes = [C.c_void_p, C.c_char_p, C.c_char_p]
    for f in ("x", "y", "z", "h", "s", "sdg", "t", "tdg", "sx"):
        getattr(L, "aer_apply_" + f).argtypes = [C.c_void_p, C.c_uint64]
    for f in ("rx", "ry", "rz", "p"):
        getattr(L, "aer_apply_" + f).argtypes = [C.c_void_p, C.c_uint64, C.c_double]
    L.aer_apply_u3.argtypes = [C.c_void_p, C.c_uint64, C.c_double, C.c_double, C.c_double]
    for f in ("cx", "cy", "cz", "ch", "swap"):
        getattr(L, "aer_apply_" + f).argtypes = [C.c_void_p, C.c_uint64, C.c_uint64]
    for f in ("cp", "crx", "cry", "crz"):
        getattr(L, "aer_apply_" + f).argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_double]
    L.aer_apply_ccx.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64]
    L.aer_apply_cswap.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64]
    L.aer_apply_cu.argtypes = [C.c_void_p, C.c_uint64, C.c_uint64] + [C.c_double] * 4
    return L


def _new(L, n, seed=7):
    st = L.aer_state()
    L.aer_state_configure(st, b"method", b"statevector")
    L.aer_state_configure(st, b"device", b"GPU")
    L.aer_state_configure(st, b"precision", b"double")
    L.aer_state_configure(st, b"seed_simulator", str(seed).encode())
    assert L.aer_allocate_qubits(st, n) == 0
    L.aer_state_initialize(st)
    return st


def test_gate_by_gate_matches_oracle():
    L = _lib()
    n = 6
    st = _new(L, n)
    o = O.OracleQV(n)
    rng = np.random.default_rng(3)
    for _ in range(40):
        q = [int(x) for x in rng.choice(n, 3, replace=False)]
        th = rng.uniform(-3, 3, 4)
        g = int(rng.integers(0, 8))
        if g == 0:
            L.aer_apply_h(st, q[0]); o.apply_mcu([q[0]], O.u4(np.pi / 2, 0, np.pi, 0))
        elif g == 1:
            L.aer_apply_u3(st, q[0], *th[:3]); o.apply_mcu([q[0]], O.u4(th[0], th[1], th[2], 0))
        elif g == 2:
            L.aer_apply_cx(st, q[0], q[1]); o.apply_mcx(q[:2])
        elif g == 3:
            L.aer_apply_cp(st, q[0], q[1], th[0]); o.apply_mcphase(q[:2], np.exp(1j * th[0]))
        elif g == 4:
            L.aer_apply_ry(st, q[0], th[0]); o.apply_mcu([q[0]], O.rotation_matrix(1, th[0]))
        elif g == 5:
            L.aer_apply_ccx(st, q[0], q[1], q[2]); o.apply_mcx(q)
        elif g == 6:
            L.aer_apply_cu(st, q[0], q[1], *th); o.apply_mcu(q[:2], O.u4(*th))
        else:
            L.aer_apply_cswap(st, q[0], q[1], q[2]); o.apply_mcswap(q)
    a5 = L.aer_amplitude(st, 5)
    assert abs(complex(a5.re, a5.im) - o.data[5]) < 1e-12
    assert abs(L.aer_probability(st, 9) - abs(o.data[9]) ** 2) < 1e-12
    ptr = L.aer_release_statevector(st)
    got = np.array([complex(ptr[i].re, ptr[i].im) for i in range(1 << n)])
    np.testing.assert_allclose(got, o.data, atol=1e-12)
    L.aer_state_finalize(st)


def test_measure_collapses_and_is_seeded():
    L = _lib()
    outs = []
    for _ in range(2):
        st = _new(L, 3, seed=1234)
        L.aer_apply_h(st, 0)
        L.aer_apply_cx(st, 0, 1)
        L.aer_apply_cx(st, 1, 2)
        q = (C.c_uint64 * 1)(0)
        m = L.aer_apply_measure(st, q, 1)
        # GHZ: all qubits follow the measured one, state stays normalised
        want = 7 if m == 1 else 0
        assert abs(L.aer_probability(st, want) - 1.0) < 1e-12
        outs.append(m)
        L.aer_state_finalize(st)
    assert outs[0] == outs[1]
