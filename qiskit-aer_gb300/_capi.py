"""ctypes binding of libgbqv.so (include/gbqv.h).

The library is built in tree by ``_build.build()``.  Loading fails loudly
when it is missing or when no CUDA device is visible at state creation:
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libgbqv.so"

GBQV_OK = 0
ERRORS = {1: "argument", 2: "qubit", 3: "cuda", 4: "allocation", 5: "kind", 6: "timeout"}
C64, C128 = 0, 1
STATEVECTOR, DENSITY_MATRIX, UNITARY = 0, 1, 2


class GBQVError(RuntimeError):
    """A non-zero status from the C ABI; ``code`` is the gbqv_status value."""

    def __init__(self, code: int, message: str):
        super().__init__(f"[{ERRORS.get(code, code)}] {message}")
        self.code = code


class c128(C.Structure):
    _fields_ = [("re", C.c_double), ("im", C.c_double)]


class FusionConfig(C.Structure):
    _fields_ = [("method", C.c_int), ("enable", C.c_int), ("max_qubit", C.c_int), ("threshold", C.c_int),
                ("cost_factor", C.c_double), ("avx2_costs", C.c_int), ("allow_superop", C.c_int),
                ("allow_kraus", C.c_int)]


u64p = C.POINTER(C.c_uint64)
dp = C.POINTER(C.c_double)
vp = C.c_void_p
H = C.c_void_p

# name -> (restype, argtypes); every function returns an int status unless noted
_SIGS = {
    "gbqv_version": (C.c_int, []),
    "gbqv_last_error": (C.c_char_p, [H]),
    "gbqv_device_count": (C.c_int, []),
    "gbqv_uniforms": (C.c_int, [C.c_uint64, C.c_uint64, dp]),
    "gbqv_uniforms_streams": (C.c_int, [C.c_uint64, C.c_uint64, C.c_uint64, dp]),
    "gbqv_create": (C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(H)]),
    "gbqv_destroy": (C.c_int, [H]),
    "gbqv_num_qubits": (C.c_int, [H, C.POINTER(C.c_int)]),
    "gbqv_num_vector_qubits": (C.c_int, [H, C.POINTER(C.c_int)]),
    "gbqv_synchronize": (C.c_int, [H]),
    "gbqv_device_data": (C.c_int, [H, C.POINTER(vp)]),
    "gbqv_get_stream": (C.c_int, [H, C.POINTER(vp)]),
    "gbqv_launch_count": (C.c_uint64, []),
    "gbqv_zero": (C.c_int, [H]),
    "gbqv_initialize": (C.c_int, [H]),
    "gbqv_initialize_from_vector": (C.c_int, [H, vp, C.c_uint64]),
    "gbqv_copy_to_host": (C.c_int, [H, vp, C.c_uint64]),
    "gbqv_checkpoint": (C.c_int, [H]),
    "gbqv_revert": (C.c_int, [H, C.c_int]),
    "gbqv_inner_product": (C.c_int, [H, C.POINTER(c128)]),
    "gbqv_apply_matrix": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_apply_diagonal_matrix": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_apply_mcx": (C.c_int, [H, u64p, C.c_int]),
    "gbqv_apply_mcy": (C.c_int, [H, u64p, C.c_int]),
    "gbqv_apply_mcswap": (C.c_int, [H, u64p, C.c_int]),
    "gbqv_apply_mcphase": (C.c_int, [H, u64p, C.c_int, c128]),
    "gbqv_apply_mcu": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_apply_rotation": (C.c_int, [H, u64p, C.c_int, C.c_int, C.c_double]),
    "gbqv_apply_pauli": (C.c_int, [H, u64p, C.c_int, C.c_char_p, c128]),
    "gbqv_apply_permutation_matrix": (C.c_int, [H, u64p, C.c_int, u64p, C.c_int]),
    "gbqv_apply_multiplexer": (C.c_int, [H, u64p, C.c_int, u64p, C.c_int, vp]),
    "gbqv_apply_multi_swaps": (C.c_int, [H, u64p, C.c_int]),
    "gbqv_norm": (C.c_int, [H, dp]),
    "gbqv_norm_matrix": (C.c_int, [H, u64p, C.c_int, vp, dp]),
    "gbqv_probabilities": (C.c_int, [H, u64p, C.c_int, dp]),
    "gbqv_probability": (C.c_int, [H, C.c_uint64, dp]),
    "gbqv_set_sample_measure_index_size": (C.c_int, [H, C.c_int]),
    "gbqv_test_stall_tensor_pipeline": (C.c_int, [H, C.c_int]),
    "gbqv_set_run_tile_qubits": (C.c_int, [H, C.c_int]),
    "gbqv_set_run_jit": (C.c_int, [H, C.c_int]),
    "gbqv_run_jit_compile_check": (C.c_int, [C.c_int, C.c_char_p, C.c_size_t]),
    "gbqv_run_jit_counts": (C.c_int, [u64p, u64p]),
    "gbqv_sample_measure": (C.c_int, [H, dp, C.c_uint64, u64p]),
    "gbqv_expval_pauli": (C.c_int, [H, u64p, C.c_int, C.c_char_p, c128, dp]),
    "gbqv_expval_pauli_many": (C.c_int, [H, C.c_int, u64p, C.POINTER(C.c_int), C.POINTER(C.c_char_p), dp, dp, dp]),
    "gbqv_expval_pauli_many_noalloc": (C.c_int, [vp, C.c_int, C.c_int, C.c_int, u64p, C.POINTER(C.c_int),
                                                 C.POINTER(C.c_char_p), dp, vp, dp, dp]),
    "gbqv_dm_apply_superop_matrix": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_dm_apply_diagonal_superop_matrix": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_dm_apply_unitary_matrix": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_dm_apply_diagonal_unitary_matrix": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_dm_apply_cnot": (C.c_int, [H, C.c_uint64, C.c_uint64]),
    "gbqv_dm_apply_swap": (C.c_int, [H, C.c_uint64, C.c_uint64]),
    "gbqv_dm_apply_x": (C.c_int, [H, C.c_uint64]),
    "gbqv_dm_apply_y": (C.c_int, [H, C.c_uint64]),
    "gbqv_dm_apply_phase": (C.c_int, [H, C.c_uint64, c128]),
    "gbqv_dm_apply_cphase": (C.c_int, [H, C.c_uint64, C.c_uint64, c128]),
    "gbqv_dm_apply_toffoli": (C.c_int, [H, C.c_uint64, C.c_uint64, C.c_uint64]),
    "gbqv_dm_apply_reset": (C.c_int, [H, u64p, C.c_int]),
    "gbqv_dm_trace": (C.c_int, [H, C.POINTER(c128)]),
    "gbqv_circuit_create": (C.c_int, [C.c_int, C.POINTER(H)]),
    "gbqv_circuit_destroy": (C.c_int, [H]),
    "gbqv_circuit_gate": (C.c_int, [H, C.c_char_p, u64p, C.c_int, dp, C.c_int]),
    "gbqv_circuit_unitary": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_circuit_diagonal": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_circuit_superop": (C.c_int, [H, u64p, C.c_int, vp]),
    "gbqv_circuit_kraus": (C.c_int, [H, u64p, C.c_int, C.c_int, vp]),
    "gbqv_circuit_reset": (C.c_int, [H, u64p, C.c_int]),
    "gbqv_circuit_barrier": (C.c_int, [H, u64p, C.c_int]),
    "gbqv_circuit_num_ops": (C.c_int, [H, C.POINTER(C.c_int)]),
    "gbqv_circuit_op_info": (C.c_int, [H, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), u64p, C.c_int,
                                       C.c_char_p, C.c_int]),
    "gbqv_circuit_op_matrix": (C.c_int, [H, C.c_int, vp, C.c_uint64]),
    "gbqv_fusion_default_config": (C.c_int, [C.c_int, C.POINTER(FusionConfig)]),
    "gbqv_circuit_fuse": (C.c_int, [H, C.POINTER(FusionConfig), C.POINTER(C.c_int), C.c_char_p, C.c_int]),
    "gbqv_execute": (C.c_int, [H, H]),
    "gbqv_circuit_bind_param": (C.c_int, [H, C.c_int, C.c_int, C.c_int, dp]),
    "gbqv_circuit_num_bindings": (C.c_int, [H, C.POINTER(C.c_int)]),
    "gbqv_execute_bound": (C.c_int, [H, H, C.c_uint64, C.c_uint64]),
    "gbqv_expval_pauli_segments": (C.c_int, [H, C.c_int, C.c_uint64, C.c_int, u64p, C.POINTER(C.c_int),
                                             C.POINTER(C.c_char_p), dp]),
    "gbqv_sample_measure_segments": (C.c_int, [H, C.c_int, C.c_uint64, C.c_uint64, dp, C.c_uint64, u64p]),
    "gbqv_initialize_segments": (C.c_int, [H, C.c_int, C.c_uint64]),
    "gbqv_execute_segments": (C.c_int, [H, H]),
    "gbqv_probabilities_segments": (C.c_int, [H, C.c_int, C.c_uint64, u64p, C.c_int, dp]),
    "gbqv_draw_segments": (C.c_int, [H, C.c_int, C.c_uint64, u64p, C.c_int, dp, vp, dp]),
    "gbqv_collapse_segments": (C.c_int, [H, C.c_int, C.c_uint64, u64p, C.c_int, vp, vp, dp]),
    "gbqv_apply_matrix_segments": (C.c_int, [H, C.c_int, C.c_uint64, u64p, C.c_int, vp, vp]),
    "gbqv_rdm_segments": (C.c_int, [H, C.c_int, C.c_uint64, u64p, C.c_int, vp]),
    "gbqv_kraus_segments": (C.c_int, [H, C.c_int, C.c_uint64, u64p, C.c_int, vp, C.c_int, vp, dp]),
    "gbqv_set_blocking": (C.c_int, [H, C.c_int]),
    "gbqv_set_tensor_c128": (C.c_int, [H, C.c_int]),
    "gbqv_batch_create": (C.c_int, [C.c_int, C.POINTER(H)]),
    "gbqv_batch_destroy": (C.c_int, [H]),
    "gbqv_batch_add": (C.c_int, [H, C.c_int, C.c_int, C.POINTER(C.c_int), u64p, C.POINTER(C.c_int), dp, C.c_int,
                                 C.c_int, u64p, C.POINTER(C.c_int), C.POINTER(C.c_char_p), dp, C.c_uint64,
                                 C.c_uint64, C.POINTER(C.c_int)]),
    "gbqv_batch_run": (C.c_int, [H, C.c_int, dp]),
    "gbqv_batch_set_teams": (C.c_int, [H, C.c_int, C.c_double]),
    "gbqv_batch_set_fp64": (C.c_int, [H, C.c_int]),
    "gbqv_batch_result": (C.c_int, [H, C.c_int, dp, dp, C.c_int, u64p, C.c_uint64, dp]),
    "gbqv_adjoint_expval_grad": (C.c_int, [H, H, C.POINTER(C.c_int), dp, C.c_int, C.c_int, u64p, C.POINTER(C.c_int),
                                           C.POINTER(C.c_char_p), dp, dp, dp]),
}

_lib = None


def lib():
    """The loaded libgbqv.so with typed entry points (built on first use)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from . import _build

            _build.build()
        if not LIB_PATH.exists():
            raise GBQVError(3, f"libgbqv.so is missing at {LIB_PATH}; run the build first")
        L = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int, handle=None) -> None:
    if rc != GBQV_OK:
        msg = lib().gbqv_last_error(handle)
        raise GBQVError(rc, msg.decode() if msg else "unknown error")


def qubits_arg(qubits):
    a = np.ascontiguousarray(np.asarray(qubits, dtype=np.uint64).reshape(-1))
    return a, a.ctypes.data_as(u64p), int(a.size)


def cmat_arg(mat):
    """Column-major flattening of a 2-D matrix; 1-D input is taken as already
    vectorised (the reference's cvector_t layout)."""
    m = np.asarray(mat, dtype=np.complex128)
    if m.ndim == 2:
        m = m.reshape(-1, order="F")
    m = np.ascontiguousarray(m)
    return m, m.ctypes.data_as(vp)


def cz(z) -> c128:
    z = complex(z)
    return c128(z.real, z.imag)
