"""Replays the golden fixtures (tests/golden/*_cases.*) on any object with the
QubitVector / DensityMatrix method surface: the oracle (CPU) or the engine's
Python mirror (GPU).  Each case starts from the recorded input state, applies
one op and yields (case, output state, reduction result)."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(kind: str):
    cases = json.loads((GOLDEN / f"{kind}_cases.json").read_text())
    arrays = np.load(GOLDEN / f"{kind}_cases.npz")
    return cases, arrays


def apply_case(obj, case, arrays, i):
    """Apply case i to obj (already holding arrays[f'in{i}']); returns the
    reduction result (or None)."""
    op = case["op"]
    q = case.get("qubits", [])
    mat = arrays[f"mat{i}"] if f"mat{i}" in arrays.files else None
    if op == "apply_matrix":
        obj.apply_matrix(q, mat)
    elif op == "apply_diagonal_matrix":
        obj.apply_diagonal_matrix(q, mat)
    elif op in ("apply_mcx", "apply_mcy", "apply_mcswap"):
        getattr(obj, op)(q)
    elif op == "apply_mcphase":
        obj.apply_mcphase(q, complex(*case["phase"]))
    elif op == "apply_mcu":
        obj.apply_mcu(q, mat)
    elif op == "apply_rotation":
        obj.apply_rotation(q, case["axis"], case["theta"])
    elif op == "apply_pauli":
        obj.apply_pauli(q, case["label"], complex(*case["coeff"]))
    elif op == "apply_permutation_matrix":
        obj.apply_permutation_matrix(q, case["pairs"])
    elif op == "apply_multiplexer":
        obj.apply_multiplexer(case["controls"], case["targets"], mat)
    elif op == "apply_multi_swaps":
        obj.apply_multi_swaps(q)
    elif op == "norm":
        return obj.norm()
    elif op == "norm_matrix":
        return obj.norm_matrix(q, mat)
    elif op == "expval_pauli":
        ph = complex(*case["phase"]) if "phase" in case else 1.0
        return obj.expval_pauli(q, case["label"], ph)
    elif op == "probabilities":
        return obj.probabilities(q)
    # density matrix
    elif op == "apply_superop_matrix":
        obj.apply_superop_matrix(q, mat)
    elif op == "apply_unitary_matrix":
        obj.apply_unitary_matrix(q, mat)
    elif op == "apply_diagonal_unitary_matrix":
        obj.apply_diagonal_unitary_matrix(q, mat)
    elif op == "apply_cnot":
        obj.apply_cnot(*q)
    elif op == "apply_swap":
        obj.apply_swap(*q)
    elif op == "apply_x":
        obj.apply_x(q[0])
    elif op == "apply_y":
        obj.apply_y(q[0])
    elif op == "apply_phase":
        obj.apply_phase(q[0], complex(*case["phase"]))
    elif op == "apply_cphase":
        obj.apply_cphase(q[0], q[1], complex(*case["phase"]))
    elif op == "apply_toffoli":
        obj.apply_toffoli(*q)
    elif op == "apply_reset":
        obj.apply_reset(q)
    else:
        raise KeyError(op)
    return None
