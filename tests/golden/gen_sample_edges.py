"""Generate tests/golden/sample_edges.npz from the reference itself: uniforms
placed exactly on the cumulative sums of QubitVector::sample_measure
(qubitvector.hpp:2148-2228) and one floating-point step below them, on
block edges, inside blocks, in the rounding gap between a block's walked
end and the next block's start, and at or above the state's total, with the
samples the reference's own QubitVector<double> / DensityMatrix<double>
(oracle/_ref/libaerref.so, built by ``make -C oracle ref``) returns for them.

The states come from tests/golden/edge_states.py (integer hashing), so the
fixture stores only the case parameters, the uniforms and the samples.

Usage:  python tests/golden/gen_sample_edges.py   (needs the reference sources)
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(HERE))
from edge_states import hash_state, reference_walk  # noqa: E402
from oracle import oracle as O  # noqa: E402

u64p = C.POINTER(C.c_uint64)
dp = C.POINTER(C.c_double)
vp = C.c_void_p

# (kind, qubits, index size, seed)
CASES = [("sv", 6, 10, 1), ("sv", 12, 10, 2), ("sv", 16, 10, 3), ("sv", 21, 10, 4), ("sv", 14, 4, 5),
         ("dm", 10, 10, 6), ("dm", 5, 10, 7)]


def state_of(kind, n, seed):
    """A statevector, or vec(rho) whose diagonal is |psi_k|^2 of a hash state
    (the sampler reads only the diagonal)."""
    if kind == "sv":
        return hash_state(1 << n, seed)
    rho = hash_state(1 << (2 * n), seed)
    sv = hash_state(1 << n, seed + 1000)
    rho[np.arange(1 << n) * ((1 << n) + 1)] = sv.real * sv.real + sv.imag * sv.imag
    return rho


def probs_of(kind, n, data):
    if kind == "sv":
        return data.real * data.real + data.imag * data.imag
    return data[np.arange(1 << n) * ((1 << n) + 1)].real.copy()


def edge_uniforms(prob, isz, rng):
    idxs, P, walk = reference_walk(prob, isz)
    down = lambda x: np.nextafter(x, -np.inf)
    picks = []
    if P is None:  # one walk from index 0
        ii = rng.choice(walk.size, min(walk.size, 200), replace=False)
        picks += [walk[ii], down(walk[ii])]
        total = walk[-1]
    else:
        nb, L = idxs.size, prob.size // idxs.size
        jj = rng.choice(nb, min(nb, 100), replace=False)
        picks += [P[jj + 1], down(P[jj + 1]), P[jj], np.nextafter(P[jj], np.inf)]
        ii = rng.choice(walk.size, 300, replace=False)
        picks += [walk[ii], down(walk[ii])]
        ends = walk[L - 1::L]
        gap = np.nonzero(ends < P[1:])[0]
        picks += [ends[gap[:50]], np.nextafter(ends[gap[:50]], np.inf)]
        over = np.nonzero(ends > P[1:])[0]
        picks += [P[over[:50] + 1], down(ends[over[:50]])]
        total = P[-1]
    picks += [np.array([0.0, total, np.nextafter(total, np.inf), down(total), 0.999999])]
    picks += [rng.uniform(0, total, 200)]
    r = np.concatenate(picks)
    return r[(r >= 0) & (r < 1)]


def main():
    O.build(ref=True)
    lib = O.RefQV.lib()
    rng = np.random.default_rng(2029)
    arrays = {}
    for idx, (kind, n, isz, seed) in enumerate(CASES):
        data = state_of(kind, n, seed)
        r = edge_uniforms(probs_of(kind, n, data), isz, rng)
        a = np.ascontiguousarray(data, dtype=np.complex128)
        out = np.empty(r.size, dtype=np.uint64)
        if kind == "sv":
            h = lib.ref_qv_create(n, 1)
            lib.ref_qv_set(vp(h), a.ctypes.data_as(vp), C.c_uint64(a.size))
            lib.ref_qv_set_sample_index_size(vp(h), isz)
            lib.ref_qv_sample_measure(vp(h), r.ctypes.data_as(dp), C.c_uint64(r.size), out.ctypes.data_as(u64p))
            lib.ref_qv_destroy(vp(h))
        else:
            h = lib.ref_dm_create(n, 1)
            lib.ref_dm_set(vp(h), a.ctypes.data_as(vp), C.c_uint64(a.size))
            lib.ref_dm_set_sample_index_size(vp(h), isz)
            lib.ref_dm_sample_measure(vp(h), r.ctypes.data_as(dp), C.c_uint64(r.size), out.ctypes.data_as(u64p))
            lib.ref_dm_destroy(vp(h))
        arrays[f"case{idx}"] = np.array([0 if kind == "sv" else 1, n, isz, seed], dtype=np.int64)
        arrays[f"rnds{idx}"] = r
        arrays[f"samples{idx}"] = out
        print(kind, n, isz, r.size, "uniforms;", int((out == (1 << n)).sum()), "at the end of the walk")
    np.savez_compressed(HERE / "sample_edges.npz", **arrays)


if __name__ == "__main__":
    main()
