"""Generate the golden fixtures in this folder from the reference itself.

Runs the reference's own QV::QubitVector<double>, QV::DensityMatrix<double>,
QV::UnitaryMatrix<double> and AER::RngEngine — compiled from the qiskit-aer
sources into oracle/_ref/libaerref.so by ``make -C oracle ref`` — on seeded
inputs and records inputs and outputs:

  qv_cases.npz / qv_cases.json   statevector ops and reductions, n = 6..7
  dm_cases.npz / dm_cases.json   density-matrix ops and reductions, n = 3
  sample_cases.npz               sample_measure (linear and two-level paths)
  rng_cases.npz                  RngEngine::rand(0,1) streams

Usage:  python tests/golden/gen_golden.py   (needs the reference sources)
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
from oracle import oracle as O  # noqa: E402

OUT = Path(__file__).resolve().parent
u64p = C.POINTER(C.c_uint64)
dp = C.POINTER(C.c_double)
vp = C.c_void_p


def u64(a):
    a = np.ascontiguousarray(a, dtype=np.uint64)
    return a, a.ctypes.data_as(u64p)


def c128(a):
    a = np.ascontiguousarray(a, dtype=np.complex128)
    return a, a.ctypes.data_as(vp)


def rand_state(rng, n):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def rand_unitary(rng, d):
    z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def rand_qubits(rng, n, k):
    return [int(x) for x in rng.choice(n, size=k, replace=False)]


def rand_label(rng, k, alphabet="IXYZ"):
    return "".join(rng.choice(list(alphabet), size=k))


def main():
    lib = O.RefQV.lib()
    rng = np.random.default_rng(20240611)
    arrays = {}
    cases = []

    def qv_case(n, op, args, inp, mutate):
        h = lib.ref_qv_create(n, 1)
        a, ap = c128(inp)
        lib.ref_qv_set(vp(h), ap, C.c_uint64(a.size))
        result = mutate(vp(h))
        if op.startswith("apply_"):
            result = None
        out = np.empty(1 << n, dtype=np.complex128)
        lib.ref_qv_get(vp(h), out.ctypes.data_as(vp))
        lib.ref_qv_destroy(vp(h))
        i = len(cases)
        arrays[f"in{i}"] = inp
        arrays[f"out{i}"] = out
        if result is not None:
            arrays[f"res{i}"] = np.atleast_1d(np.asarray(result))
        cases.append({"op": op, "n": n, **args, "has_res": result is not None})

    n = 7
    # dense matrices, k = 1..5, arbitrary qubit order
    for k in range(1, 6):
        for _ in range(3):
            q = rand_qubits(rng, n, k)
            m = rand_unitary(rng, 1 << k)
            arrays[f"mat{len(cases)}"] = m.reshape(-1, order="F")
            mm, mp = c128(m.reshape(-1, order="F"))
            qq, qp = u64(q)
            qv_case(n, "apply_matrix", {"qubits": q}, rand_state(rng, n),
                    lambda h, qp=qp, k=k, mp=mp: lib.ref_qv_apply_matrix(h, qp, k, mp))
    # single-qubit special forms of apply_matrix_1 / apply_diagonal_matrix_1
    specials = [
        np.array([[0, 1], [1, 0]]), np.array([[0, 0], [0.6 + 0.8j, 0]]), np.array([[0, 0.6 - 0.8j], [0, 0]]),
        np.array([[0, 1j], [0.5 + 0.5j, 0]]), np.array([[1, 0], [0, -1j]]), np.array([[1, 0], [0, 1j]]),
        np.array([[1, 0], [0, 0]]), np.array([[0, 0], [0, 1]]), np.array([[1, 0], [0, np.exp(0.3j)]]),
        np.array([[np.exp(0.7j), 0], [0, 1]]), np.array([[np.exp(0.7j), 0], [0, np.exp(-0.2j)]]),
    ]
    for m in specials:
        m = np.asarray(m, dtype=np.complex128)
        q = rand_qubits(rng, n, 1)
        arrays[f"mat{len(cases)}"] = m.reshape(-1, order="F")
        mm, mp = c128(m.reshape(-1, order="F"))
        qq, qp = u64(q)
        qv_case(n, "apply_matrix", {"qubits": q}, rand_state(rng, n),
                lambda h, qp=qp, mp=mp: lib.ref_qv_apply_matrix(h, qp, 1, mp))
    # diagonals (including entries equal to one)
    for k in range(1, 5):
        for _ in range(2):
            q = rand_qubits(rng, n, k)
            d = np.exp(1j * rng.uniform(0, 2 * np.pi, size=1 << k))
            d[0] = 1.0
            arrays[f"mat{len(cases)}"] = d
            dd, dp_ = c128(d)
            qq, qp = u64(q)
            qv_case(n, "apply_diagonal_matrix", {"qubits": q}, rand_state(rng, n),
                    lambda h, qp=qp, k=k, dp_=dp_: lib.ref_qv_apply_diagonal(h, qp, k, dp_))
    # multi-controlled gates
    for N in range(1, 5):
        q = rand_qubits(rng, n, N)
        qq, qp = u64(q)
        qv_case(n, "apply_mcx", {"qubits": q}, rand_state(rng, n), lambda h, qp=qp, N=N: lib.ref_qv_apply_mcx(h, qp, N))
        qv_case(n, "apply_mcy", {"qubits": q}, rand_state(rng, n), lambda h, qp=qp, N=N: lib.ref_qv_apply_mcy(h, qp, N))
        ph = np.exp(1j * rng.uniform(0, 2 * np.pi))
        qv_case(n, "apply_mcphase", {"qubits": q, "phase": [ph.real, ph.imag]}, rand_state(rng, n),
                lambda h, qp=qp, N=N, ph=ph: lib.ref_qv_apply_mcphase(h, qp, N, C.c_double(ph.real), C.c_double(ph.imag)))
        for m in (rand_unitary(rng, 2), np.diag(np.exp(1j * rng.uniform(0, 6, 2))), np.diag([1, np.exp(0.4j)])):
            m = np.asarray(m, dtype=np.complex128)
            arrays[f"mat{len(cases)}"] = m.reshape(-1, order="F")
            mm, mp = c128(m.reshape(-1, order="F"))
            qv_case(n, "apply_mcu", {"qubits": q}, rand_state(rng, n),
                    lambda h, qp=qp, N=N, mp=mp: lib.ref_qv_apply_mcu(h, qp, N, mp))
        if N >= 2:
            qv_case(n, "apply_mcswap", {"qubits": q}, rand_state(rng, n),
                    lambda h, qp=qp, N=N: lib.ref_qv_apply_mcswap(h, qp, N))
    # rotations
    for axis in range(7):
        k = 1 if axis < 3 else 2
        for nc in ((0, 1) if axis < 3 else (0,)):
            q = rand_qubits(rng, n, k + nc)
            th = float(rng.uniform(-np.pi, np.pi))
            qq, qp = u64(q)
            qv_case(n, "apply_rotation", {"qubits": q, "axis": axis, "theta": th}, rand_state(rng, n),
                    lambda h, qp=qp, q=q, axis=axis, th=th: lib.ref_qv_apply_rotation(h, qp, len(q), axis, C.c_double(th)))
    # Pauli application and expectation values
    for _ in range(8):
        k = int(rng.integers(1, 6))
        q = rand_qubits(rng, n, k)
        lab = rand_label(rng, k)
        c = np.exp(1j * rng.uniform(0, 6))
        qq, qp = u64(q)
        qv_case(n, "apply_pauli", {"qubits": q, "label": lab, "coeff": [c.real, c.imag]}, rand_state(rng, n),
                lambda h, qp=qp, k=k, lab=lab, c=c: lib.ref_qv_apply_pauli(h, qp, k, lab.encode(), C.c_double(c.real), C.c_double(c.imag)))
    for lab_alpha in ("IXYZ", "IZ", "XY"):
        for _ in range(5):
            k = int(rng.integers(1, 7))
            q = rand_qubits(rng, n, k)
            lab = rand_label(rng, k, lab_alpha)
            ph = np.exp(1j * rng.uniform(0, 6)) if rng.uniform() < 0.3 else 1.0 + 0j
            qq, qp = u64(q)
            qv_case(n, "expval_pauli", {"qubits": q, "label": lab, "phase": [ph.real, ph.imag]}, rand_state(rng, n),
                    lambda h, qp=qp, k=k, lab=lab, ph=ph: lib.ref_qv_expval_pauli(h, qp, k, lab.encode(), C.c_double(ph.real), C.c_double(ph.imag)))
    # permutation, multiplexer, multi-swaps
    for k in (1, 2, 3):
        q = rand_qubits(rng, n, k)
        perm = rng.permutation(1 << k)
        pairs = [(int(a), int(b)) for a, b in zip(range(1 << k), perm) if a < b][:3]
        pp, ppp = u64(np.array(pairs).reshape(-1))
        qq, qp = u64(q)
        qv_case(n, "apply_permutation_matrix", {"qubits": q, "pairs": pairs}, rand_state(rng, n),
                lambda h, qp=qp, k=k, ppp=ppp, pairs=pairs: lib.ref_qv_apply_permutation(h, qp, k, ppp, len(pairs)))
    for nc, nt in ((1, 1), (2, 1), (1, 2)):
        qs = rand_qubits(rng, n, nc + nt)
        ctrl, targ = qs[:nc], qs[nc:]
        blocks = [rand_unitary(rng, 1 << nt) for _ in range(1 << nc)]
        m = np.vstack(blocks)
        arrays[f"mat{len(cases)}"] = m.reshape(-1, order="F")
        mm, mp = c128(m.reshape(-1, order="F"))
        cc, cp = u64(ctrl)
        tt, tp = u64(targ)
        qv_case(n, "apply_multiplexer", {"controls": ctrl, "targets": targ}, rand_state(rng, n),
                lambda h, cp=cp, tp=tp, nc=nc, nt=nt, mp=mp: lib.ref_qv_apply_multiplexer(h, cp, nc, tp, nt, mp))
    for k in (2, 4):
        q = rand_qubits(rng, n, k)
        qq, qp = u64(q)
        qv_case(n, "apply_multi_swaps", {"qubits": q}, rand_state(rng, n),
                lambda h, qp=qp, k=k: lib.ref_qv_apply_multi_swaps(h, qp, k))
    # reductions
    for _ in range(2):
        qv_case(n, "norm", {}, rand_state(rng, n) * 1.3, lambda h: lib.ref_qv_norm(h))
    for k in (1, 2, 3, 5, 0):
        q = rand_qubits(rng, n, k) if k else []
        qq, qp = u64(q)
        out = np.empty(1 << (k if k else n))
        qv_case(n, "probabilities", {"qubits": q}, rand_state(rng, n),
                lambda h, qp=qp, k=k, out=out: (lib.ref_qv_probabilities(h, qp, k, out.ctypes.data_as(dp)), out.copy())[1])
    for k in (1, 2):
        q = rand_qubits(rng, n, k)
        m = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        arrays[f"mat{len(cases)}"] = m.reshape(-1, order="F")
        mm, mp = c128(m.reshape(-1, order="F"))
        qq, qp = u64(q)
        qv_case(n, "norm_matrix", {"qubits": q}, rand_state(rng, n),
                lambda h, qp=qp, k=k, mp=mp: lib.ref_qv_norm_matrix(h, qp, k, mp))

    np.savez_compressed(OUT / "qv_cases.npz", **arrays)
    (OUT / "qv_cases.json").write_text(json.dumps(cases, indent=0))
    print("qv cases", len(cases))

    # ---------------- density matrix ----------------
    arrays, cases = {}, []

    def dm_case(nq, op, args, psi, mutate):
        h = lib.ref_dm_create(nq, 1)
        # a mixed input: rho = sum_i w_i |psi_i><psi_i|
        rho = sum(w * np.kron(p.conj(), p) for w, p in zip([0.6, 0.3, 0.1], psi))
        a, ap = c128(rho)
        lib.ref_dm_set(vp(h), ap, C.c_uint64(a.size))
        result = mutate(vp(h))
        if op.startswith("apply_"):
            result = None
        out = np.empty(1 << (2 * nq), dtype=np.complex128)
        lib.ref_dm_get(vp(h), out.ctypes.data_as(vp))
        lib.ref_dm_destroy(vp(h))
        i = len(cases)
        arrays[f"in{i}"] = rho
        arrays[f"out{i}"] = out
        if result is not None:
            arrays[f"res{i}"] = np.atleast_1d(np.asarray(result))
        cases.append({"op": op, "n": nq, **args, "has_res": result is not None})

    nq = 3

    def psis():
        return [rand_state(rng, nq) for _ in range(3)]

    for k in (1, 2):
        q = rand_qubits(rng, nq, k)
        s = O.kraus_superop([rand_unitary(rng, 1 << k) * np.sqrt(0.7), rand_unitary(rng, 1 << k) * np.sqrt(0.3)])
        arrays[f"mat{len(cases)}"] = s.reshape(-1, order="F")
        mm, mp = c128(s.reshape(-1, order="F"))
        qq, qp = u64(q)
        dm_case(nq, "apply_superop_matrix", {"qubits": q}, psis(), lambda h, qp=qp, k=k, mp=mp: lib.ref_dm_apply_superop(h, qp, k, mp))
    for k in (1, 2, 3):
        q = rand_qubits(rng, nq, k)
        u = rand_unitary(rng, 1 << k)
        arrays[f"mat{len(cases)}"] = u.reshape(-1, order="F")
        mm, mp = c128(u.reshape(-1, order="F"))
        qq, qp = u64(q)
        dm_case(nq, "apply_unitary_matrix", {"qubits": q}, psis(), lambda h, qp=qp, k=k, mp=mp: lib.ref_dm_apply_unitary(h, qp, k, mp))
    for k in (1, 2):
        q = rand_qubits(rng, nq, k)
        d = np.exp(1j * rng.uniform(0, 6, size=1 << k))
        arrays[f"mat{len(cases)}"] = d
        dd, dp_ = c128(d)
        qq, qp = u64(q)
        dm_case(nq, "apply_diagonal_unitary_matrix", {"qubits": q}, psis(),
                lambda h, qp=qp, k=k, dp_=dp_: lib.ref_dm_apply_diagonal_unitary(h, qp, k, dp_))
    a, b, c = rand_qubits(rng, nq, 3)
    ph = np.exp(0.9j)
    dm_case(nq, "apply_cnot", {"qubits": [a, b]}, psis(), lambda h: lib.ref_dm_apply_cnot(h, C.c_uint64(a), C.c_uint64(b)))
    dm_case(nq, "apply_swap", {"qubits": [a, c]}, psis(), lambda h: lib.ref_dm_apply_swap(h, C.c_uint64(a), C.c_uint64(c)))
    dm_case(nq, "apply_x", {"qubits": [b]}, psis(), lambda h: lib.ref_dm_apply_x(h, C.c_uint64(b)))
    dm_case(nq, "apply_y", {"qubits": [c]}, psis(), lambda h: lib.ref_dm_apply_y(h, C.c_uint64(c)))
    dm_case(nq, "apply_phase", {"qubits": [a], "phase": [ph.real, ph.imag]}, psis(),
            lambda h: lib.ref_dm_apply_phase(h, C.c_uint64(a), C.c_double(ph.real), C.c_double(ph.imag)))
    dm_case(nq, "apply_cphase", {"qubits": [b, c], "phase": [ph.real, ph.imag]}, psis(),
            lambda h: lib.ref_dm_apply_cphase(h, C.c_uint64(b), C.c_uint64(c), C.c_double(ph.real), C.c_double(ph.imag)))
    dm_case(nq, "apply_toffoli", {"qubits": [a, b, c]}, psis(),
            lambda h: lib.ref_dm_apply_toffoli(h, C.c_uint64(a), C.c_uint64(b), C.c_uint64(c)))
    for k in (1, 2):
        q = rand_qubits(rng, nq, k)
        qq, qp = u64(q)
        dm_case(nq, "apply_reset", {"qubits": q}, psis(), lambda h, qp=qp, k=k: lib.ref_dm_apply_reset(h, qp, k))
    for _ in range(8):
        k = int(rng.integers(1, 4))
        q = rand_qubits(rng, nq, k)
        lab = rand_label(rng, k)
        qq, qp = u64(q)
        dm_case(nq, "expval_pauli", {"qubits": q, "label": lab}, psis(),
                lambda h, qp=qp, k=k, lab=lab: lib.ref_dm_expval_pauli(h, qp, k, lab.encode()))
    for k in (1, 2, 0):
        q = rand_qubits(rng, nq, k) if k else []
        qq, qp = u64(q)
        out = np.empty(1 << (k if k else nq))
        dm_case(nq, "probabilities", {"qubits": q}, psis(),
                lambda h, qp=qp, k=k, out=out: (lib.ref_dm_probabilities(h, qp, k, out.ctypes.data_as(dp)), out.copy())[1])
    np.savez_compressed(OUT / "dm_cases.npz", **arrays)
    (OUT / "dm_cases.json").write_text(json.dumps(cases, indent=0))
    print("dm cases", len(cases))

    # ---------------- sampling and RNG ----------------
    arrays = {}
    for idx, (n, shots, seed) in enumerate(((5, 500, 11), (12, 2000, 12), (13, 1000, 13))):
        psi = rand_state(rng, n)
        # concentrate mass so that both the block walk and the tail matter
        psi[: 1 << (n - 1)] *= 0.3
        psi /= np.linalg.norm(psi)
        r = np.empty(shots)
        lib.ref_uniforms(C.c_uint64(seed), C.c_uint64(shots), r.ctypes.data_as(dp))
        h = lib.ref_qv_create(n, 1)
        a, ap = c128(psi)
        lib.ref_qv_set(vp(h), ap, C.c_uint64(a.size))
        out = np.empty(shots, dtype=np.uint64)
        lib.ref_qv_sample_measure(vp(h), r.ctypes.data_as(dp), C.c_uint64(shots), out.ctypes.data_as(u64p))
        lib.ref_qv_destroy(vp(h))
        arrays[f"psi{idx}"] = psi
        arrays[f"rnds{idx}"] = r
        arrays[f"samples{idx}"] = out
        arrays[f"seed{idx}"] = np.array([seed])
    # density-matrix sampling
    nq = 4
    psi = rand_state(rng, nq)
    rho = np.kron(psi.conj(), psi)
    r = np.empty(300)
    lib.ref_uniforms(C.c_uint64(99), C.c_uint64(300), r.ctypes.data_as(dp))
    h = lib.ref_dm_create(nq, 1)
    a, ap = c128(rho)
    lib.ref_dm_set(vp(h), ap, C.c_uint64(a.size))
    out = np.empty(300, dtype=np.uint64)
    lib.ref_dm_sample_measure(vp(h), r.ctypes.data_as(dp), C.c_uint64(300), out.ctypes.data_as(u64p))
    lib.ref_dm_destroy(vp(h))
    arrays["dm_rho"], arrays["dm_rnds"], arrays["dm_samples"] = rho, r, out
    np.savez_compressed(OUT / "sample_cases.npz", **arrays)

    arrays = {}
    for seed in (0, 1, 9000, 2**40 + 7):
        r = np.empty(1000)
        lib.ref_uniforms(C.c_uint64(seed), C.c_uint64(1000), r.ctypes.data_as(dp))
        arrays[f"seed_{seed}"] = r
    np.savez_compressed(OUT / "rng_cases.npz", **arrays)

    # ---------------- fused-matrix builder (UnitaryMatrix) ----------------
    arrays = {}
    k = 3
    h = lib.ref_um_create(k)
    seq = []
    for step in range(6):
        kk = int(rng.integers(1, 3))
        q = rand_qubits(rng, k, kk)
        u = rand_unitary(rng, 1 << kk)
        qq, qp = u64(q)
        mm, mp = c128(u.reshape(-1, order="F"))
        lib.ref_um_apply_matrix(vp(h), qp, kk, mp)
        arrays[f"u{step}"] = u.reshape(-1, order="F")
        seq.append(q)
    out = np.empty(1 << (2 * k), dtype=np.complex128)
    lib.ref_um_get(vp(h), out.ctypes.data_as(vp))
    lib.ref_um_destroy(vp(h))
    arrays["result"] = out
    np.savez_compressed(OUT / "unitary_cases.npz", **arrays)
    (OUT / "unitary_cases.json").write_text(json.dumps({"k": k, "qubits": seq}))
    print("done")


if __name__ == "__main__":
    main()
