"""Pins the oracle (oracle/oracle_qv.c via oracle/oracle.py) against golden
vectors produced by the reference's own QubitVector<double> /
DensityMatrix<double> / RngEngine (tests/golden/gen_golden.py).  CPU only."""
import numpy as np
import pytest

from golden_replay import GOLDEN, apply_case, load
from oracle import oracle as O

TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    O.build()


def _qv_cases():
    cases, arrays = load("qv")
    return [(i, c) for i, c in enumerate(cases)]


@pytest.mark.parametrize("i,case", _qv_cases(), ids=lambda x: x if isinstance(x, int) else x["op"])
def test_qv_case(i, case):
    _, arrays = load("qv")
    o = O.OracleQV(case["n"], arrays[f"in{i}"])
    res = apply_case(o, case, arrays, i)
    np.testing.assert_allclose(o.data, arrays[f"out{i}"], atol=TOL, rtol=0)
    if case["has_res"]:
        np.testing.assert_allclose(np.atleast_1d(res), arrays[f"res{i}"], atol=TOL, rtol=0)


def _dm_cases():
    cases, arrays = load("dm")
    return [(i, c) for i, c in enumerate(cases)]


class _DMAdapter(O.OracleDM):
    """DensityMatrix special gates expressed through the oracle surface."""

    def apply_x(self, q):
        self.apply_unitary_matrix([q], np.array([[0, 1], [1, 0]], dtype=complex))

    def apply_y(self, q):
        self.apply_unitary_matrix([q], np.array([[0, -1j], [1j, 0]]))

    def apply_phase(self, q, ph):
        self.apply_diagonal_unitary_matrix([q], [1, ph])

    def apply_cphase(self, a, b, ph):
        self.apply_diagonal_unitary_matrix([a, b], [1, 1, 1, ph])


@pytest.mark.parametrize("i,case", _dm_cases(), ids=lambda x: x if isinstance(x, int) else x["op"])
def test_dm_case(i, case):
    _, arrays = load("dm")
    o = _DMAdapter(case["n"])
    o.data[:] = arrays[f"in{i}"]
    res = apply_case(o, case, arrays, i)
    np.testing.assert_allclose(o.data, arrays[f"out{i}"], atol=TOL, rtol=0)
    if case["has_res"]:
        np.testing.assert_allclose(np.atleast_1d(res), arrays[f"res{i}"], atol=TOL, rtol=0)


def test_sample_measure_bit_exact():
    a = np.load(GOLDEN / "sample_cases.npz")
    for idx in range(3):
        psi = a[f"psi{idx}"]
        n = int(np.log2(psi.size))
        o = O.OracleQV(n, psi)
        r = O.uniforms(int(a[f"seed{idx}"][0]), a[f"rnds{idx}"].size)
        np.testing.assert_array_equal(r, a[f"rnds{idx}"])
        np.testing.assert_array_equal(o.sample_measure(r), a[f"samples{idx}"])
    d = O.OracleDM(4)
    d.data[:] = a["dm_rho"]
    np.testing.assert_array_equal(d.sample_measure(a["dm_rnds"]), a["dm_samples"])


def _edge_cases():
    import sys
    sys.path.insert(0, str(GOLDEN))
    from gen_sample_edges import CASES, state_of

    a = np.load(GOLDEN / "sample_edges.npz")
    for idx, (kind, n, isz, seed) in enumerate(CASES):
        assert list(a[f"case{idx}"]) == [0 if kind == "sv" else 1, n, isz, seed]
        yield kind, n, isz, state_of(kind, n, seed), a[f"rnds{idx}"], a[f"samples{idx}"]


def test_sample_measure_on_boundaries_bit_exact():
    """Uniforms exactly on the reference's cumulative sums, one step below
    them, in the rounding gaps after blocks and above the total
    (tests/golden/gen_sample_edges.py): the oracle returns the reference's
    samples, the walk's end (2^n) included."""
    for kind, n, isz, data, r, want in _edge_cases():
        o = O.OracleQV(n, data) if kind == "sv" else O.OracleDM(n, data)
        np.testing.assert_array_equal(o.sample_measure(r, index_size=isz), want, err_msg=f"{kind} {n} {isz}")


def test_rng_streams_bit_exact():
    a = np.load(GOLDEN / "rng_cases.npz")
    for key in a.files:
        seed = int(key.split("_", 1)[1])
        np.testing.assert_array_equal(O.uniforms(seed, 1000), a[key])


def test_unitary_builder():
    import json

    a = np.load(GOLDEN / "unitary_cases.npz")
    meta = json.loads((GOLDEN / "unitary_cases.json").read_text())
    k = meta["k"]
    u = O.OracleQV(2 * k, np.eye(1 << k, dtype=complex).reshape(-1, order="F"))
    for step, q in enumerate(meta["qubits"]):
        u.apply_matrix(q, a[f"u{step}"])
    np.testing.assert_allclose(u.data, a["result"], atol=TOL)


def test_noise_superops_are_cptp():
    for s in (O.depolarizing_superop(1e-3), O.amplitude_damping_superop(2e-3), O.depolarizing_superop(0.05, 2)):
        d = int(round(np.sqrt(s.shape[0])))
        # trace preservation: sum_i S[(i,i), :] = vec(I)
        tp = sum(s[i * d + i, :] for i in range(d))
        np.testing.assert_allclose(tp, np.eye(d).reshape(-1), atol=1e-14)


@pytest.mark.skipif(not O.RefQV.available(), reason="reference build (oracle/_ref) not present here")
def test_live_reference_random_circuit():
    """When the reference compiled here, run a 12-qubit random circuit through
    both and compare (beyond the stored fixtures)."""
    import ctypes as C

    lib = O.RefQV.lib()
    rng = np.random.default_rng(7)
    n = 12
    psi = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    psi /= np.linalg.norm(psi)
    h = lib.ref_qv_create(n, 1)
    p = np.ascontiguousarray(psi)
    lib.ref_qv_set(C.c_void_p(h), p.ctypes.data_as(C.c_void_p), C.c_uint64(p.size))
    o = O.OracleQV(n, psi)
    for _ in range(40):
        k = int(rng.integers(1, 5))
        q = [int(x) for x in rng.choice(n, size=k, replace=False)]
        z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
        u, _ = np.linalg.qr(z)
        m = np.ascontiguousarray(u.reshape(-1, order="F"))
        qa = np.ascontiguousarray(q, dtype=np.uint64)
        lib.ref_qv_apply_matrix(C.c_void_p(h), qa.ctypes.data_as(C.POINTER(C.c_uint64)), k,
                                m.ctypes.data_as(C.c_void_p))
        o.apply_matrix(q, m)
    out = np.empty(1 << n, dtype=np.complex128)
    lib.ref_qv_get(C.c_void_p(h), out.ctypes.data_as(C.c_void_p))
    lib.ref_qv_destroy(C.c_void_p(h))
    np.testing.assert_allclose(o.data, out, atol=1e-12)
