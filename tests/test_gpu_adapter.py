"""The C++ QubitVector adapter (include/gbqv_qubitvector.hpp), compiled with
g++ into tests/adapter_driver.cpp, driven on the GPU and compared with the
oracle: gates of every kind, initialize_component, probabilities /
probability / norm / norm(qubits, mat) / norm_diagonal / expval_pauli /
vector_ket / sample_measure / the final state (statevector, complex128 and
complex64), and the density-matrix members (unitary, superoperator, reset)."""
import numpy as np
import pytest

from _pkg import pkg
from adapter_build import build_driver, run_driver
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def driver(tmp_path_factory):
    return build_driver(tmp_path_factory.mktemp("adapter"))


def _fmt_c(values):
    return " ".join(f"{float(z.real):.17g} {float(z.imag):.17g}"
                    for z in np.asarray(values, dtype=np.complex128).reshape(-1))


def _unitary(rng, k):
    z = rng.normal(size=(1 << k, 1 << k)) + 1j * rng.normal(size=(1 << k, 1 << k))
    q, r = np.linalg.qr(z)
    return q * (np.diag(r) / np.abs(np.diag(r)))


def _parse(out):
    res = []
    for line in out.strip().splitlines():
        head, *rest = line.split()
        res.append((head, rest))
    return res


def _sv_script(rng, n):
    """Ops on qubits 0..n-3 (the top two stay |0> for initialize_component),
    with the oracle applying the same."""
    o = O.OracleQV(n)
    lines = []
    low = n - 2
    for _ in range(12):
        k = int(rng.integers(1, 5))
        q = [int(x) for x in rng.choice(low, k, replace=False)]
        u = _unitary(rng, k)
        lines.append(f"matrix {k} {' '.join(map(str, q))} {_fmt_c(u.reshape(-1, order='F'))}")
        o.apply_matrix(q, u.reshape(-1, order="F"))
        d = np.exp(1j * rng.uniform(0, 2 * np.pi, 4))
        q = [int(x) for x in rng.choice(low, 2, replace=False)]
        lines.append(f"diag 2 {' '.join(map(str, q))} {_fmt_c(d)}")
        o.apply_diagonal_matrix(q, d)
    q = [int(x) for x in rng.choice(low, 3, replace=False)]
    lines.append(f"mcx 3 {' '.join(map(str, q))}")
    o.apply_mcx(q)
    m = _unitary(rng, 1).reshape(-1, order="F")
    q = [int(x) for x in rng.choice(low, 2, replace=False)]
    lines.append(f"mcu 2 {' '.join(map(str, q))} {_fmt_c(m)}")
    o.apply_mcu(q, m)
    lines.append(f"rotation 2 1 3 5 0.731")  # rzz
    o.apply_rotation([1, 3], 5, 0.731)
    lines.append(f"rotation 1 2 1 -1.25")  # ry
    o.apply_rotation([2], 1, -1.25)
    lines.append("pauli 3 0 2 4 XYZ 0 1")
    o.apply_pauli([0, 2, 4], "XYZ", 1j)
    comp = rng.normal(size=4) + 1j * rng.normal(size=4)
    comp /= np.linalg.norm(comp)
    top = [n - 1, n - 2]
    lines.append(f"component 2 {top[0]} {top[1]} {_fmt_c(comp)}")
    cm = np.zeros((4, 4), dtype=np.complex128)
    cm[:, 0] = comp
    o.apply_matrix(top, cm.reshape(-1, order="F"))
    return lines, o


@pytest.mark.parametrize("precision,tol", [("c128", 1e-12), ("c64", 2e-6)])
def test_adapter_statevector_vs_oracle(driver, precision, tol):
    rng = np.random.default_rng(77 if precision == "c128" else 78)
    n = 10
    lines, o = _sv_script(rng, n)
    pq = [3, 9, 0]
    nm = rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))
    nq = [0, 4, 5, 6, 8, 9]
    dg = rng.normal(size=8) + 1j * rng.normal(size=8)
    u = O.uniforms(5, 64)
    lines += [f"probs 3 {' '.join(map(str, pq))}", "expval 4 0 3 7 9 ZXYI", "probability 517", "norm",
              f"normmat 6 {' '.join(map(str, nq))} {_fmt_c(nm.reshape(-1, order='F'))}",
              f"normdiag 3 1 2 8 {_fmt_c(dg)}", "ket 1e-3",
              f"sample 64 {' '.join(repr(float(x)) for x in u)}", "state", "end"]
    rc, out, err = run_driver(driver, f"sv {precision} {n}\n" + "\n".join(lines) + "\n")
    assert rc == 0, (rc, out[-2000:], err)
    res = dict(_parse(out))
    np.testing.assert_allclose(np.array(res["probs"], float), o.probabilities(pq), atol=tol)
    assert abs(float(res["expval"][0]) - o.expval_pauli([0, 3, 7, 9], "ZXYI")) < tol
    assert abs(float(res["probability"][0]) - abs(o.data[517]) ** 2) < tol
    norms = [float(v[0]) for h, v in _parse(out) if h == "norm"]
    assert abs(norms[0] - o.norm()) < tol * 10
    assert abs(norms[1] - o.norm_matrix(nq, nm.reshape(-1, order="F"))) < tol * 1e3
    dense = np.diag(dg).reshape(-1, order="F")
    assert abs(norms[2] - o.norm_matrix([1, 2, 8], dense)) < tol * 100
    sv = np.array(res["state"], float).reshape(-1, 2) @ np.array([1, 1j])
    np.testing.assert_allclose(sv, o.data, atol=tol)
    ket = res["ket"]
    got = {ket[i]: complex(float(ket[i + 1]), float(ket[i + 2])) for i in range(0, len(ket), 3)}
    want = {}
    for k, z in enumerate(o.data):
        zc = complex(z.real if abs(z.real) >= 1e-3 else 0.0, z.imag if abs(z.imag) >= 1e-3 else 0.0)
        if abs(zc) > 1e-3:
            want[f"0x{k:x}"] = zc
    # entries within float error of the cut-off may fall either side in complex64
    near = {f"0x{k:x}" for k, z in enumerate(o.data)
            if min(abs(abs(z.real) - 1e-3), abs(abs(z.imag) - 1e-3), abs(abs(z) - 1e-3)) < 1e-5}
    assert set(got) - near == set(want) - near
    for key in set(got) & set(want) - near:
        assert abs(got[key] - want[key]) < tol * 10
    if precision == "c128":
        np.testing.assert_array_equal(np.array(res["sample"], np.uint64), o.sample_measure(u))


def test_adapter_density_matrix_vs_oracle(driver):
    rng = np.random.default_rng(91)
    n = 5
    o = O.OracleDM(n)
    lines = []
    for _ in range(6):
        k = int(rng.integers(1, 3))
        q = [int(x) for x in rng.choice(n, k, replace=False)]
        u = _unitary(rng, k).reshape(-1, order="F")
        lines.append(f"matrix {k} {' '.join(map(str, q))} {_fmt_c(u)}")
        o.apply_unitary_matrix(q, u)
    sop = O.depolarizing_superop(0.1, 1)
    lines.append(f"superop 1 2 {_fmt_c(sop.reshape(-1, order='F'))}")
    o.apply_superop_matrix([2], sop.reshape(-1, order="F"))
    lines.append("reset 1 4")
    o.apply_reset([4])
    lines += ["probs 2 4 0", "expval 3 0 1 3 XZY", "probability 6", "norm", "state", "end"]
    rc, out, err = run_driver(driver, f"dm c128 {n}\n" + "\n".join(lines) + "\n")
    assert rc == 0, (rc, out[-2000:], err)
    res = dict(_parse(out))
    np.testing.assert_allclose(np.array(res["probs"], float), o.probabilities([4, 0]), atol=1e-12)
    assert abs(float(res["expval"][0]) - o.expval_pauli([0, 1, 3], "XZY")) < 1e-12
    assert abs(float(res["probability"][0]) - o.data[6 * ((1 << n) + 1)].real) < 1e-12
    assert abs(float(res["norm"][0]) - o.norm()) < 1e-12
    vec = np.array(res["state"], float).reshape(-1, 2) @ np.array([1, 1j])
    np.testing.assert_allclose(vec, o.data, atol=1e-12)


def test_adapter_errors_are_exceptions(driver):
    """A bad Pauli letter is std::invalid_argument (qubitvector.hpp:2266-2268),
    reported by the driver without crashing."""
    rc, out, _ = run_driver(driver, "sv c128 4\nexpval 1 0 Q\nend\n")
    assert rc == 3 and "invalid_argument: Invalid Pauli" in out, out
