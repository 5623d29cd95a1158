"""Engine (libgbqv.so on the GPU, through the C ABI) against the golden
vectors produced by the reference's own QubitVector<double> /
DensityMatrix<double> (tests/golden).  complex128: 1e-12 absolute;
complex64: 2e-6 absolute (float32 arithmetic on unit-norm states)."""
import numpy as np
import pytest

from _pkg import ROOT, pkg
from golden_replay import GOLDEN, apply_case, load

pytestmark = pytest.mark.gpu
TOL = {"double": 1e-12, "single": 2e-6}


def _qv():
    cases, _ = load("qv")
    return list(enumerate(cases))


def _dm():
    cases, _ = load("dm")
    return list(enumerate(cases))


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("i,case", _qv(), ids=lambda x: x if isinstance(x, int) else x["op"])
def test_qv_golden(precision, i, case):
    P = pkg()
    _, arrays = load("qv")
    with P.QubitVector(case["n"], precision) as qv:
        qv.initialize_from_vector(arrays[f"in{i}"])
        res = apply_case(qv, case, arrays, i)
        out = qv.copy_to_vector()
    np.testing.assert_allclose(out, arrays[f"out{i}"], atol=TOL[precision], rtol=0)
    if case["has_res"]:
        np.testing.assert_allclose(np.atleast_1d(res), arrays[f"res{i}"], atol=TOL[precision] * 8, rtol=0)


@pytest.mark.parametrize("precision", ["double", "single"])
@pytest.mark.parametrize("i,case", _dm(), ids=lambda x: x if isinstance(x, int) else x["op"])
def test_dm_golden(precision, i, case):
    P = pkg()
    _, arrays = load("dm")
    with P.DensityMatrix(case["n"], precision) as dm:
        dm.initialize_from_vector(arrays[f"in{i}"])
        res = apply_case(dm, case, arrays, i)
        out = dm.copy_to_vector()
    np.testing.assert_allclose(out, arrays[f"out{i}"], atol=TOL[precision], rtol=0)
    if case["has_res"]:
        np.testing.assert_allclose(np.atleast_1d(res), arrays[f"res{i}"], atol=TOL[precision] * 8, rtol=0)


def test_sampling_golden_bit_exact():
    P = pkg()
    a = np.load(GOLDEN / "sample_cases.npz")
    for idx in range(3):
        psi = a[f"psi{idx}"]
        n = int(np.log2(psi.size))
        with P.QubitVector(n) as qv:
            qv.initialize_from_vector(psi)
            np.testing.assert_array_equal(qv.sample_measure(a[f"rnds{idx}"]), a[f"samples{idx}"])
    with P.DensityMatrix(4) as dm:
        dm.initialize_from_vector(a["dm_rho"])
        np.testing.assert_array_equal(dm.sample_measure(a["dm_rnds"]), a["dm_samples"])


def test_sampling_boundaries_bit_exact():
    """The uniforms of tests/golden/sample_edges.npz (on and one step below
    the reference's cumulative sums, in the gaps after blocks, above the
    total): the engine returns the reference's samples, through the
    statevector and density-matrix handles, with the reference's block
    count (index size) set where it differs from 10."""
    import sys
    sys.path.insert(0, str(GOLDEN))
    from gen_sample_edges import CASES, state_of

    P = pkg()
    a = np.load(GOLDEN / "sample_edges.npz")
    for idx, (kind, n, isz, seed) in enumerate(CASES):
        data = state_of(kind, n, seed)
        st = P.QubitVector(n) if kind == "sv" else P.DensityMatrix(n)
        with st:
            st.initialize_from_vector(data)
            st.set_sample_measure_index_size(isz)
            got = st.sample_measure(a[f"rnds{idx}"])
        np.testing.assert_array_equal(got, a[f"samples{idx}"], err_msg=f"{kind} {n} {isz}")
