"""Host check of the complex128 digit-slice arithmetic used on the tensor
cores (qiskit-aer_gb300/csrc/gbqv_ozaki.h): split -> exact level sums ->
int64 recombination -> double, against __float128 matrix-vector products,
for 4- and 5-qubit gates (32 / 64 reals), including zeros, one dominant
entry and a 2^-60..2^2 dynamic range.  Bound: 1e-13 of (row max x column max).
Mode "signed" is the tcgen05 kernel's variant (signed digits, fp32 level
sums through the magic-add recombination, fast int64 -> double)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
@pytest.mark.parametrize("reals,trials,mode", [(32, 3000, "rounded"), (64, 1500, "rounded"),
                                               (32, 3000, "signed"), (64, 1500, "signed")])
def test_digit_slices_against_quad(tmp_path, reals, trials, mode):
    exe = tmp_path / "ozk"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "qiskit-aer_gb300" / "csrc"),
                           str(ROOT / "tests" / "ozaki_check.cpp"), "-o", str(exe), "-lquadmath"])
    out = subprocess.run([str(exe), str(reals), str(trials), mode], capture_output=True, text=True,
                         check=True).stdout
    rel, absolute = map(float, out.split())
    assert rel < 1e-13, out


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_fast_split_equals_generic_split(tmp_path):
    """The tcgen05 kernel's fast split (two 32-bit funnel shifts, used when
    every shift of a warp's reals is <= 31) gives the generic split's word bit
    for bit."""
    exe = tmp_path / "ozk"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "qiskit-aer_gb300" / "csrc"),
                           str(ROOT / "tests" / "ozaki_check.cpp"), "-o", str(exe), "-lquadmath"])
    out = subprocess.run([str(exe), "32", "400000", "near"], capture_output=True, text=True, check=True).stdout
    assert out.split()[0] == "0", out


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_converting_output_path_matches_integer_path(tmp_path):
    """The tcgen05 epilogue's converting output path (int64 -> double, then
    an exponent-field add) gives the integer normalisation's double to within
    one unit in the last place (plus one unit of v, which the integer path
    drops for negative v), for every sign and scale of the fast path."""
    exe = tmp_path / "ozk"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "qiskit-aer_gb300" / "csrc"),
                           str(ROOT / "tests" / "ozaki_check.cpp"), "-o", str(exe), "-lquadmath"])
    out = subprocess.run([str(exe), "32", "400000", "cvt"], capture_output=True, text=True, check=True).stdout
    bad, seen = map(int, out.split())
    assert bad == 0 and seen > 300000, out
