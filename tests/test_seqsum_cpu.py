"""Host check of the sampler's grid-step sums (qiskit-aer_gb300/csrc/
gbqv_seqsum.h): steps of 256 terms advanced by an integer sum on the running
sum's ulp grid, or term by term where a step ties, leaves its binade or
starts from zero, give the reference's in-order double additions
(qubitvector.hpp:2184-2220) bit for bit after every step, over probability
distributions that include ties, binade crossings, zeros, subnormals and
negative or infinite terms; ties are decided by prefix parities, not term
by term.  The warp routine that adds 32 terms at a time (one per lane) and
the chain kernel's 32-step batches are replayed lane by lane and checked
after every term and every step."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _exe(tmp_path):
    exe = tmp_path / "seqsum"
    subprocess.check_call(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "qiskit-aer_gb300" / "csrc"),
                           str(ROOT / "tests" / "seqsum_check.cpp"), "-o", str(exe)])
    return exe


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_grid_steps_equal_sequential_sums(tmp_path):
    out = subprocess.run([str(_exe(tmp_path)), "65536", "66"], capture_output=True, text=True,
                         check=True).stdout
    bad, steps, slow, lanes_bad, batch_bad = map(int, out.split())
    assert bad == 0 and lanes_bad == 0 and batch_bad == 0 and steps == 66 * 3 * 256, out
    # most steps take the grid path (the adversarial cases force the rest)
    assert slow < steps // 4, out


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_word_form_equals_grid_units(tmp_path):
    out = subprocess.run([str(_exe(tmp_path)), "words", "400000"], capture_output=True, text=True,
                         check=True).stdout
    assert out.split() == ["0"], out


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_integer_add_equals_double_add(tmp_path):
    """The probabilities pass adds fl(re^2) + fl(im^2) in integer arithmetic
    (seq::add_nonneg): bit for bit the double addition, ties, exponent gaps,
    zeros and overflow included."""
    out = subprocess.run([str(_exe(tmp_path)), "add", "2000000"], capture_output=True, text=True,
                         check=True).stdout
    assert out.split() == ["0"], out
