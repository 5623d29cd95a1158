"""The per-shot executor's outcome draw (simulator.discrete_draw) against
libstdc++'s std::discrete_distribution on the same std::mt19937_64 stream
(RngEngine::rand_int, framework/rng.hpp:94-96), including unnormalised
weights, zero weights and weights that do not sum to one exactly."""
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from _pkg import pkg

ROOT = Path(__file__).resolve().parents[1]


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
@pytest.mark.parametrize("weights", [
    [0.5, 0.5],
    [0.1, 0.2, 0.3, 0.4],
    [0.0, 0.25, 0.0, 0.75],
    [1e-300, 1.0],
    [0.3333333333333333, 0.3333333333333333, 0.33333333333333337],
    list(np.random.default_rng(5).random(16)),
])
def test_discrete_draw_matches_libstdcxx(tmp_path, weights):
    exe = tmp_path / "dc"
    subprocess.check_call(["g++", "-O2", "-std=c++17", str(ROOT / "tests" / "discrete_check.cpp"), "-o", str(exe)])
    P = pkg()
    for seed in (0, 7, 2024, 123456789):
        out = subprocess.run([str(exe), str(seed), "200"] + [repr(float(w)) for w in weights],
                             capture_output=True, text=True, check=True).stdout.split("\n")
        for line in filter(None, out):
            u, k = line.split()
            assert P.simulator.discrete_draw(weights, float(u)) == int(k)


def test_needs_shots_rules():
    P = pkg()
    qc = P.QuantumCircuit(2, 2).h(0).measure(0, 0).measure(1, 1)
    assert not qc.needs_shots()
    assert P.QuantumCircuit(2, 2).h(0).measure(0, 0).x(1).needs_shots()
    assert P.QuantumCircuit(2, 1).h(0).reset(0).needs_shots("statevector")
    assert not P.QuantumCircuit(2, 1).h(0).reset(0).needs_shots("density_matrix")
    assert P.QuantumCircuit(2, 1).measure(0, 0).x(1).c_if(0, 1).needs_shots()
