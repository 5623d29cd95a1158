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


def test_row_draws_equal_one_draw_per_row():
    """The stacked-shot path draws every shot's outcome at once; each row must
    give discrete_draw's index for its own uniform (same sequential sums)."""
    P = pkg()
    rng = np.random.default_rng(11)
    for d in (2, 4, 8, 32):
        probs = rng.random((300, d)) ** 3
        probs[::7, 0] = 0.0
        probs /= probs.sum(axis=1, keepdims=True) * (1 + 1e-15 * rng.standard_normal((300, 1)))
        u = rng.random(300)
        u[:5] = [0.0, 1 - 2 ** -53, probs[5, 0], 0.5, 1e-300]
        got = P.simulator.discrete_draws(probs, u)
        want = [P.simulator.discrete_draw(p, x) for p, x in zip(probs, u)]
        np.testing.assert_array_equal(got, want)
    assert P.simulator.discrete_draws(np.zeros((0, 2)), np.zeros(0)).shape == (0,)


def test_uniform_streams_are_per_shot_seeds():
    P = pkg()
    out = np.empty((5, 7))
    P._capi.check(P.lib().gbqv_uniforms_streams(2**64 - 2, 5, 7, out.ctypes.data_as(P._capi.dp)))
    for s in range(5):
        np.testing.assert_array_equal(out[s], P.uniforms((2**64 - 2 + s) % 2**64, 7))


def test_stacked_shot_group_sizes():
    P = pkg()
    sim = P.AerSimulator()
    g = sim._shot_group_bits
    assert g(10, 1, [1]) == 0                 # one shot: one state
    assert g(10, 50, [1]) == 6                # 64 states hold 50 shots
    assert g(10, 10**6, [1]) == 16            # at most 2^16 shots per group
    assert g(20, 10**6, [1]) == 8             # stack of at most 28 qubits
    assert g(12, 10**6, [10]) == 12           # 2^12 x 2^10 host probabilities
    assert g(16, 10**6, [3, 16]) == 11        # 2^11 x 2^16 device probabilities
    assert g(30, 4096, [30]) == 0


def test_conditioned_ops_become_matrices():
    """Conditioned gates, matrices and diagonals of up to 4 qubits are applied
    to the shots whose condition holds as one matrix; wider ones need the
    one-state loop."""
    P = pkg()
    items = []
    qc = P.QuantumCircuit(5, 2).measure(0, 0)
    nc_x = P.NativeCircuit(5, P.QuantumCircuit(5).x(3).data)
    d = np.exp(1j * np.arange(4))
    nc_d = P.NativeCircuit(5, P.QuantumCircuit(5).diagonal(d, [1, 4]).data)
    items = [("measure", qc.data[0], None), ("ops", nc_x, ([0], 1)), ("ops", nc_d, ([0], 0)),
             ("ops", nc_x, None)]
    mats = P.AerSimulator._conditioned_matrices(items)
    assert set(mats) == {1, 2}
    q, m = mats[1]
    assert q == [3]
    np.testing.assert_array_equal(m.reshape(2, 2, order="F"), [[0, 1], [1, 0]])
    q, m = mats[2]
    assert q == [1, 4]
    np.testing.assert_array_equal(m.reshape(4, 4, order="F"), np.diag(d))
    wide = P.NativeCircuit(5, P.QuantumCircuit(5).unitary(np.eye(32), [0, 1, 2, 3, 4]).data)
    assert P.AerSimulator._conditioned_matrices([("ops", wide, ([0], 1))]) is None
