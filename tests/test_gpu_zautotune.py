"""Schedule autotuner on the GPU: an autotuned AerSimulator run times the
three execution forms of its op list, keeps one, gives the oracle's state
and reuses the choice on the next run of the same structure; a tuned batch
team setting gives the default setting's energies and gradients."""
import json

import numpy as np
import pytest

from _pkg import pkg
from test_gpu_runs import haar, oracle_of, random_small_ops

pytestmark = pytest.mark.gpu


def test_autotuned_statevector_run(tmp_path):
    P = pkg()
    n = 13  # below the fusion threshold: the small ops reach the cache-blocked runs as they are
    rng = np.random.default_rng(77)
    qc = P.QuantumCircuit(n)
    for q in range(n):
        qc.unitary(haar(rng, 2), [q])
    qc.data += random_small_ops(P, n, 150, rng).data
    want = oracle_of(qc)
    qc.save_statevector()
    qc.measure_all()
    path = tmp_path / "tune.json"
    sim = P.AerSimulator(autotune=True, autotune_cache=str(path))
    res = sim.run(qc, shots=256, seed_simulator=5)
    mode = res.metadata()["autotune"]["blocking"]
    assert mode in (0, 1, 2)
    if mode != 0:
        assert res.metadata()["autotune"]["tile_qubits"] in (0, 11, 10)
    np.testing.assert_allclose(res.get_statevector(), want, atol=1e-12)
    assert sum(res.get_counts().values()) == 256
    entries = json.loads(path.read_text())["entries"]
    assert len(entries) == (1 if mode == 0 else 2)
    entry = next(v for k, v in entries.items() if k.startswith("execute"))
    assert entry["choice"] == str(mode)
    assert set(entry["ms"]) == {"0", "1", "2"} and all(v > 0 for v in entry["ms"].values())
    timed = sim.tuner().measurements
    res2 = sim.run(qc, shots=256, seed_simulator=5)
    assert sim.tuner().measurements == timed  # same structure: the cached choice, no timing
    assert res2.metadata()["autotune"]["blocking"] == mode
    np.testing.assert_allclose(res2.get_statevector(), want, atol=1e-12)


def test_tuned_batch_team_setting(tmp_path):
    P = pkg()
    B, T = P.batched, P.autotune
    insts = B.config5_instances(8, seed=9, qmin=11, qmax=14, dmin=2, dmax=4, tmin=5, tmax=10, shots=64)
    tuner = T.Autotuner(str(tmp_path / "batch.json"), warmup=1, repeats=1)
    candidates = [(64, 0.0), (0, 0.0)]
    choice = T.tune_batch(insts, "double", True, tuner, candidates=candidates)
    assert choice in candidates
    entry = next(iter(tuner.entries.values()))
    assert len(entry["ms"]) == 2 and not entry["errors"]
    out = []
    for teams in (choice, None):
        b = T.build_batch(insts, "double", teams)
        try:
            b.run(want_grad=True)
            out.append([b.result(i) for i in range(len(insts))])
        finally:
            b.close()
    for (e0, g0, s0, _), (e1, g1, s1, _) in zip(*out):
        assert abs(e0 - e1) < 1e-12 * max(1.0, abs(e0))
        np.testing.assert_allclose(g0, g1, atol=1e-11)
        np.testing.assert_array_equal(s0, s1)


@pytest.mark.parametrize("precision,tiles,tol", [("double", (0, 11, 10), 1e-12), ("single", (0, 12, 11), 2e-5)])
def test_every_run_tile_gives_the_oracle_state(precision, tiles, tol):
    """The tile sizes the tuner chooses between (gbqv_set_run_tile_qubits)
    change only the schedule: each gives the oracle's state."""
    P = pkg()
    n = 15
    rng = np.random.default_rng(31)
    qc = random_small_ops(P, n, 200, rng)
    want = oracle_of(qc)
    nc = P.NativeCircuit(n, qc.data)
    for m in tiles:
        with P.QubitVector(n, precision) as st:
            assert st._L.gbqv_set_run_tile_qubits(st.handle, m) == 0
            st.initialize()
            assert st._L.gbqv_execute(st.handle, nc.handle) == 0
            np.testing.assert_allclose(st.copy_to_vector(), want, atol=tol, err_msg=f"tile {m}")
