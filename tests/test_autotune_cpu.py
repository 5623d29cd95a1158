"""Schedule autotuner (qiskit-aer_gb300/autotune.py) on the host: selection by
median device time with ties to the default, the cache and its file, the
workload keys, and the tuning loops of gbqv_execute and gbqv_batch_run
driven through fakes of the state, the library and the device timer."""
import json

import numpy as np
import pytest

from _pkg import pkg


def tuner_mod():
    return pkg().autotune


def test_select_takes_lowest_median_and_ties_keep_the_earlier():
    T = tuner_mod()
    t = T.Autotuner(warmup=1, repeats=3)
    # candidate "b" has one slow outlier: its median (2.0) still wins over "a" (3.0)
    series = {"a": iter([9.0, 3.0, 3.0, 3.0]), "b": iter([9.0, 2.0, 50.0, 2.0]), "c": iter([1.0, 4.0, 4.0, 4.0])}
    assert t.select("k1", ["a", "b", "c"], lambda c: next(series[c])) == "b"
    assert t.measurements == 12
    entry = t.entries["k1"]
    assert entry["ms"] == {'"a"': 3.0, '"b"': 2.0, '"c"': 4.0}
    # equal medians: the first candidate (the engine's default) stays
    assert t.select("k2", [1, 2, 0], lambda c: 5.0) == 1


def test_cached_choice_is_reused_without_timing():
    T = tuner_mod()
    t = T.Autotuner(warmup=0, repeats=1)
    assert t.select(("execute", "dev", 20), [1, 2, 0], lambda c: {1: 3.0, 2: 1.0, 0: 2.0}[c]) == 2
    n = t.measurements

    def boom(c):
        raise AssertionError("a cached key is timed again")

    assert t.select(("execute", "dev", 20), [1, 2, 0], boom) == 2
    assert t.measurements == n
    # a cached choice outside the new candidate list is not used: the key is timed again
    assert t.select(("execute", "dev", 20), [1, 0], lambda c: {1: 3.0, 0: 2.0}[c]) == 0


def test_single_candidate_and_empty_list():
    T = tuner_mod()
    t = T.Autotuner()
    assert t.select("k", [7], lambda c: pytest.fail("one candidate needs no timing")) == 7
    with pytest.raises(ValueError):
        t.select("k", [], lambda c: 1.0)
    with pytest.raises(ValueError):
        T.Autotuner(repeats=0)


def test_failing_candidates_are_skipped_and_recorded():
    P = pkg()
    T = P.autotune
    t = T.Autotuner(warmup=0, repeats=2)

    def measure(c):
        if c == 2:
            raise P.GBQVError(7, "pipeline wait gave up")
        return {1: 4.0, 0: 6.0}[c]

    assert t.select("k", [2, 1, 0], measure) == 1
    assert "gave up" in t.entries["k"]["errors"]["2"]
    assert "2" not in t.entries["k"]["ms"]

    def all_fail(c):
        raise P.GBQVError(7, f"candidate {c} failed")

    with pytest.raises(P.GBQVError, match="candidate 0 failed"):
        t.select("k-all", [1, 0], all_fail)
    assert "k-all" not in t.entries
    # other exceptions are not swallowed
    with pytest.raises(ZeroDivisionError):
        t.select("k-bug", [1, 0], lambda c: 1 / 0)


def test_cache_file_round_trip(tmp_path, monkeypatch):
    T = tuner_mod()
    path = tmp_path / "tune.json"
    t = T.Autotuner(str(path), warmup=0, repeats=1)
    assert t.select(("batch", "dev", "double", 1, "sig"), [(64, 0.5), (0, 0.5)],
                    lambda c: {(64, 0.5): 2.0, (0, 0.5): 1.0}[c]) == (0, 0.5)
    data = json.loads(path.read_text())
    assert data["version"] == 1 and len(data["entries"]) == 1
    # a new tuner on the same file answers without timing; the candidate comes back as given
    t2 = T.Autotuner(str(path))
    got = t2.select(("batch", "dev", "double", 1, "sig"), [(64, 0.5), (0, 0.5)], lambda c: pytest.fail("timed"))
    assert got == (0, 0.5) and isinstance(got, tuple)
    # the environment variable names the file when no path is passed
    monkeypatch.setenv("GBQV_TUNE_CACHE", str(path))
    assert T.Autotuner().lookup(("batch", "dev", "double", 1, "sig"), [(0, 0.5)]) == (0, 0.5)
    bad = tmp_path / "bad.json"
    bad.write_text("[1, 2]")
    with pytest.raises(ValueError):
        T.Autotuner(str(bad))


def test_circuit_signature_is_structure_only():
    P = pkg()
    T = P.autotune
    rng = np.random.default_rng(3)

    def circ(mats, qubits):
        qc = P.QuantumCircuit(4)
        for m, q in zip(mats, qubits):
            qc.unitary(m, q)
        qc.h(0).cx(0, 3)
        return P.NativeCircuit(4, qc.data)

    def rand_u(d):
        q, _ = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
        return q

    a = circ([rand_u(4), rand_u(2)], [[0, 1], [2]])
    b = circ([rand_u(4), rand_u(2)], [[0, 1], [2]])
    c = circ([rand_u(4), rand_u(2)], [[1, 2], [2]])
    assert T.circuit_signature([a]) == T.circuit_signature([b])
    assert T.circuit_signature([a]) != T.circuit_signature([c])
    # segment boundaries are part of the structure
    assert T.circuit_signature([a, b]) != T.circuit_signature([a])


class FakeLib:
    """Records gbqv_set_blocking / gbqv_execute calls; every call succeeds."""

    def __init__(self):
        self.mode = 1
        self.calls = []

    def gbqv_set_blocking(self, h, mode):
        self.mode = mode
        self.calls.append(("blocking", mode))
        return 0

    def gbqv_execute(self, h, c):
        self.calls.append(("execute", self.mode, c))
        return 0

    def gbqv_set_run_tile_qubits(self, h, m):
        self.tile = m
        self.calls.append(("tile", m))
        return 0


class FakeState:
    def __init__(self, kind=None, n=4):
        P = pkg()
        self._L = FakeLib()
        self.n = n
        self.handle = object()
        self.precision = "double"
        self._kind = P._capi.STATEVECTOR if kind is None else kind
        self.inits = 0

    def num_qubits(self):
        return self.n

    def initialize(self):
        self.inits += 1
        self._L.calls.append(("init",))

    def stream(self):
        return 1234


class FakeCircuit:
    def __init__(self, tag, ops):
        self.handle = tag
        self._ops = ops

    def ops(self):
        return self._ops


def test_tune_execute_times_every_form_and_leaves_the_choice_set():
    P = pkg()
    T = P.autotune
    st = FakeState()
    circuits = [FakeCircuit("seg0", [(1, "unitary", [0, 1])]), FakeCircuit("seg1", [(0, "h", [2])])]
    cost = {1: 5.0, 2: 3.0, 0: 8.0}
    streams = []

    def timer(stream, fn):
        streams.append(stream)
        fn()
        return cost[st._L.mode]

    t = T.Autotuner(warmup=1, repeats=2)
    assert T.tune_execute(st, circuits, t, timer=timer) == 2
    assert set(streams) == {1234}
    # every timed run starts from |0...0> and applies both segments in order under one form
    runs = [c for c in st._L.calls if c[0] == "execute"]
    assert len(runs) == 2 * 3 * 3
    assert [r[2] for r in runs[:2]] == ["seg0", "seg1"]
    # the state is re-initialised with the chosen form set, after the last timed run
    assert st._L.calls[-2:] == [("blocking", 2), ("init",)]
    # the same structure on another state is not timed again
    st2 = FakeState()
    assert T.tune_execute(st2, circuits, t, timer=lambda s, fn: pytest.fail("timed")) == 2
    assert st2._L.mode == 2
    with pytest.raises(ValueError):
        T.tune_execute(FakeState(kind=P._capi.DENSITY_MATRIX), circuits, t, timer=timer)


def test_tune_tile_times_each_tile_and_caches_the_choice():
    P = pkg()
    T = P.autotune
    st = FakeState(n=20)
    circuits = [FakeCircuit("seg0", [(1, "unitary", [0, 1])])]
    cost = {0: 4.0, 11: 3.5, 10: 6.0}
    st._L.tile = 0

    def timer(stream, fn):
        fn()
        return cost[st._L.tile]

    t = T.Autotuner(warmup=1, repeats=2)
    assert T.tune_tile(st, circuits, t, timer=timer) == 11
    assert st._L.calls[-2:] == [("tile", 11), ("init",)]
    assert {c[1] for c in st._L.calls if c[0] == "tile"} == {0, 11, 10}
    # cached: a second state of the same structure is not timed
    st2 = FakeState(n=20)
    assert T.tune_tile(st2, circuits, t, timer=lambda s, fn: pytest.fail("timed")) == 11
    # tiles above the state size are not candidates
    small = FakeState(n=10)
    small._L.tile = 0
    seen = []

    def timer2(stream, fn):
        seen.append(small._L.tile)
        return 1.0

    T.tune_tile(small, [FakeCircuit("x", [(0, "h", [0])])], T.Autotuner(warmup=0, repeats=1), timer=timer2)
    assert set(seen) == {0, 10}


class FakeBatch:
    live = 0

    def __init__(self, teams, cost):
        self.teams, self.cost = teams, cost
        self.closed = False
        FakeBatch.live += 1
        assert FakeBatch.live == 1, "one candidate's batch resident at a time"

    def run(self, want_grad):
        assert not self.closed
        return self.cost[self.teams] * (2 if want_grad else 1)

    def close(self):
        if not self.closed:
            self.closed = True
            FakeBatch.live -= 1


def test_tune_batch_keeps_one_batch_resident_and_closes_it():
    T = tuner_mod()
    insts = [dict(n=12 + i % 3, gates=[0] * (5 + i), theta=[0.0] * 3, terms=[0] * 4, shots=16) for i in range(6)]
    cost = {(64, 0.5): 3.0, (0, 0.5): 2.0, (16, 0.5): 2.5, (64, 0.25): 2.0, (64, 0.75): 4.0}
    built = []

    def builder(instances, precision, teams):
        assert instances is insts and precision == "single"
        b = FakeBatch(teams, cost)
        built.append(b)
        return b

    t = T.Autotuner(warmup=1, repeats=2)
    assert T.tune_batch(insts, "single", True, t, builder=builder) == (0, 0.5)
    assert len(built) == 5 and FakeBatch.live == 0
    # the same shape in another order is the same key; want_grad is part of the key
    assert T.tune_batch(list(reversed(insts)), "single", True, t, builder=builder) == (0, 0.5)
    assert len(built) == 5
    T.tune_batch(insts, "single", False, t, builder=builder)
    assert len(built) == 10 and FakeBatch.live == 0


def test_simulator_option():
    P = pkg()
    sim = P.AerSimulator(autotune=True, autotune_cache="/nonexistent-dir/tune.json")
    assert sim.options["autotune"] is True
    assert sim.tuner().path == "/nonexistent-dir/tune.json"
    assert sim.tuner() is sim.tuner()
    assert P.AerSimulator().options["autotune"] is False
    assert P.AerSimulator(autotune=True).tuner() is P.autotune.default_tuner()
