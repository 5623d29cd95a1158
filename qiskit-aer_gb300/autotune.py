"""Schedule autotuner: for each workload, times the engine's schedule
candidates on the device and keeps the fastest.

Aer fixes these choices from configuration instead of measurement: the
cache-blocking qubit count (``blocking_qubits``,
src/transpile/cacheblocking.hpp:130-131, AerState::set_blocking_qubits in
src/controllers/state_controller.hpp:600-602) and the number of equal-size
states per batched launch (src/simulators/batch_shots_executor.hpp:152-314).
This module picks, per workload shape:

* ``gbqv_execute``: the cache-blocking form of a statevector op list.  It is
  one of: one kernel per op (0); cache-blocked runs with the tile held in
  registers (1, the default); or cache-blocked runs with the tile swept in
  shared memory (2).
* the tile of those cache-blocked runs (``gbqv_set_run_tile_qubits``): a
  run's ops act inside tiles of 2^m amplitudes, one state pass per run;
  larger tiles hold more ops per run, smaller ones fewer registers and
  shared memory per CTA.  Candidates: the default m (12 at complex128, 13
  at complex64) and one and two qubits less.
* ``gbqv_batch_run``: how the costliest instances of a batch of uneven
  circuits are split over two-CTA teams.  A setting is (at most
  ``max_team_instances`` teams, for instances costing at least
  ``min_cost_fraction`` of the largest).

Every candidate computes the same result; only the schedule changes.  The
tuner runs each candidate ``warmup`` times untimed, then ``repeats`` times
timed with CUDA events on the engine's stream, and keeps the lowest median.
A tie keeps the earlier candidate, so the engine's default wins unless
another form is strictly faster.  Choices are cached under a key made of the
device name, the precision and the workload's shape (qubit count, op types
and qubit sets; not matrix values or parameters).  So a later circuit of the
same structure, such as the next point of a parameter sweep, reuses the
choice without timing.  With a file path (argument, or the environment
variable ``GBQV_TUNE_CACHE``) the cache is read at start and rewritten after
each new choice.
"""
from __future__ import annotations

import hashlib
import json
import os
import statistics
from typing import Callable, Sequence

from . import _capi as A

# statevector execution forms, the default first (gbqv_set_blocking)
EXECUTE_CANDIDATES = (1, 2, 0)
# run tile qubits (gbqv_set_run_tile_qubits), the default (0) first
TILE_CANDIDATES = {"double": (0, 11, 10), "single": (0, 12, 11)}
# (max_team_instances, min_cost_fraction) for gbqv_batch_set_teams, the default first
TEAM_CANDIDATES = ((64, 0.5), (0, 0.5), (16, 0.5), (64, 0.25), (64, 0.75))


def _enc(candidate) -> str:
    """Canonical text of a candidate (tuples and lists alike)."""
    if isinstance(candidate, tuple):
        candidate = list(candidate)
    return json.dumps(candidate, sort_keys=True)


def _key_text(key) -> str:
    return "|".join(str(k) for k in key) if isinstance(key, (tuple, list)) else str(key)


def device_tag() -> str:
    """Name and compute capability of the current CUDA device ('no-device'
    without one); part of every cache key, so a cache file shared between
    machines keeps one choice per GPU model."""
    try:
        import torch

        if not torch.cuda.is_available():
            return "no-device"
        i = torch.cuda.current_device()
        major, minor = torch.cuda.get_device_capability(i)
        return f"{torch.cuda.get_device_name(i)} sm_{major}{minor}"
    except Exception:  # torch without CUDA support
        return "no-device"


class Autotuner:
    """Keeps the fastest schedule candidate per workload key.

    ``select(key, candidates, measure)`` returns the cached choice for
    ``key`` when it is still one of ``candidates``.  Otherwise it calls
    ``measure(candidate)``, which runs the workload once with that
    candidate and returns its device time in ms.  The calls are ``warmup``
    untimed plus ``repeats`` timed per candidate.  A candidate whose
    ``measure`` raises GBQVError (for example a bounded wait that gave up,
    GBQV_ERR_TIMEOUT) is skipped and its message recorded; when every
    candidate fails, the last error is raised."""

    def __init__(self, path: str | None = None, warmup: int = 1, repeats: int = 3):
        if warmup < 0 or repeats < 1:
            raise ValueError("warmup must be >= 0 and repeats >= 1")
        self.path = path if path is not None else (os.environ.get("GBQV_TUNE_CACHE") or None)
        self.warmup = int(warmup)
        self.repeats = int(repeats)
        self.entries: dict[str, dict] = {}
        self.measurements = 0  # measure() calls made by this tuner, warm-up included
        if self.path and os.path.exists(self.path):
            with open(self.path) as f:
                data = json.load(f)
            if not isinstance(data, dict) or not isinstance(data.get("entries", {}), dict):
                raise ValueError(f"{self.path}: not an autotune cache file")
            self.entries = dict(data.get("entries", {}))

    def lookup(self, key, candidates: Sequence):
        """The cached choice for key if it is one of candidates, else None."""
        hit = self.entries.get(_key_text(key))
        if hit is None:
            return None
        for c in candidates:
            if _enc(c) == hit["choice"]:
                return c
        return None

    def select(self, key, candidates: Sequence, measure: Callable[[object], float]):
        candidates = list(candidates)
        if not candidates:
            raise ValueError("no candidates to choose from")
        cached = self.lookup(key, candidates)
        if cached is not None:
            return cached
        if len(candidates) == 1:
            return candidates[0]
        times, errors, last_error = {}, {}, None
        best, best_ms = None, None
        for c in candidates:
            try:
                for _ in range(self.warmup):
                    self.measurements += 1
                    measure(c)
                samples = []
                for _ in range(self.repeats):
                    self.measurements += 1
                    samples.append(float(measure(c)))
            except A.GBQVError as e:
                errors[_enc(c)] = str(e)
                last_error = e
                continue
            ms = statistics.median(samples)
            times[_enc(c)] = ms
            if best_ms is None or ms < best_ms:
                best, best_ms = c, ms
        if best is None:
            raise last_error
        self.entries[_key_text(key)] = {"choice": _enc(best), "ms": times, "errors": errors}
        self._save()
        return best

    def _save(self) -> None:
        if not self.path:
            return
        tmp = f"{self.path}.tmp{os.getpid()}"
        with open(tmp, "w") as f:
            json.dump({"version": 1, "entries": self.entries}, f, indent=1, sort_keys=True)
        os.replace(tmp, self.path)


_default = None


def default_tuner() -> Autotuner:
    """The process-wide tuner (its file, if any, from GBQV_TUNE_CACHE)."""
    global _default
    if _default is None:
        _default = Autotuner()
    return _default


def device_timer(stream_ptr: int, fn: Callable[[], None]) -> float:
    """Device time in ms of the work fn() enqueues on the engine stream
    stream_ptr: CUDA events recorded on that stream on either side."""
    import torch

    stream = torch.cuda.ExternalStream(stream_ptr)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1)


def circuit_signature(circuits) -> str:
    """Structure of a list of engine op lists (NativeCircuit): op types,
    names and qubits in order, not matrices or parameter values."""
    h = hashlib.sha256()
    for nc in circuits:
        h.update(b"#")
        for t, name, qubits in nc.ops():
            h.update(f"{t}:{name}:{','.join(str(q) for q in qubits)};".encode())
    return h.hexdigest()[:32]


def tune_execute(state, circuits, tuner: Autotuner | None = None, candidates=EXECUTE_CANDIDATES,
                 timer: Callable[[int, Callable[[], None]], float] | None = None) -> int:
    """Picks the execution form (gbqv_set_blocking) of the op lists
    `circuits`, applied in order to the statevector `state`, by timing each
    candidate on that state.  On return the state is back in |0...0> with
    the chosen form set, ready for the real run.  Density-matrix and unitary
    handles are not tuned (their runs keep the default form)."""
    if getattr(state, "_kind", A.STATEVECTOR) != A.STATEVECTOR:
        raise ValueError("tune_execute tunes statevector handles only")
    tuner = tuner if tuner is not None else default_tuner()
    timer = timer if timer is not None else device_timer
    circuits = list(circuits)
    L, h = state._L, state.handle
    key = ("execute", device_tag(), state.precision, state.num_qubits(), circuit_signature(circuits))

    def run_all():
        for nc in circuits:
            A.check(L.gbqv_execute(h, nc.handle), h)

    def measure(mode):
        A.check(L.gbqv_set_blocking(h, int(mode)), h)
        state.initialize()
        return timer(state.stream(), run_all)

    choice = tuner.select(key, candidates, measure)
    A.check(L.gbqv_set_blocking(h, int(choice)), h)
    state.initialize()
    return int(choice)


def tune_tile(state, circuits, tuner: Autotuner | None = None, candidates=None,
              timer: Callable[[int, Callable[[], None]], float] | None = None) -> int:
    """Picks the tile qubits of the cache-blocked runs (gbqv_set_run_tile_qubits,
    0 = the engine's default) for the op lists `circuits` on the statevector
    `state`, under the execution form already set on it, by timing each
    candidate.  On return the state is back in |0...0> with the chosen tile
    set."""
    if getattr(state, "_kind", A.STATEVECTOR) != A.STATEVECTOR:
        raise ValueError("tune_tile tunes statevector handles only")
    tuner = tuner if tuner is not None else default_tuner()
    timer = timer if timer is not None else device_timer
    candidates = candidates if candidates is not None else TILE_CANDIDATES[state.precision]
    candidates = [c for c in candidates if c == 0 or c <= state.num_qubits()]
    circuits = list(circuits)
    L, h = state._L, state.handle
    key = ("tile", device_tag(), state.precision, state.num_qubits(), circuit_signature(circuits))

    def run_all():
        for nc in circuits:
            A.check(L.gbqv_execute(h, nc.handle), h)

    def measure(m):
        A.check(L.gbqv_set_run_tile_qubits(h, int(m)), h)
        state.initialize()
        return timer(state.stream(), run_all)

    choice = tuner.select(key, candidates, measure)
    A.check(L.gbqv_set_run_tile_qubits(h, int(choice)), h)
    state.initialize()
    return int(choice)


def batch_signature(instances) -> str:
    """Shape of a batch of instances (dicts as made by
    batched.config5_instances): per instance its qubits, gate count,
    parameter count, term count and shots, as a multiset."""
    rows = sorted((int(i["n"]), len(i["gates"]), len(i["theta"]), len(i["terms"]), int(i["shots"]))
                  for i in instances)
    return hashlib.sha256(repr(rows).encode()).hexdigest()[:32]


def build_batch(instances, precision: str = "double", teams=None):
    """A batched.Batch holding `instances`, with team setting `teams`
    ((max_team_instances, min_cost_fraction); None keeps the default)."""
    from .batched import Batch

    b = Batch(precision)
    try:
        if teams is not None:
            b.set_teams(int(teams[0]), float(teams[1]))
        for inst in instances:
            b.add(inst["n"], inst["gates"], inst["theta"], inst["terms"], inst["coeffs"], inst["shots"], inst["seed"])
    except Exception:
        b.close()
        raise
    return b


def tune_batch(instances, precision: str = "double", want_grad: bool = True, tuner: Autotuner | None = None,
               candidates=TEAM_CANDIDATES, builder=build_batch):
    """Picks the two-CTA team setting of one persistent launch over
    `instances` by running the whole batch under each candidate; the time
    is the launch's own device time (gbqv_batch_run).  One candidate's
    batch is resident at a time.  Returns the chosen
    (max_team_instances, min_cost_fraction)."""
    tuner = tuner if tuner is not None else default_tuner()
    key = ("batch", device_tag(), precision, int(bool(want_grad)), batch_signature(instances))
    live = {"teams": None, "batch": None}

    def measure(teams):
        if live["teams"] != teams:
            if live["batch"] is not None:
                live["batch"].close()
                live["batch"] = None
            live["batch"] = builder(instances, precision, teams)
            live["teams"] = teams
        return live["batch"].run(want_grad)

    try:
        return tuple(tuner.select(key, [tuple(c) for c in candidates], measure))
    finally:
        if live["batch"] is not None:
            live["batch"].close()
