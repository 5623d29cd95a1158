"""``EstimatorV2`` over the engine, the shape of qiskit_aer.primitives.EstimatorV2
(qiskit_aer/primitives/estimator_v2.py:46-159) without the qiskit dependency.

A pub is ``(circuit, observables[, parameter_values[, precision]])``:

* ``observables``: a Pauli label (``"XZI"``, qubit 0 rightmost), a dict
  ``{label: coeff}``, a list of ``(label, coeff)`` pairs (one observable, the
  ``SparsePauliOp.to_list()`` form), or a nested list / object array of those
  (an array of observables);
* ``parameter_values``: ``None``, an array of shape ``(..., P)`` whose last
  axis follows ``circuit.parameters`` (sorted by name), or a dict
  ``{Parameter: array of shape (...)}``;
* ``precision``: standard deviation of the Gaussian noise added to the
  expectation values (0: exact).

As in the reference, the parameter and observable shapes broadcast, every
distinct Pauli gets one ``save_expectation_value`` over all qubits, and the
circuit runs once with every binding through ``AerSimulator.run(...,
parameter_binds=[...])`` — which runs all bindings together on one stack of
states.  ``evs[i] = sum_p coeff_p <p>`` for the broadcast index i; ``stds`` is
the precision.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .circuit import Parameter, QuantumCircuit
from .simulator import AerSimulator


@dataclass
class Options:
    """Options of EstimatorV2 (estimator_v2.py:30-42)."""

    default_precision: float = 0.0
    backend_options: dict = field(default_factory=dict)
    run_options: dict = field(default_factory=dict)


class DataBin:
    def __init__(self, **kw):
        self._fields = list(kw)
        for k, v in kw.items():
            setattr(self, k, v)

    def __repr__(self):
        return "DataBin(" + ", ".join(f"{k}={getattr(self, k)!r}" for k in self._fields) + ")"


class PubResult:
    def __init__(self, data: DataBin, metadata: dict):
        self.data = data
        self.metadata = metadata


class PrimitiveResult(list):
    def __init__(self, pub_results, metadata=None):
        super().__init__(pub_results)
        self.metadata = metadata or {}


class PrimitiveJob:
    """Runs on submission; result() returns the PrimitiveResult."""

    def __init__(self, fn, *args):
        self._fn, self._args, self._result = fn, args, None

    def _submit(self):
        self._result = self._fn(*self._args)

    def result(self):
        if self._result is None:
            self._submit()
        return self._result

    def status(self):
        return "DONE" if self._result is not None else "INITIALIZING"


def _is_label(x) -> bool:
    return isinstance(x, str)


def _one_observable(obs) -> dict | None:
    """obs as {pauli label: coeff}, or None when it is an array of observables."""
    if _is_label(obs):
        return {obs: 1.0}
    if isinstance(obs, dict):
        return {str(k): complex(v) if np.iscomplexobj(v) else float(v) for k, v in obs.items()}
    if (isinstance(obs, (list, tuple)) and obs and all(isinstance(t, tuple) and len(t) == 2 and _is_label(t[0])
                                                       for t in obs)):
        out: dict = {}
        for lab, c in obs:
            out[lab] = out.get(lab, 0.0) + c
        return out
    return None


def coerce_observables(obs, num_qubits: int) -> np.ndarray:
    """An object array of {label: coeff} dicts (ObservablesArray.coerce)."""
    one = _one_observable(obs)
    if one is not None:
        arr = np.empty((), dtype=object)
        arr[()] = one
    else:
        items = [coerce_observables(o, num_qubits) for o in obs]
        arr = np.empty(len(items), dtype=object)
        if items and items[0].shape:
            arr = np.empty((len(items),) + items[0].shape, dtype=object)
        for i, it in enumerate(items):
            if it.shape != arr.shape[1:]:
                raise ValueError("observables array is ragged")
            if it.shape:
                arr[i] = it
            else:
                arr[i] = it[()]
    for d in arr.reshape(-1):
        for lab in d:
            if len(lab) != num_qubits or set(lab) - set("IXYZ"):
                raise ValueError(f"observable '{lab}' is not a Pauli label on {num_qubits} qubits")
    return arr


def coerce_parameter_values(values, circuit: QuantumCircuit) -> np.ndarray:
    """Array of shape (..., P), the last axis in the order of circuit.parameters."""
    params = circuit.parameters
    if values is None:
        if params:
            raise ValueError(f"the circuit has {len(params)} parameters and no parameter values")
        return None
    if isinstance(values, dict):
        by_name = {}
        for k, v in values.items():
            keys = k if isinstance(k, tuple) else (k,)
            v = np.asarray(v, dtype=np.float64)
            if len(keys) > 1:
                for i, kk in enumerate(keys):
                    by_name[kk.name if isinstance(kk, Parameter) else str(kk)] = v[..., i]
            else:
                kk = keys[0]
                by_name[kk.name if isinstance(kk, Parameter) else str(kk)] = v
        missing = [p.name for p in params if p.name not in by_name]
        if missing:
            raise ValueError(f"no values for parameters {missing}")
        cols = np.broadcast_arrays(*[by_name[p.name] for p in params])
        return np.stack(cols, axis=-1)
    arr = np.asarray(values, dtype=np.float64)
    if arr.ndim == 0 or arr.shape[-1] != len(params):
        raise ValueError(f"parameter values of shape {arr.shape} for {len(params)} parameters")
    return arr


class EstimatorV2:
    """Expectation values of observables on (parameterised) circuits."""

    def __init__(self, *, options: dict | None = None):
        self._options = Options(**options) if options else Options()
        self._backend = AerSimulator(**self._options.backend_options)

    @classmethod
    def from_backend(cls, backend: AerSimulator, **options):
        est = cls(**options)
        est._backend = backend
        return est

    @property
    def options(self) -> Options:
        return self._options

    def run(self, pubs, *, precision: float | None = None) -> PrimitiveJob:
        if precision is None:
            precision = self._options.default_precision
        coerced = [self._coerce(pub, precision) for pub in pubs]
        for i, (_, _, _, prec) in enumerate(coerced):
            if prec < 0.0:
                raise ValueError(f"The {i}-th pub has precision less than 0 ({prec}). "
                                 "But precision should be equal to or larger than 0.")
        job = PrimitiveJob(self._run, coerced)
        job._submit()
        return job

    @staticmethod
    def _coerce(pub, default_precision):
        if isinstance(pub, QuantumCircuit):
            raise ValueError("an estimator pub needs observables")
        circuit, obs = pub[0], pub[1]
        values = pub[2] if len(pub) > 2 else None
        prec = pub[3] if len(pub) > 3 and pub[3] is not None else default_precision
        observables = coerce_observables(obs, circuit.num_qubits)
        pv = coerce_parameter_values(values, circuit)
        return circuit, observables, pv, float(prec)

    def _run(self, pubs) -> PrimitiveResult:
        return PrimitiveResult([self._run_pub(*pub) for pub in pubs], metadata={"version": 2})

    def _run_pub(self, circuit: QuantumCircuit, observables: np.ndarray, values, precision: float) -> PubResult:
        circ = circuit.copy()
        params = circ.parameters
        param_shape = values.shape[:-1] if values is not None else ()
        # position of each parameter set in the flattened binding list
        # (the reference's param_indices / flat_indices, as integers)
        param_pos = np.arange(int(np.prod(param_shape, dtype=np.int64))).reshape(param_shape)
        obs_flat = observables.reshape(-1)
        obs_id = np.arange(obs_flat.size).reshape(observables.shape)
        bc_pos, bc_oid = np.broadcast_arrays(param_pos, obs_id)
        paulis = sorted({lab for d in obs_flat for lab in d})
        col = {lab: i for i, lab in enumerate(paulis)}
        n = circ.num_qubits
        for lab in paulis:
            circ.save_expectation_value([(1.0, lab, list(range(n)))], label=lab)
        run_options = dict(self._options.run_options)
        sim_meta = None
        if params and self._fast_bound(circ, run_options):
            # every binding on the bound stack, the expectation values straight
            # into E (the same kernels as backend.run; no per-binding results)
            flat = values.reshape(-1, len(params))
            binds = self._backend._check_binds([circ], [{p: flat[:, i] for i, p in enumerate(params)}], True)[0]
            nbind = flat.shape[0]
            arrays, sim_meta = self._backend._run_bound(circ, binds, nbind, [0] * nbind, 0, arrays_only=True)
            E = np.stack([arrays[lab] for lab in paulis], axis=1) if paulis else np.zeros((nbind, 0))
            nexp = nbind
        else:
            if params:
                flat = values.reshape(-1, len(params))
                binds = [{p: flat[:, i] for i, p in enumerate(params)}]
                result = self._backend.run(circ, parameter_binds=binds, **run_options)
            else:
                result = self._backend.run(circ, **run_options)
            # E[binding, pauli] and the observables' coefficients C[observable, pauli]
            nexp = len(result.results) if params else 1
            E = np.array([[result.data(j)[lab] for lab in paulis] for j in range(nexp)]).reshape(nexp, len(paulis))
            sim_meta = result.metadata(0) if result.results else {}
        Cm = np.zeros((obs_flat.size, len(paulis)), dtype=complex)
        for i, d in enumerate(obs_flat):
            for lab, coeff in d.items():
                Cm[i, col[lab]] += coeff
        # every (binding, observable) pair as one product, then the pub's
        # broadcast positions gathered from it
        F = np.real(E.astype(complex) @ Cm.T)  # [binding, observable]
        pos = bc_pos.reshape(-1) if params else np.zeros(bc_pos.size, dtype=np.int64)
        evs = F[pos, bc_oid.reshape(-1)].reshape(bc_pos.shape).astype(float)
        stds = np.full(bc_pos.shape, precision)
        if precision > 0:
            rng = np.random.default_rng(self._options.run_options.get("seed_simulator"))
            evs = rng.normal(evs, precision, evs.shape)
        return PubResult(DataBin(evs=evs, stds=stds, shape=evs.shape),
                         metadata={"target_precision": precision, "circuit_metadata": circuit.metadata,
                                   "simulator_metadata": sim_meta})

    def _fast_bound(self, circ: QuantumCircuit, run_options: dict) -> bool:
        """The bound stack serves the pub directly when the backend is this
        engine's simulator with its own options (no per-call overrides) and
        the circuit runs bound (unitary body, saves at the end)."""
        b = self._backend
        return (not run_options and isinstance(b, AerSimulator) and hasattr(b, "_run_bound")
                and b._bound_batchable(circ))


# ---------------------------------------------------------------------------
# SamplerV2 (qiskit_aer/primitives/sampler_v2.py): shots of (parameterised)
# circuits, returned per classical register as bit arrays of the pub's shape.
# ---------------------------------------------------------------------------
class BitArray:
    """Shots of one classical register: `values` holds each shot's register
    value, shape pub_shape + (shots,); `array` is the packed big-endian byte
    form of qiskit's BitArray."""

    def __init__(self, values: np.ndarray, num_bits: int):
        self._values = np.asarray(values, dtype=np.uint64)
        self.num_bits = int(num_bits)

    @property
    def shape(self):
        return self._values.shape[:-1]

    @property
    def num_shots(self) -> int:
        return self._values.shape[-1]

    @property
    def array(self) -> np.ndarray:
        nbytes = max(1, (self.num_bits + 7) // 8)
        out = np.zeros(self._values.shape + (nbytes,), dtype=np.uint8)
        for b in range(nbytes):
            out[..., nbytes - 1 - b] = ((self._values >> np.uint64(8 * b)) & np.uint64(0xFF)).astype(np.uint8)
        return out

    def _sel(self, loc):
        v = self._values if loc is None else self._values[loc]
        return v.reshape(-1)

    def get_int_counts(self, loc=None) -> dict:
        vals, cnt = np.unique(self._sel(loc), return_counts=True)
        return {int(v): int(c) for v, c in zip(vals, cnt)}

    def get_counts(self, loc=None) -> dict:
        return {format(v, f"0{self.num_bits}b"): c for v, c in self.get_int_counts(loc).items()}

    def get_bitstrings(self, loc=None) -> list:
        return [format(int(v), f"0{self.num_bits}b") for v in self._sel(loc)]


class SamplerPubResult(PubResult):
    def join_data(self):
        return next(iter(v for k, v in vars(self.data).items() if k not in ("_fields", "shape")))


class SamplerV2:
    """Samples of circuits with their final measurements (sampler_v2.py:53-228):
    pubs with the same shot count run as one job with their parameter
    bindings, `seed` as seed_simulator, per-shot memory turned into bit
    arrays."""

    def __init__(self, *, default_shots: int = 1024, seed: int | None = None, options: dict | None = None):
        self._default_shots = int(default_shots)
        self._seed = seed
        opts = dict(options or {})
        self._options = Options(backend_options=opts.get("backend_options", {}),
                                run_options=opts.get("run_options", {}))
        self._backend = AerSimulator(**self._options.backend_options)

    @property
    def default_shots(self) -> int:
        return self._default_shots

    @property
    def seed(self):
        return self._seed

    @property
    def options(self) -> Options:
        return self._options

    def run(self, pubs, *, shots: int | None = None) -> PrimitiveJob:
        if shots is None:
            shots = self._default_shots
        coerced = []
        for pub in pubs:
            if isinstance(pub, QuantumCircuit):
                pub = (pub,)
            circuit = pub[0]
            values = pub[1] if len(pub) > 1 else None
            s = pub[2] if len(pub) > 2 and pub[2] is not None else shots
            if int(s) < 1:
                raise ValueError("shots must be positive")
            coerced.append((circuit, coerce_parameter_values(values, circuit), int(s)))
        job = PrimitiveJob(self._run, coerced)
        job._submit()
        return job

    def _run(self, pubs) -> PrimitiveResult:
        by_shots: dict = {}
        for i, pub in enumerate(pubs):
            by_shots.setdefault(pub[2], []).append(i)
        results = [None] * len(pubs)
        for shots, idx in by_shots.items():
            for i, r in zip(idx, self._run_pubs([pubs[i] for i in idx], shots)):
                results[i] = r
        return PrimitiveResult(results, metadata={"version": 2})

    def _run_pubs(self, pubs, shots: int):
        circuits, binds, shapes = [], [], []
        for circuit, values, _ in pubs:
            params = circuit.parameters
            shape = values.shape[:-1] if values is not None else ()
            flat = values.reshape(-1, len(params)) if values is not None else np.zeros((1, 0))
            circuits.append(circuit)
            binds.append({p: flat[:, i] for i, p in enumerate(params)} if params else {})
            shapes.append(shape)
        run_options = {k: v for k, v in self._options.run_options.items()
                       if k not in ("shots", "parameter_binds", "memory", "seed_simulator")}
        result = self._backend.run(circuits, shots=shots, seed_simulator=self._seed, parameter_binds=binds,
                                   memory=True, **run_options)
        out, k = [], 0
        for (circuit, _, _), shape in zip(pubs, shapes):
            size = int(np.prod(shape, dtype=np.int64))
            vals = np.zeros((size, shots), dtype=np.uint64)
            for j in range(size):
                mem = result.data(k + j).get("memory")
                if mem:
                    vals[j] = [int(x, 16) for x in mem]
            k += size
            bits = BitArray(vals.reshape(tuple(shape) + (shots,)), circuit.num_clbits)
            out.append(SamplerPubResult(DataBin(**{circuit.creg_name: bits, "shape": tuple(shape)}),
                                        metadata={"shots": shots, "circuit_metadata": circuit.metadata,
                                                  "simulator_metadata": result.metadata(0) if result.results
                                                  else {}}))
        return out

