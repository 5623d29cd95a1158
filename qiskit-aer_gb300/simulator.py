"""``AerSimulator``-shaped front end over the GB300 engine.

Mirrors the drop-in site ``AerSimulator(method='statevector'|'density_matrix',
device='GPU', precision=...)`` (qiskit_aer/backends/aer_simulator.py:713-716)
and the controller path it drives: per-circuit seeds
``seed_simulator + 2113*i`` (src/controllers/controller_execute.hpp:188-210),
the Fusion pass with the per-method defaults of
``Executor::transpile_fusion`` (simulators/circuit_executor.hpp:1228-1287),
noise inserted as superoperators for the density-matrix method and sampled
per shot as Kraus channels for the statevector method
(circuit_executor.hpp:648-657, State::apply_kraus), ops applied
in order (State::apply_ops, state.hpp:295-340), final measurements sampled
from ``shots`` uniforms of one RngEngine stream
(statevector_state.hpp:1016-1052), and save instructions evaluated where
they sit.  Result metadata carries the reference's fusion keys
(fusion.hpp:864-945).
"""
from __future__ import annotations

import copy
import ctypes as C
import time
import warnings

import numpy as np

from . import _capi as A
from .autotune import Autotuner, default_tuner, tune_execute, tune_tile
from .circuit import Instruction, NativeCircuit, QuantumCircuit, expval_params
from .noise import apply_readout
from .qubitvector import DensityMatrix, QubitVector, UnitaryMatrix


def discrete_draw(probs, u: float) -> int:
    """RngEngine::rand_int(probs) (rng.hpp:94-96) given the uniform u that the
    draw consumes: libstdc++'s std::discrete_distribution normalises the
    weights by their sequential sum, takes sequential partial sums, sets the
    last to 1 and returns lower_bound(cumulative, u), where u is the same
    generate_canonical<double, 53> value that uniform_real_distribution(0, 1)
    yields for the engine's next 64-bit word."""
    p = np.asarray(probs, dtype=np.float64)
    total = np.add.accumulate(p)[-1]
    cp = np.add.accumulate(p / total)
    cp[-1] = 1.0
    return int(np.searchsorted(cp, u, side="left"))


def ket_dict(values, epsilon: float) -> dict:
    """Utils::vec2ket(values, epsilon, 16) (framework/utils.hpp:963-990):
    each value chopped (real and imaginary parts below epsilon in magnitude
    set to 0, utils.hpp:909-934), kept when its magnitude then exceeds
    epsilon, keyed by its index as "0x..." hex without leading zeros."""
    v = np.asarray(values)
    if np.iscomplexobj(v):
        v = np.where(np.abs(v.real) < epsilon, 0.0, v.real) + 1j * np.where(np.abs(v.imag) < epsilon, 0.0, v.imag)
    else:
        v = np.where(np.abs(v) < epsilon, 0.0, v)
    return {hex(int(k)): v[k].item() for k in np.nonzero(np.abs(v) > epsilon)[0]}


def discrete_draws(probs: np.ndarray, u: np.ndarray) -> np.ndarray:
    """discrete_draw for each row of probs with its own uniform: the same
    sequential sums per row, so every row gives discrete_draw's index."""
    p = np.asarray(probs, dtype=np.float64)
    if p.shape[0] == 0:
        return np.zeros(0, dtype=np.int64)
    total = np.add.accumulate(p, axis=1)[:, -1]
    cp = np.add.accumulate(p / total[:, None], axis=1)
    cp[:, -1] = 1.0
    return np.sum(cp < np.asarray(u, dtype=np.float64)[:, None], axis=1).astype(np.int64)


def uniforms(seed: int, count: int) -> np.ndarray:
    """RngEngine::rand(0,1) stream for `seed` (std::mt19937_64)."""
    out = np.empty(int(count), dtype=np.float64)
    A.check(A.lib().gbqv_uniforms(int(seed) & (2**64 - 1), out.size, out.ctypes.data_as(A.dp)))
    return out


def kraus_draws(probs: np.ndarray, u: np.ndarray):
    """State::apply_kraus's choice for each row (statevector_state.hpp:
    1112-1156): probs[s, j] = ||K_j psi_s||^2; with r = u[s], the first
    operator j < m - 1 whose sequential sum of probabilities exceeds r is
    applied scaled by 1/sqrt(p_j); if none, the last, scaled by
    1/sqrt(1 - that sum).  Returns (operator index, scale) per row."""
    p = np.asarray(probs, dtype=np.float64)
    rows, m = p.shape
    branch = np.full(rows, m - 1, dtype=np.int64)
    scale = np.ones(rows, dtype=np.float64)
    if m > 1 and rows:
        acc = np.add.accumulate(p[:, :m - 1], axis=1)
        hit = acc > np.asarray(u, dtype=np.float64)[:, None]
        got = hit.any(axis=1)
        first = np.argmax(hit, axis=1)
        branch[got] = first[got]
        scale[got] = 1.0 / np.sqrt(p[got, first[got]])
        scale[~got] = 1.0 / np.sqrt(1.0 - acc[~got, -1])
    return branch, scale


class KrausOp:
    """A Kraus channel sampled once per shot on a statevector
    (State::apply_kraus): the operators as given (a circuit's kraus
    instruction) or a noise model error's canonical ones
    (Utils::superop2kraus).  `gram` holds K^dag K, from which each shot's
    probabilities follow from its reduced density matrix; `fixed` the
    probabilities when every K^dag K is a multiple of the identity (a
    mixture of unitaries), which then need no pass over the states."""

    def __init__(self, qubits, mats):
        self.qubits = [int(q) for q in qubits]
        D = 1 << len(self.qubits)
        self.mats = np.stack([np.asarray(m, dtype=np.complex128) for m in mats])
        if self.mats.shape[1:] != (D, D):
            raise ValueError(f"Kraus operators on {len(self.qubits)} qubits must be {D}x{D}")
        if not 1 <= len(mats) <= 255:
            raise ValueError("a Kraus channel takes 1..255 operators")
        self.gram = np.einsum("jba,jbc->jac", self.mats.conj(), self.mats)
        # column-major matrices, one after another
        self.colmajor = np.ascontiguousarray(self.mats.transpose(0, 2, 1)).reshape(-1)
        c = np.einsum("jaa->j", self.gram).real / D
        flat = np.max(np.abs(self.gram - c[:, None, None] * np.eye(D)))
        self.fixed = c if flat <= 1e-13 else None
        # operators that are multiples of the identity: normalised, they
        # leave a state as it is (to within one rounding) and are skipped
        self.corner = self.mats[:, 0, 0].copy()
        self.ident = np.array([abs(M[0, 0]) > 0 and np.max(np.abs(M - M[0, 0] * np.eye(D))) <= 1e-15
                               for M in self.mats])


class Result:
    def __init__(self, results, time_taken):
        self.results = results
        self.time_taken = time_taken

    def result(self):
        """The job's result: run() completes before it returns, so the
        AerJob-style `backend.run(...).result()` chain is this object."""
        return self

    def get_counts(self, i=0):
        return self.results[i]["counts"]

    def get_memory(self, i=0):
        return self.results[i]["data"]["memory"]

    def data(self, i=0):
        return self.results[i]["data"]

    def metadata(self, i=0):
        return self.results[i]["metadata"]

    def get_statevector(self, i=0):
        return self.results[i]["data"]["statevector"]

    def get_unitary(self, i=0):
        return self.results[i]["data"]["unitary"]


class AerSimulator:
    METHODS = ("statevector", "density_matrix", "unitary")

    def __init__(self, method: str = "statevector", device: str = "GPU", precision: str = "double",
                 noise_model=None, fusion_enable: bool = True, fusion_max_qubit: int | None = None,
                 fusion_threshold: int | None = None, fusion_cost_factor: float = 1.8,
                 fusion_avx2_costs: bool = True, blocking_enable: bool = True, seed_simulator: int | None = None,
                 autotune: bool = False, autotune_cache: str | None = None, runtime_compile: int = 1):
        if method not in self.METHODS:
            raise ValueError(f"method must be one of {self.METHODS}")
        if device != "GPU":
            raise ValueError("this engine runs on the GPU only (device='GPU')")
        self.method = method
        self.precision = precision
        self.noise_model = noise_model
        self.options = dict(fusion_enable=fusion_enable, fusion_max_qubit=fusion_max_qubit,
                            fusion_threshold=fusion_threshold, fusion_cost_factor=fusion_cost_factor,
                            fusion_avx2_costs=fusion_avx2_costs, blocking_enable=blocking_enable,
                            seed_simulator=seed_simulator, autotune=autotune, autotune_cache=autotune_cache,
                            runtime_compile=runtime_compile)
        self._tuner = None

    # ---- options (AerBackend.set_option / set_options, aerbackend.py:623-658;
    # AerSimulator.set_option, available_methods / available_devices,
    # aer_simulator.py:877-935) ----
    _DEFAULTS = dict(method="statevector", device="GPU", precision="double", noise_model=None, fusion_enable=True,
                     fusion_max_qubit=None, fusion_threshold=None, fusion_cost_factor=1.8, fusion_avx2_costs=True,
                     blocking_enable=True, seed_simulator=None, autotune=False, autotune_cache=None,
                     runtime_compile=1)

    @property
    def name(self) -> str:
        return f"aer_simulator_{self.method}_gpu"

    def available_methods(self) -> list:
        return list(self.METHODS)

    def available_devices(self) -> list:
        return ["GPU"]

    def set_option(self, key: str, value) -> None:
        """Set one option; None restores its default.  Unknown keys and
        methods, devices or precisions this engine does not have are errors
        (the reference's AerError messages, as ValueError)."""
        if key not in self._DEFAULTS:
            raise ValueError(f"Invalid option {key}")
        if value is None:
            value = self._DEFAULTS[key]
        if key == "method":
            if value not in self.METHODS:
                raise ValueError(f"Invalid simulation method {value}. Available methods are: {self.available_methods()}")
            self.method = value
        elif key == "device":
            if value != "GPU":
                raise ValueError("this engine runs on the GPU only (device='GPU')")
        elif key == "precision":
            if value not in ("double", "single"):
                raise ValueError(f"Invalid precision {value}: 'double' or 'single'")
            self.precision = value
        elif key == "noise_model":
            self.noise_model = value
        elif key == "runtime_compile":
            if value not in (0, 1, 2):
                raise ValueError(f"Invalid runtime_compile {value}: 0 (never), 1 (recurring runs) or 2 (always)")
            self.options[key] = value
        else:
            self.options[key] = value
            if key == "autotune_cache":
                self._tuner = None

    def set_options(self, **fields) -> None:
        for key, value in fields.items():
            self.set_option(key, value)

    def _state_options(self, st) -> None:
        """Per-state engine settings taken from the options: runs compiled
        for their op sequence (gbqv_set_run_jit) unless runtime_compile is
        the default."""
        if self.options["runtime_compile"] != 1:
            A.check(st._L.gbqv_set_run_jit(st.handle, int(self.options["runtime_compile"])), st.handle)

    def tuner(self) -> Autotuner:
        """The schedule autotuner of this simulator: its own cache file when
        autotune_cache is given, else the process-wide tuner."""
        if self._tuner is None:
            path = self.options["autotune_cache"]
            self._tuner = Autotuner(path) if path else default_tuner()
        return self._tuner

    # ---- fusion configuration ----
    def fusion_config(self, has_superop=False, has_kraus=False) -> A.FusionConfig:
        cfg = A.FusionConfig()
        A.check(A.lib().gbqv_fusion_default_config(1 if self.method == "density_matrix" else 0, C.byref(cfg)))
        o = self.options
        # Executor::transpile_fusion: flags from the circuit's op set, then halving
        # for Kraus on statevector, then the user config overrides
        cfg.allow_superop = int(has_superop)
        cfg.allow_kraus = int(has_kraus)
        if self.method == "statevector" and has_kraus:
            cfg.max_qubit //= 2
        cfg.enable = int(o["fusion_enable"])
        if o["fusion_max_qubit"] is not None:
            cfg.max_qubit = int(o["fusion_max_qubit"])
        if self.method == "unitary":
            cfg.threshold //= 2  # Executor::transpile_fusion, Method::unitary (circuit_executor.hpp:1259-1262)
        if o["fusion_threshold"] is not None:
            cfg.threshold = int(o["fusion_threshold"])
        cfg.cost_factor = float(o["fusion_cost_factor"])
        cfg.avx2_costs = int(o["fusion_avx2_costs"])
        return cfg

    def _noise_ops(self, name, qubits) -> list:
        """The noise model's errors on one instruction as superop
        instructions (NoiseModel::op_errors)."""
        if self.noise_model is None or not self.noise_model.has_quantum_errors():
            return []
        out = []
        for q, err in self.noise_model.op_errors(name, qubits):
            if err.num_qubits != len(q):
                raise ValueError(f"error on '{name}' acts on {err.num_qubits} qubits, the instruction on {len(q)}")
            out.append(Instruction("superop", "superop", list(q), data=err.superop))
        return out

    def _with_noise(self, body, positions=None):
        """Insert the noise model's superoperators: after each matching gate
        or reset, before each measure (the reference sets measure errors to
        act before the op, noise_model.hpp:1075-1085).  `positions` (op
        indices into `body`) are mapped to the new list."""
        if self.noise_model is None or not self.noise_model.has_quantum_errors():
            return (body, list(positions)) if positions is not None else body
        if self.method != "density_matrix":
            if any(self._error_kraus(ins) for ins in body):
                raise ValueError("noise on a statevector is sampled per shot as Kraus channels, in circuits run "
                                 "shot by shot; use method='density_matrix' for superoperator noise")
            return (body, list(positions)) if positions is not None else body
        out, new_index = [], []
        for ins in body:
            new_index.append(len(out))
            if ins.kind == "measure":
                out.extend(self._noise_ops("measure", ins.qubits))
                out.append(ins)
                continue
            out.append(ins)
            if ins.kind == "gate":
                out.extend(self._noise_ops(ins.name, ins.qubits))
            elif ins.kind == "reset":
                out.extend(self._noise_ops("reset", ins.qubits))
        if positions is None:
            return out
        new_index.append(len(out))
        return out, [new_index[p] for p in positions]

    def compile(self, circuit: QuantumCircuit):
        """Assemble + fuse; returns (NativeCircuit list per save segment,
        measures, saves, metadata)."""
        body, meas, saves = circuit.split_final()
        body, pos = self._with_noise(body, [p for p, _ in saves])
        saves = [(p, ins) for p, (_, ins) in zip(pos, saves)]
        # errors on the final measurements act before them: after every op and save
        body = body + [e for m in meas for e in self._noise_ops("measure", m.qubits)]
        kinds = {i.kind for i in body}
        cfg = self.fusion_config(has_superop="superop" in kinds, has_kraus="kraus" in kinds)
        meta = {"fusion": {"enabled": bool(cfg.enable)}}
        # saves split the op list: fuse each segment separately
        bounds = sorted({pos for pos, _ in saves} | {len(body)})
        segments, start, applied_any, method_name = [], 0, False, ""
        t0 = time.perf_counter()
        for b in bounds:
            nc = NativeCircuit(circuit.num_qubits, body[start:b])
            applied, method_name = nc.fuse(cfg)
            applied_any |= applied
            segments.append((b, nc))
            start = b
        if cfg.enable:
            meta["fusion"].update({"threshold": cfg.threshold, "max_fused_qubits": cfg.max_qubit,
                                   "applied": applied_any, "cost_factor": cfg.cost_factor,
                                   "time_taken": time.perf_counter() - t0})
            if method_name:
                meta["fusion"]["method"] = method_name
        return segments, meas, saves, meta

    _want_memory = False

    def run(self, circuits, shots: int = 1024, seed_simulator: int | None = None, parameter_binds=None,
            memory: bool = False, **run_options):
        """parameter_binds: one dict {Parameter: values} per circuit (AerBackend.run,
        qiskit_aer/backends/aerbackend.py:146-185); a parameterised circuit
        becomes one experiment per binding, in order, and experiment k of the
        job gets seed seed_simulator + 2113 * k (controller_execute.hpp:188-210).
        Other keyword options (method, noise_model, precision, fusion_*, ...)
        override the simulator's options for this call only, as the
        reference's run_options do; options this engine does not have are
        ignored with a warning."""
        unknown = sorted(k for k in run_options if k not in self._DEFAULTS)
        if unknown:
            warnings.warn(f"run options not used by this engine: {', '.join(unknown)}", stacklevel=2)
        run_options = {k: v for k, v in run_options.items() if k in self._DEFAULTS}
        call = self
        if run_options or bool(memory) != self._want_memory:
            # the overrides and the memory flag go to a per-call copy, as the
            # reference builds a per-call config (aerbackend.py
            # generate_aer_config); the simulator itself is left unchanged, so
            # concurrent run() calls do not see each other's options
            call = copy.copy(self)
            call.options = dict(self.options)
            call._want_memory = bool(memory)
            call.set_options(**run_options)
        return call._run(circuits, shots, seed_simulator, parameter_binds, memory)

    def _run(self, circuits, shots, seed_simulator, parameter_binds, memory):
        single = isinstance(circuits, QuantumCircuit)
        if single:
            circuits = [circuits]
        binds = self._check_binds(circuits, parameter_binds, single)
        seed = seed_simulator if seed_simulator is not None else self.options["seed_simulator"]
        if seed is None:
            seed = int(np.random.SeedSequence().entropy & 0x7FFFFFFF)
        t0 = time.perf_counter()
        results, k = [], 0
        for c, b in zip(circuits, binds):
            if not b:
                results.append(self._run_one(c, shots, seed + 2113 * k))
                k += 1
                continue
            nbind = len(next(iter(b.values())))
            seeds = [seed + 2113 * (k + j) for j in range(nbind)]
            if self._bound_batchable(c):
                results.extend(self._run_bound(c, b, nbind, seeds, shots))
            else:
                for j in range(nbind):
                    results.append(self._run_one(c.assign_parameters({p: v[j] for p, v in b.items()}), shots,
                                                 seeds[j]))
            k += nbind
        return Result(results, time.perf_counter() - t0)

    @staticmethod
    def _check_binds(circuits, parameter_binds, single):
        """Per circuit, {Parameter: values} restricted to its parameters (empty
        for a circuit without any), with the reference's validation
        (AerBackend._convert_binds, aerbackend.py:128-144, and the length
        check of controller_execute.hpp:104-155)."""
        if parameter_binds is None:
            if any(c.parameters for c in circuits):
                raise ValueError("circuits have parameters but parameter_binds is not specified.")
            return [{} for _ in circuits]
        if single and len(parameter_binds) > 1:
            raise ValueError("More than 1 parameter table provided for a single circuit")
        if len(parameter_binds) != len(circuits):
            raise ValueError("Number of input circuits does not match number of input parameter bind dictionaries")
        out = []
        for c, table in zip(circuits, parameter_binds):
            params = c.parameters
            if not params:
                out.append({})
                continue
            missing = [p.name for p in params if p not in table]
            if missing:
                raise ValueError(f"no values bound to parameters {missing}")
            b = {p: np.atleast_1d(np.asarray(table[p], dtype=np.float64)).reshape(-1) for p in params}
            lens = {v.size for v in b.values()}
            if len(lens) != 1 or 0 in lens:
                raise ValueError("Invalid parameterization: every parameter needs the same number of values")
            out.append(b)
        return out

    def _bound_batchable(self, circuit: QuantumCircuit) -> bool:
        """Bindings run together on one stack of states when the circuit is a
        unitary statevector circuit whose saves (expectation values,
        statevectors) and measurements all sit at its end; each binding's
        shots are then drawn from its own state of the stack."""
        if self.method != "statevector" or (self.noise_model is not None and not self.noise_model.is_ideal()):
            return False
        if circuit.needs_shots("statevector"):
            return False
        body, meas, saves = circuit.split_final()
        if any(ins.kind not in ("gate", "unitary", "diagonal", "barrier") for ins in body):
            return False
        return all(pos == len(body) and ins.kind == "save" and ins.name in ("expval", "statevector")
                   for pos, ins in saves)

    # largest stack of bound states held at once: 2^31 amplitudes (34 GB at complex128)
    MAX_STACK_QUBITS = 31

    def _run_bound(self, circuit: QuantumCircuit, binds: dict, nbind: int, seeds, shots: int,
                   arrays_only: bool = False):
        """Every binding of a parameterised circuit at once
        (BatchShotsExecutor over runtime-bound parameters,
        batch_shots_executor.hpp:152-314): the circuit is assembled once, its
        parameterised gates get per-binding values (gbqv_circuit_bind_param),
        and each chunk of bindings runs on one stack of states
        (gbqv_execute_bound); expectation values are reduced per state, every
        saved observable's Paulis in one call.  arrays_only: only the
        expectation values, as {label: value per binding} with the run's
        metadata (the EstimatorV2 path, no per-binding result dicts)."""
        n = circuit.num_qubits
        body, meas, saves = circuit.split_final()
        mq = [q for m in meas for q in m.qubits]
        mc = [c for m in meas for c in m.clbits]
        counts = [None] * nbind
        nc = NativeCircuit(n, body)
        nc.bind(binds, nbind)
        data = [{} for _ in range(nbind)] if not arrays_only else None
        arrays = {}
        # the expectation-value saves: their Paulis in one list, and per save
        # the coefficient of each
        ev_saves = [ins for _, ins in saves if ins.name != "statevector"]
        ev_terms, ev_coef = [], []
        for ins in ev_saves:
            label, terms = ins.data
            params = expval_params(terms)
            ev_coef.append((label, len(ev_terms), np.array([c1 for _, c1, _ in params])))
            ev_terms.extend(ql for ql, _, _ in params)
            arrays[label] = np.zeros(nbind)
        chunk = 1 << max(0, self.MAX_STACK_QUBITS - n)
        L = A.lib()
        st, st_bits = None, -1
        try:
            for first in range(0, nbind, chunk):
                cnt = min(chunk, nbind - first)
                b = (cnt - 1).bit_length()
                if st is None or st_bits != b:
                    if st is not None:
                        st.close()
                    st, st_bits = QubitVector(n + b, self.precision), b
                    self._state_options(st)
                A.check(L.gbqv_execute_bound(st.handle, nc.handle, first, cnt), st.handle)
                if meas and shots > 0:
                    # every binding draws from its own RngEngine stream, seed_simulator + 2113 k
                    rnds = np.ascontiguousarray(np.concatenate([uniforms(seeds[first + j], shots) for j in range(cnt)]))
                    smp = np.empty(cnt * shots, dtype=np.uint64)
                    A.check(L.gbqv_sample_measure_segments(st.handle, n, 0, cnt, rnds.ctypes.data_as(A.dp), shots,
                                                           smp.ctypes.data_as(A.u64p)), st.handle)
                    for j in range(cnt):
                        sj = smp[j * shots:(j + 1) * shots]
                        counts[first + j] = self._counts(sj, mq, mc, circuit.num_clbits)
                        if self._want_memory:
                            data[first + j]["memory"] = self._memory(self._memory_values(sj, mq, mc))
                for _, ins in saves:
                    if ins.name == "statevector" and not arrays_only:
                        vec = st.copy_to_vector()
                        for j in range(cnt):
                            data[first + j][ins.data] = vec[j << n:(j + 1) << n].copy()
                if ev_terms:
                    vals = st.expval_pauli_segments(n, cnt, ev_terms)  # [term, binding]
                    for label, off, coef in ev_coef:
                        total = np.zeros(cnt)
                        for c1, v in zip(coef, vals[off:off + coef.size]):  # in parameter order, per binding
                            total += c1 * v
                        arrays[label][first:first + cnt] = total
                        if not arrays_only:
                            for j in range(cnt):
                                data[first + j][label] = float(total[j])
            if st is not None:
                st.synchronize()
        finally:
            if st is not None:
                st.close()
        meta = {"fusion": {"enabled": False}, "parameter_binding": {"batched": True, "bindings": nbind,
                                                                   "stack_qubits": n + max(st_bits, 0)}}
        if arrays_only:
            return arrays, meta
        return [{"counts": counts[j], "data": data[j], "metadata": dict(meta), "seed_simulator": seeds[j],
                 "shots": shots} for j in range(nbind)]

    def _sampled_noise(self, circuit: QuantumCircuit) -> bool:
        """A statevector run whose noise model puts an error on some
        instruction of the circuit: every such error becomes a Kraus channel
        sampled per shot (the reference's Kraus noise method,
        circuit_executor.hpp:648-657), so the circuit runs shot by shot."""
        if self.method != "statevector" or self.noise_model is None or not self.noise_model.has_quantum_errors():
            return False
        return any(self._error_kraus(ins) for ins in circuit.data)

    def _error_kraus(self, ins, before: bool | None = None) -> list:
        """The noise model's errors on one instruction as KrausOps: after a
        gate or reset, before a measure (noise_model.hpp:1075-1085)."""
        if self.noise_model is None or not self.noise_model.has_quantum_errors():
            return []
        if ins.kind == "measure":
            name = "measure"
        elif ins.kind == "reset":
            name = "reset"
        elif ins.kind == "gate":
            name = ins.name
        else:
            return []
        if before is not None and before != (name == "measure"):
            return []
        out = []
        for q, err in self.noise_model.op_errors(name, ins.qubits):
            if err.num_qubits != len(q):
                raise ValueError(f"error on '{name}' acts on {err.num_qubits} qubits, the instruction on {len(q)}")
            if not err.ideal():
                out.append(KrausOp(q, err.kraus()))
        return out

    def _run_one(self, circuit: QuantumCircuit, shots: int, seed: int):
        if self.method == "statevector" and (circuit.needs_shots("statevector") or self._sampled_noise(circuit)):
            return self._run_shots(circuit, shots, seed)
        if self.method == "density_matrix" and circuit.needs_shots("density_matrix"):
            return self._run_shots_dm(circuit, shots, seed)
        if self.method == "unitary":
            self._check_unitary_circuit(circuit)
        segments, meas, saves, meta = self.compile(circuit)
        cls = {"density_matrix": DensityMatrix, "unitary": UnitaryMatrix}.get(self.method, QubitVector)
        data = {}
        with cls(circuit.num_qubits, self.precision) as st:
            self._state_options(st)
            if not self.options["blocking_enable"]:
                A.check(st._L.gbqv_set_blocking(st.handle, 0))
            elif self.options["autotune"] and self.method == "statevector":
                ncs = [nc for _, nc in segments]
                mode = tune_execute(st, ncs, self.tuner())
                meta["autotune"] = {"blocking": mode}
                if mode != 0:  # the cache-blocked forms: their tile as well
                    meta["autotune"]["tile_qubits"] = tune_tile(st, ncs, self.tuner())
            save_iter = iter(saves)
            pending = next(save_iter, None)
            for bound, nc in segments:
                if nc.num_ops():  # a save or set before any op leaves an empty segment
                    A.check(st._L.gbqv_execute(st.handle, nc.handle), st.handle)
                while pending is not None and pending[0] == bound:
                    self._save(st, pending[1], data)
                    pending = next(save_iter, None)
            counts = None
            if meas:
                qubits = [q for m in meas for q in m.qubits]
                clbits = [c for m in meas for c in m.clbits]
                ro = self._readout_ops(meas)
                stream = uniforms(seed, shots * (1 + len(ro)))
                samples = st.sample_measure(stream[:shots])
                if ro:
                    mem = self._readout_sampled(self._memory_values(samples, qubits, clbits), ro, stream[shots:])
                    counts = self._counts_of(mem, circuit.num_clbits)
                    if self._want_memory:
                        data["memory"] = self._memory(mem)
                else:
                    counts = self._counts(samples, qubits, clbits, circuit.num_clbits)
                    if self._want_memory:
                        data["memory"] = self._memory(self._memory_values(samples, qubits, clbits))
            st.synchronize()
        return {"counts": counts, "data": data, "metadata": meta, "seed_simulator": seed, "shots": shots}

    # shots per stacked group and the largest stack (qubits of the circuit +
    # shot bits), about 4 GB of complex128 amplitudes
    CHOP_THRESHOLD = 1e-8  # Config::chop_threshold (framework/config.hpp:125)
    SHOT_GROUP_BITS = 16
    SHOT_STACK_QUBITS = 28
    HOST_DRAW_QUBITS = 10  # wider registers are drawn on the device

    def _run_shots(self, circuit: QuantumCircuit, shots: int, seed: int):
        """A circuit that cannot be measure-sampled (CircuitExecutor::
        run_circuit_shots, circuit_executor.hpp:880-940): shot i starts from
        |0...0> with RngEngine seed + i; unitary stretches between
        measurements, resets and conditional ops are fused once; measure and
        reset draw one outcome each (State::sample_measure_with_prob) and
        collapse the state (State::measure_reset_update,
        statevector_state.hpp:936-1011).  Shots run in groups, one stacked
        state per shot (the reference's batched shots on a GPU,
        QubitVectorThrust::apply_batched_measure / apply_batched_reset,
        qubitvector_thrust.hpp:2251-2448): each stretch runs once over the
        whole group, each measurement is one probability pass, a host draw
        per shot from its own stream and one collapse pass."""
        cfg = self.fusion_config()
        items, stretch = [], []
        noisy = self._sampled_noise(circuit)

        def flush():
            if stretch:
                nc = NativeCircuit(circuit.num_qubits, list(stretch))
                nc.fuse(cfg)
                items.append(("ops", nc, None))
                stretch.clear()

        for ins in circuit.data:
            if ins.kind == "set":
                raise NotImplementedError("set instructions in a circuit run shot by shot")
            if ins.kind == "save" and ins.name not in self.SHOT_SAVES:
                raise NotImplementedError(f"save instructions other than {', '.join(self.SHOT_SAVES)} in a circuit "
                                          "run shot by shot")
            if ins.kind == "save":
                flush()
                items.append(("save", ins, None))
                continue
            if ins.kind == "superop":
                raise ValueError("superop instructions need method='density_matrix'")
            # noise ops inherit the instruction's condition (noise_model.hpp:422-431)
            errs = self._error_kraus(ins) if noisy else []
            if ins.kind == "kraus":
                flush()
                items.append(("kraus", KrausOp(ins.qubits, ins.data), ins.condition))
            elif ins.kind in ("measure", "reset"):
                flush()
                if ins.kind == "measure":
                    items.extend(("kraus", e, ins.condition) for e in errs)
                items.append((ins.kind, ins, ins.condition))
                if ins.kind == "reset":
                    items.extend(("kraus", e, ins.condition) for e in errs)
            elif ins.condition is not None:
                flush()
                cond = Instruction(ins.kind, ins.name, ins.qubits, ins.params, ins.data, ins.clbits)
                items.append(("ops", NativeCircuit(circuit.num_qubits, [cond]), ins.condition))
                items.extend(("kraus", e, ins.condition) for e in errs)
            elif ins.kind != "barrier":
                stretch.append(ins)
                if errs:
                    flush()
                    items.extend(("kraus", e, None) for e in errs)
        flush()
        meta = {"fusion": {"enabled": bool(cfg.enable)}, "shot_branching": False, "measure_sampling": False}
        if noisy:
            meta["noise"] = "kraus"
        matrices = self._conditioned_matrices(items)
        sums = {}
        if matrices is not None and circuit.num_clbits <= 63:
            memory = self._shots_batched(circuit.num_qubits, items, matrices, shots, seed, sums)
            meta["batched_shots_optimization"] = True  # batch_shots_executor.hpp:373
        else:
            memory = self._shots_serial(circuit.num_qubits, items, shots, seed, sums)
        data = {}
        names = {(obj.data if obj.name == "probabilities" else obj.data[0]): obj.name
                 for kind, obj, _ in items if kind == "save"}
        for label, total in sums.items():  # the average over the shots
            avg = total / shots
            data[label] = {"expval": float, "expval_var": lambda a: a.tolist()}.get(names[label], np.asarray)(avg)
        if self._want_memory and circuit.num_clbits:
            data["memory"] = self._memory(memory)
        counts = None
        if circuit.num_clbits:
            counts = {}
            for v in memory:
                key = format(int(v), f"0{circuit.num_clbits}b")
                counts[key] = counts.get(key, 0) + 1
        return {"counts": counts, "data": data, "metadata": meta, "seed_simulator": seed, "shots": shots}

    # saves a circuit run shot by shot supports: each averaged over the shots
    SHOT_SAVES = ("expval", "expval_var", "probabilities")

    @staticmethod
    def _save_shots(st, n, cnt, ins, sums) -> None:
        """A save in a circuit run shot by shot.  The reference averages it
        over the shots (save_data_average, the default `average` subtype of
        save_expval and save_probabilities: Base::apply_save_expval,
        state.hpp:416-447, the probabilities in statevector_state.hpp); here
        each group adds its states' values to a running sum, divided by the
        number of shots at the end."""
        L, h = A.lib(), st.handle
        if ins.name == "probabilities":
            k = len(ins.qubits)
            qarr = (C.c_uint64 * k)(*ins.qubits)
            probs = np.empty((cnt, 1 << k), dtype=np.float64)
            A.check(L.gbqv_probabilities_segments(h, n, cnt, qarr, k, probs.ctypes.data_as(A.dp)), h)
            label, val = ins.data, probs.sum(axis=0)
        else:
            label, terms = ins.data
            if not terms:
                raise ValueError("Invalid save expval instruction (Pauli components are empty).")
            variance = ins.name == "expval_var"
            params = expval_params(terms, variance)
            vals = st.expval_pauli_segments(n, cnt, [ql for ql, _, _ in params])  # [term, state]
            ev, sq = np.zeros(cnt), np.zeros(cnt)
            for (_, c1, c2), v in zip(params, vals):
                ev += c1 * v
                if variance:
                    sq += c2 * v
            val = np.array([ev.sum(), (sq - ev * ev).sum()]) if variance else ev.sum()
        sums[label] = sums[label] + val if label in sums else val

    @staticmethod
    def _conditioned_matrices(items):
        """The matrix of every classically conditioned op, for applying it to
        the shots whose condition holds; None when an item needs the one-shot
        path (a conditioned op on more than 4 qubits)."""
        out = {}
        for idx, (kind, obj, cond) in enumerate(items):
            if kind in ("measure", "reset", "kraus", "save"):
                continue
            if cond is None:
                continue
            ops = obj.ops()
            if len(ops) != 1 or not 1 <= len(ops[0][2]) <= 4 or ops[0][0] not in (0, 1, 2):
                return None
            m = obj.op_matrix(0)
            if ops[0][0] == 2:
                m = np.diag(m).reshape(-1, order="F")
            out[idx] = (ops[0][2], np.ascontiguousarray(m, dtype=np.complex128))
        return out

    def _shot_group_bits(self, n: int, shots: int, ks) -> int:
        """log2 of the shots stacked per group: enough for every shot (up to
        2^SHOT_GROUP_BITS), a stack of at most SHOT_STACK_QUBITS qubits, and a
        group's outcome probabilities (group x 2^k doubles) below 32 MB on the
        host (registers drawn there) and 1 GB on the device (wider ones)."""
        k_host = max([k for k in ks if k <= self.HOST_DRAW_QUBITS], default=0)
        k_dev = max([k for k in ks if k > self.HOST_DRAW_QUBITS], default=0)
        return max(0, min((int(shots) - 1).bit_length(), self.SHOT_GROUP_BITS, self.SHOT_STACK_QUBITS - n,
                          22 - k_host, 27 - k_dev))

    def _draws_per_shot(self, items) -> int:
        """Uniforms one shot consumes at most: one per measure / reset /
        Kraus channel, one per readout error after a measurement."""
        return sum(1 + (len(self._readout_ops([obj])) if kind == "measure" else 0)
                   for kind, obj, _ in items if kind in ("measure", "reset", "kraus"))

    def _shots_batched(self, n, items, matrices, shots, seed, sums):
        L = A.lib()
        ndraw = self._draws_per_shot(items)
        # a Kraus channel's 4^k complex values per state count as 2k + 1 qubits of probabilities
        ks = [len(obj.qubits) if kind != "kraus" else 2 * len(obj.qubits) + 1
              for kind, obj, _ in items
              if kind in ("measure", "reset", "kraus") or (kind == "save" and obj.name == "probabilities")]
        b = self._shot_group_bits(n, shots, ks)
        group = 1 << b
        out = np.zeros(shots, dtype=np.uint64)
        with QubitVector(n + b, self.precision) as st:
            h = st.handle
            if not self.options["blocking_enable"]:
                A.check(L.gbqv_set_blocking(h, 0))
            for g0 in range(0, shots, group):
                cnt = min(group, shots - g0)
                u = np.empty((cnt, ndraw), dtype=np.float64)
                if ndraw:
                    A.check(L.gbqv_uniforms_streams((seed + g0) & (2**64 - 1), cnt, ndraw, u.ctypes.data_as(A.dp)))
                used = np.zeros(cnt, dtype=np.int64)
                memory = np.zeros(cnt, dtype=np.uint64)
                A.check(L.gbqv_initialize_segments(h, n, cnt), h)
                for idx, (kind, obj, cond) in enumerate(items):
                    active = np.ones(cnt, dtype=bool)
                    if cond is not None:
                        cbits, value = cond
                        for i, c in enumerate(cbits):
                            active &= ((memory >> np.uint64(c)) & np.uint64(1)) == ((value >> i) & 1)
                        if not active.any():
                            continue
                    if kind == "save":
                        self._save_shots(st, n, cnt, obj, sums)
                        continue
                    if kind == "ops":
                        if active.all():
                            A.check(L.gbqv_execute_segments(h, obj.handle), h)
                        else:
                            qubits, mat = matrices[idx]
                            mask = active.astype(np.uint8)
                            A.check(L.gbqv_apply_matrix_segments(h, n, cnt, (C.c_uint64 * len(qubits))(*qubits),
                                                                 len(qubits), mat.ctypes.data_as(A.vp),
                                                                 mask.ctypes.data_as(A.vp)), h)
                        continue
                    qubits = obj.qubits
                    k = len(qubits)
                    qarr = (C.c_uint64 * k)(*qubits)
                    rows = np.nonzero(active)[0]
                    if kind == "kraus":
                        self._kraus_apply(st, n, cnt, obj, rows, u[rows, used[rows]])
                        used[rows] += 1
                        continue
                    if k <= self.HOST_DRAW_QUBITS:
                        probs = np.empty((cnt, 1 << k), dtype=np.float64)
                        A.check(L.gbqv_probabilities_segments(h, n, cnt, qarr, k, probs.ctypes.data_as(A.dp)), h)
                        outcome = discrete_draws(probs[rows], u[rows, used[rows]])
                        p_out = probs[rows, outcome]
                    else:
                        ur = np.full(cnt, -1.0)
                        ur[rows] = u[rows, used[rows]]
                        drawn = np.empty(cnt, dtype=np.uint32)
                        pd = np.empty(cnt, dtype=np.float64)
                        A.check(L.gbqv_draw_segments(h, n, cnt, qarr, k, ur.ctypes.data_as(A.dp),
                                                     drawn.ctypes.data_as(A.vp), pd.ctypes.data_as(A.dp)), h)
                        outcome, p_out = drawn[rows].astype(np.int64), pd[rows]
                    used[rows] += 1
                    meas = np.full(cnt, 0xFFFFFFFF, dtype=np.uint32)
                    meas[rows] = outcome
                    final = meas.copy()
                    if kind == "reset":
                        final[rows] = 0
                    scale = np.zeros(cnt, dtype=np.float64)
                    scale[rows] = 1.0 / np.sqrt(p_out)
                    A.check(L.gbqv_collapse_segments(h, n, cnt, qarr, k, meas.ctypes.data_as(A.vp),
                                                     final.ctypes.data_as(A.vp), scale.ctypes.data_as(A.dp)), h)
                    if kind == "measure":
                        o = outcome.astype(np.uint64)
                        for i, c in enumerate(obj.clbits):
                            bit = np.uint64(1) << np.uint64(c)
                            memory[rows] = (memory[rows] & ~bit) | (((o >> np.uint64(i)) & np.uint64(1)) << np.uint64(c))
                        for bits, probs in self._readout_ops([obj]):   # ClassicalRegister::apply_roerror per shot
                            mem = memory[rows]
                            actual = np.zeros(rows.size, dtype=np.int64)
                            for j, b in enumerate(bits):
                                actual |= ((mem >> np.uint64(b)) & np.uint64(1)).astype(np.int64) << j
                            read = discrete_draws(probs[actual], u[rows, used[rows]]).astype(np.uint64)
                            used[rows] += 1
                            for j, b in enumerate(bits):
                                bit = np.uint64(1) << np.uint64(b)
                                mem = (mem & ~bit) | (((read >> np.uint64(j)) & np.uint64(1)) << np.uint64(b))
                            memory[rows] = mem
                out[g0:g0 + cnt] = memory
            st.synchronize()
        return out

    @staticmethod
    def _kraus_apply(st, n, cnt, op: KrausOp, rows, u) -> None:
        """State::apply_kraus on the states `rows` of a stack of cnt states
        of n qubits, each with its uniform u: the operators' probabilities
        from each state's reduced density matrix (one pass; none for a
        mixture of unitaries), the choice per state, then one pass applying
        each state's normalised operator, over the states whose operator
        is not a multiple of the identity."""
        L, h = A.lib(), st.handle
        k, m = len(op.qubits), op.mats.shape[0]
        qarr = (C.c_uint64 * k)(*op.qubits)
        if op.fixed is not None:
            probs = np.broadcast_to(op.fixed, (rows.size, m))
        else:
            D = 1 << k
            rho = np.empty((cnt, D, D), dtype=np.complex128)
            A.check(L.gbqv_rdm_segments(h, n, cnt, qarr, k, rho.ctypes.data_as(A.vp)), h)
            probs = np.einsum("jab,sba->sj", op.gram, rho[rows]).real
        chosen, sc = kraus_draws(probs, u)
        keep = ~(op.ident[chosen] & (np.abs(op.corner[chosen] * sc - 1.0) <= 1e-14))
        if not keep.any():
            return
        branch = np.full(cnt, 255, dtype=np.uint8)
        branch[rows[keep]] = chosen[keep]
        scale = np.zeros(cnt, dtype=np.float64)
        scale[rows[keep]] = sc[keep]
        A.check(L.gbqv_kraus_segments(h, n, cnt, qarr, k, op.colmajor.ctypes.data_as(A.vp), m,
                                      branch.ctypes.data_as(A.vp), scale.ctypes.data_as(A.dp)), h)

    def _shots_serial(self, n, items, shots, seed, sums):
        """One state, one shot at a time (classical memory wider than 63
        bits, or a conditioned op beyond the stacked kernels)."""
        ndraw = self._draws_per_shot(items)
        out = []
        with QubitVector(n, self.precision) as st:
            for shot in range(shots):
                u = uniforms(seed + shot, ndraw) if ndraw else np.empty(0)
                used, memory = 0, 0
                st.initialize()
                for kind, obj, cond in items:
                    if cond is not None:
                        cbits, value = cond
                        if any(((memory >> c) & 1) != ((value >> i) & 1) for i, c in enumerate(cbits)):
                            continue
                    if kind == "ops":
                        A.check(st._L.gbqv_execute(st.handle, obj.handle), st.handle)
                        continue
                    if kind == "kraus":
                        self._kraus_apply(st, n, 1, obj, np.zeros(1, dtype=np.int64), u[used:used + 1])
                        used += 1
                        continue
                    if kind == "save":
                        self._save_shots(st, n, 1, obj, sums)
                        continue
                    qubits = obj.qubits
                    probs = st.probabilities(qubits)
                    outcome = discrete_draw(probs, u[used])
                    used += 1
                    self._collapse(st, qubits, outcome, outcome if kind == "measure" else 0, probs[outcome])
                    if kind == "measure":
                        for i, c in enumerate(obj.clbits):
                            memory = (memory & ~(1 << c)) | (((outcome >> i) & 1) << c)
                        for bits, rp in self._readout_ops([obj]):
                            memory = apply_readout(memory, bits, rp, u[used])
                            used += 1
                out.append(memory)
            st.synchronize()
        return out

    def _run_shots_dm(self, circuit: QuantumCircuit, shots: int, seed: int):
        """The density-matrix method on a circuit that cannot be
        measure-sampled: every shot runs the circuit on one density matrix
        (CircuitExecutor::run_circuit_shots, seed + i per shot).  Noise stays
        superoperators inserted after each gate (under the gate's condition),
        resets are the reset channel, and a measurement draws one outcome and
        projects, D rho D^dag with D = diag(1/sqrt(p) at the outcome)
        (DensityMatrix::State::measure_reset_update,
        densitymatrix_state.hpp:949-990)."""
        items, stretch = [], []
        fused = {"enabled": False}

        def flush():
            if stretch:
                body = self._with_noise(list(stretch))
                kinds = {i.kind for i in body}
                cfg = self.fusion_config(has_superop="superop" in kinds, has_kraus="kraus" in kinds)
                fused["enabled"] |= bool(cfg.enable)
                nc = NativeCircuit(circuit.num_qubits, body)
                nc.fuse(cfg)
                items.append(("ops", nc, None))
                stretch.clear()

        for ins in circuit.data:
            if ins.kind in ("save", "set"):
                raise NotImplementedError(f"{ins.kind} instructions in a circuit run shot by shot")
            if ins.kind == "measure":
                flush()
                errs = self._noise_ops("measure", ins.qubits)
                if errs:  # measure errors act before the measurement, under its condition
                    items.append(("ops", NativeCircuit(circuit.num_qubits, errs), ins.condition))
                items.append(("measure", ins, ins.condition))
            elif ins.condition is not None:
                flush()
                plain = Instruction(ins.kind, ins.name, ins.qubits, ins.params, ins.data, ins.clbits)
                items.append(("ops", NativeCircuit(circuit.num_qubits, self._with_noise([plain])), ins.condition))
            elif ins.kind != "barrier":
                stretch.append(ins)
        flush()
        ndraw = self._draws_per_shot(items)
        memories = []
        with DensityMatrix(circuit.num_qubits, self.precision) as st:
            if not self.options["blocking_enable"]:
                A.check(st._L.gbqv_set_blocking(st.handle, 0))
            for shot in range(shots):
                u = uniforms(seed + shot, ndraw) if ndraw else np.empty(0)
                used, memory = 0, 0
                st.initialize()
                for kind, obj, cond in items:
                    if cond is not None:
                        cbits, value = cond
                        if any(((memory >> c) & 1) != ((value >> i) & 1) for i, c in enumerate(cbits)):
                            continue
                    if kind == "ops":
                        A.check(st._L.gbqv_execute(st.handle, obj.handle), st.handle)
                        continue
                    probs = st.probabilities(obj.qubits)
                    outcome = discrete_draw(probs, u[used])
                    used += 1
                    diag = np.zeros(1 << len(obj.qubits), dtype=complex)
                    diag[outcome] = 1.0 / np.sqrt(probs[outcome])
                    st.apply_diagonal_unitary_matrix(obj.qubits, diag)
                    for i, c in enumerate(obj.clbits):
                        memory = (memory & ~(1 << c)) | (((outcome >> i) & 1) << c)
                    for bits, rp in self._readout_ops([obj]):
                        memory = apply_readout(memory, bits, rp, u[used])
                        used += 1
                memories.append(memory)
            st.synchronize()
        data = {}
        if self._want_memory and circuit.num_clbits:
            data["memory"] = self._memory(memories)
        counts = None
        if circuit.num_clbits:
            counts = {}
            for v in memories:
                key = format(int(v), f"0{circuit.num_clbits}b")
                counts[key] = counts.get(key, 0) + 1
        meta = {"fusion": fused, "shot_branching": False, "measure_sampling": False}
        return {"counts": counts, "data": data, "metadata": meta, "seed_simulator": seed, "shots": shots}

    @staticmethod
    def _collapse(st, qubits, meas_state: int, final_state: int, prob: float):
        """measure_reset_update on one state: the amplitude of meas_state
        times 1/sqrt(p) moves to final_state, the others become 0 (the
        stacked collapse kernel on a stack of one state, any register
        width)."""
        k = len(qubits)
        qarr = (C.c_uint64 * k)(*qubits)
        meas = np.array([meas_state], dtype=np.uint32)
        final = np.array([final_state], dtype=np.uint32)
        scale = np.array([1.0 / np.sqrt(prob)])
        A.check(A.lib().gbqv_collapse_segments(st.handle, st.num_qubits(), 1, qarr, k, meas.ctypes.data_as(A.vp),
                                               final.ctypes.data_as(A.vp), scale.ctypes.data_as(A.dp)), st.handle)

    def _readout_ops(self, meas) -> list:
        """Readout errors after the measurements, in order: (clbits, probs)."""
        if self.noise_model is None or not self.noise_model.has_readout_errors():
            return []
        return [op for m in meas for op in self.noise_model.readout_ops(m.qubits, m.clbits)]

    @staticmethod
    def _readout_sampled(memory, ro, u) -> list:
        """Executor::measure_sampler with readout errors
        (circuit_executor.hpp:1097-1121): after the samples have taken the
        stream's first `shots` draws, the samples are walked from the last to
        the first, each readout error drawing the stream's next uniform; the
        memories come out in that order."""
        out, k = [], 0
        for i in range(len(memory) - 1, -1, -1):
            m = int(memory[i])
            for bits, probs in ro:
                m = apply_readout(m, bits, probs, float(u[k]))
                k += 1
            out.append(m)
        return out

    @staticmethod
    def _counts_of(memory, num_clbits: int) -> dict:
        counts = {}
        for v in memory:
            key = format(int(v), f"0{num_clbits}b")
            counts[key] = counts.get(key, 0) + 1
        return counts

    @staticmethod
    def _memory_values(samples, qubits, clbits):
        """Classical memory per shot (measured qubit q -> clbit c)."""
        memory = np.zeros(samples.size, dtype=np.uint64)
        for q, c in zip(qubits, clbits):
            memory |= ((samples >> np.uint64(q)) & np.uint64(1)) << np.uint64(c)
        return memory

    @classmethod
    def _counts(cls, samples, qubits, clbits, num_clbits):
        vals, cnt = np.unique(cls._memory_values(samples, qubits, clbits), return_counts=True)
        return {format(int(v), f"0{num_clbits}b"): int(n) for v, n in zip(vals, cnt)}

    @staticmethod
    def _memory(values):
        """Per-shot memory in the reference's hex form (ExperimentResult
        memory, one "0x..." string per shot in draw order)."""
        return [hex(int(v)) for v in values]

    def _check_unitary_circuit(self, circuit: QuantumCircuit):
        """The unitary method's op set (QubitUnitary::StateOpSet,
        unitary_state.hpp:35-54): gates, unitary / diagonal matrices,
        barriers, save_unitary."""
        if self.noise_model is not None and not self.noise_model.is_ideal():
            raise ValueError("the unitary method does not support noise")
        for ins in circuit.data:
            if ins.kind in ("gate", "unitary", "diagonal", "barrier"):
                continue
            if ins.kind in ("save", "set") and ins.name == "unitary" or ins.kind == "save" and ins.name == "state":
                continue
            raise ValueError(f"QubitUnitary::State::invalid instruction '{ins.name}'.")

    def _set_state(self, st, ins):
        """A set instruction: the state becomes the given one.  The
        density-matrix method takes a statevector as the pure state
        |v><v| (DensityMatrix::initialize_from_vector) or a density matrix;
        the unitary method a unitary; the statevector method a statevector."""
        allowed = {"statevector": ("statevector",), "density_matrix": ("statevector", "density_matrix"),
                   "unitary": ("unitary",)}[self.method]
        if ins.name not in allowed:
            raise ValueError(f"set_{ins.name} is not supported by the {self.method} method")
        if ins.name == "statevector" and self.method == "density_matrix":
            st.initialize_from_matrix(np.outer(ins.data, np.conj(ins.data)))
        elif ins.name == "statevector":
            st.initialize_from_vector(ins.data)
        else:
            st.initialize_from_matrix(ins.data)

    def _save(self, st, ins, data):
        if ins.kind == "set":
            self._set_state(st, ins)
        elif ins.name == "state":
            key = self.method if ins.data == "_method_" else ins.data
            data[key] = st.copy_to_vector() if self.method == "statevector" else st.copy_to_matrix()
        elif ins.name == "unitary":
            data[ins.data] = st.copy_to_matrix()
        elif ins.name == "statevector":
            data[ins.data] = st.copy_to_vector()
        elif ins.name == "density_matrix":
            data[ins.data] = st.copy_to_matrix()
        elif ins.name == "probabilities":
            data[ins.data] = st.probabilities(ins.qubits)
        elif ins.name in ("expval", "expval_var"):
            # Base::apply_save_expval (state.hpp:416-447) over the reference's
            # parameters: real coefficients of O (and of O.O for the variance)
            label, terms = ins.data
            if not terms:
                raise ValueError("Invalid save expval instruction (Pauli components are empty).")
            variance = ins.name == "expval_var"
            params = expval_params(terms, variance)
            vals, _ = st.expval_pauli_many([ql for ql, _, _ in params])
            expval, sq = 0.0, 0.0
            for (_, c1, c2), v in zip(params, vals):
                expval += c1 * float(v)
                if variance:
                    sq += c2 * float(v)
            data[label] = [expval, sq - expval * expval] if variance else expval
        elif ins.name in ("amplitudes", "amplitudes_squared"):
            label, idx = ins.data
            if not idx:
                raise ValueError("Invalid save_amplitudes instructions (empty params).")
            if ins.name == "amplitudes":
                if isinstance(st, (DensityMatrix, UnitaryMatrix)):
                    raise ValueError("save_amplitudes needs the statevector method")
                vec = st.copy_to_vector()
                data[label] = np.array([vec[i] for i in idx], dtype=complex)
            else:
                probs = st.probabilities()
                data[label] = np.array([probs[i] for i in idx], dtype=np.float64)
        elif ins.name == "probabilities_dict":
            probs = st.probabilities(ins.qubits)
            data[ins.data] = ket_dict(probs, self.CHOP_THRESHOLD)
        elif ins.name == "statevector_dict":
            if isinstance(st, (DensityMatrix, UnitaryMatrix)):
                raise ValueError("save_statevector_dict needs the statevector method")
            vec = st.copy_to_vector()
            data[ins.data] = ket_dict(vec, self.CHOP_THRESHOLD)
