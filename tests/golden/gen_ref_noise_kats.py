"""Generate ref_noise_kats.json: the reference's own known-answer tests for
noise models.

test/terra/reference/ref_pauli_noise.py, ref_reset_noise.py and
ref_kraus_noise.py pair small circuits (gates, reset, final measurements)
with noise models: Pauli, reset and amplitude-damping errors on gates, on
reset and on measure.  ref_readout_noise.py does the same with readout
errors, on single measurements and on one 2-qubit measurement.  All four
files give the exact outcome distributions as counts of a number of shots.
ref_reset.py adds reset circuits, noiseless, with their distributions.
They need qiskit's circuit builder and qiskit_aer's noise module; neither
is importable here.  This script puts recording stand-ins for both in
sys.modules, imports the five files from the reference tree and writes,
per case: the circuit (instruction kind,
name, qubits, parameters, classical bits), the noise model as the list of
add_*_quantum_error calls with the error constructor and its arguments
(readout cases: the add_*_readout_error calls with their matrices), and the
target probabilities (counts / shots).

Usage:  python tests/golden/gen_ref_noise_kats.py [reference test dir]
(default: the reference checkout's test/terra/reference folder).
"""
from __future__ import annotations

import importlib.util
import json
import sys
import types
from pathlib import Path

OUT = Path(__file__).resolve().parent / "ref_noise_kats.json"
DEFAULT_DIR = Path("/root/reference/test/terra/reference")
# (file, stem): stem_circuits(), stem_noise_models(), stem_counts(shots)
SETS = (("ref_pauli_noise", "pauli_gate_error"), ("ref_pauli_noise", "pauli_measure_error"),
        ("ref_pauli_noise", "pauli_reset_error"), ("ref_reset_noise", "reset_gate_error"),
        ("ref_kraus_noise", "kraus_gate_error"))
READOUT_SETS = (("ref_readout_noise", "readout_error"),)
# ref_reset.py: (circuits function, counts function), circuits that end in
# their only measurements (reset_circuits_repeated measures mid-circuit and is left out)
RESET_SETS = (("reset_circuits_deterministic", "reset_counts_deterministic"),
              ("reset_circuits_nondeterministic", "reset_counts_nondeterministic"),
              ("reset_circuits_sampling_optimization", "reset_counts_sampling_optimization"),
              ("reset_circuits_with_entangled_and_moving_qubits", "reset_counts_with_entangled_and_moving_qubits"))
SHOTS = 4096


class _Bit:
    def __init__(self, reg, index):
        self.reg, self.index = reg, index


class _Register:
    def __init__(self, size, name=None):
        self.size, self.name = int(size), name

    def __len__(self):
        return self.size

    def __getitem__(self, i):
        return _Bit(self, i + self.size if i < 0 else i)

    def __iter__(self):
        return (_Bit(self, j) for j in range(self.size))


class QuantumRegister(_Register):
    pass


class ClassicalRegister(_Register):
    pass


class QuantumCircuit:
    """Records [kind, name, qubits, params, clbits]; register arguments
    broadcast one instruction per bit, as qiskit does."""

    def __init__(self, *regs, name=None):
        self.qoff, self.coff, self.num_qubits, self.num_clbits = {}, {}, 0, 0
        for r in regs:
            if isinstance(r, QuantumRegister):
                self.qoff[id(r)] = self.num_qubits
                self.num_qubits += r.size
            else:
                self.coff[id(r)] = self.num_clbits
                self.num_clbits += r.size
        self.ops = []

    def _bits(self, arg, table):
        if isinstance(arg, _Bit):
            return [table[id(arg.reg)] + arg.index]
        if isinstance(arg, _Register):
            return [table[id(arg)] + j for j in range(arg.size)]
        if isinstance(arg, (list, tuple)):
            return [b for a in arg for b in self._bits(a, table)]
        return [int(arg)]

    def _one_qubit(self, kind, name, arg):
        for q in self._bits(arg, self.qoff):
            self.ops.append([kind, name, [q], [], []])
        return self

    def x(self, q):
        return self._one_qubit("gate", "x", q)

    def h(self, q):
        return self._one_qubit("gate", "h", q)

    def cx(self, c, t):
        for a, b in zip(self._bits(c, self.qoff), self._bits(t, self.qoff)):
            self.ops.append(["gate", "cx", [a, b], [], []])
        return self

    def append(self, instruction, qargs, cargs=()):
        if instruction.name != "measure":
            raise AssertionError(f"unexpected instruction {instruction.name}")
        # one measure over all of its qubits (a multi-qubit measurement)
        self.ops.append(["measure", "measure", self._bits(list(qargs), self.qoff), [],
                         self._bits(list(cargs), self.coff)])
        return self

    def id(self, q):
        return self._one_qubit("gate", "id", q)

    def reset(self, q):
        return self._one_qubit("reset", "reset", q)

    def barrier(self, *args, **kw):
        return self

    def measure(self, qarg, carg):
        for q, c in zip(self._bits(qarg, self.qoff), self._bits(carg, self.coff)):
            self.ops.append(["measure", "measure", [q], [], [c]])
        return self


def _plain(v):
    if isinstance(v, (list, tuple)):
        return [_plain(x) for x in v]
    return v


class _ErrorSpec:
    """An error constructor call: its name and arguments."""

    def __init__(self, fn, args, kwargs):
        self.spec = {"fn": fn, "args": _plain(list(args)), "kwargs": _plain(dict(kwargs))}


def _ctor(fn):
    return lambda *args, **kw: _ErrorSpec(fn, args, kw)


class Instruction:
    def __init__(self, name, num_qubits, num_clbits, params):
        self.name, self.num_qubits, self.num_clbits, self.params = name, num_qubits, num_clbits, params


class NoiseModel:
    def __init__(self, *args, **kw):
        self.calls = []

    def add_readout_error(self, error, qubits, warnings=True):
        self.calls.append({"call": "add_readout_error", "matrix": _plain(error), "qubits": [int(q) for q in qubits]})

    def add_all_qubit_readout_error(self, error, warnings=True):
        self.calls.append({"call": "add_all_qubit_readout_error", "matrix": _plain(error)})

    def add_all_qubit_quantum_error(self, error, instructions, warnings=True):
        names = [instructions] if isinstance(instructions, str) else list(instructions)
        self.calls.append({"call": "add_all_qubit_quantum_error", "error": error.spec, "instructions": names})

    def add_quantum_error(self, error, instructions, qubits, warnings=True):
        names = [instructions] if isinstance(instructions, str) else list(instructions)
        self.calls.append({"call": "add_quantum_error", "error": error.spec, "instructions": names,
                           "qubits": [int(q) for q in qubits]})


def _list2dict(counts_list, hex_counts=True):
    # the reference's test helper (test/terra/utils/utils.py:20-33), hex keys only
    assert hex_counts
    return {hex(i): val for i, val in enumerate(counts_list) if val > 0}


def _install_stubs():
    def module(name, **attrs):
        m = types.ModuleType(name)
        for k, v in attrs.items():
            setattr(m, k, v)
        sys.modules[name] = m
        return m

    module("qiskit", QuantumRegister=QuantumRegister, ClassicalRegister=ClassicalRegister,
           QuantumCircuit=QuantumCircuit)
    module("qiskit.circuit", Instruction=Instruction)
    errors = dict(QuantumError=_ErrorSpec, PauliError=_ctor("PauliError"))
    std = {f: _ctor(f) for f in ("pauli_error", "reset_error", "amplitude_damping_error", "depolarizing_error",
                                 "kraus_error", "thermal_relaxation_error")}
    module("qiskit_aer")
    module("qiskit_aer.noise", NoiseModel=NoiseModel, **errors)
    module("qiskit_aer.noise.errors", **errors)
    module("qiskit_aer.noise.errors.standard_errors", **std)
    module("test")
    module("test.terra")
    module("test.terra.utils")
    module("test.terra.utils.utils", list2dict=_list2dict)


def _load(path: Path):
    spec = importlib.util.spec_from_file_location(path.stem, path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def main(ref_dir: Path = DEFAULT_DIR):
    _install_stubs()
    cases, readout_cases = [], []
    for fname, stem in SETS + READOUT_SETS:
        m = _load(ref_dir / f"{fname}.py")
        circuits = getattr(m, f"{stem}_circuits")()
        models = getattr(m, f"{stem}_noise_models")()
        counts = getattr(m, f"{stem}_counts")(SHOTS)
        # paired by position, as the reference's tests zip them
        for i, (qc, nm, ct) in enumerate(zip(circuits, models, counts)):
            (readout_cases if (fname, stem) in READOUT_SETS else cases).append({"source": f"{fname}.py:{stem}", "index": i, "num_qubits": qc.num_qubits,
                          "num_clbits": qc.num_clbits, "ops": qc.ops, "noise": nm.calls,
                          "probabilities": {str(int(k, 16)): v / SHOTS for k, v in ct.items()}})
    reset_cases = []
    m = _load(ref_dir / "ref_reset.py")
    for circ_fn, count_fn in RESET_SETS:
        for i, (qc, ct) in enumerate(zip(getattr(m, circ_fn)(), getattr(m, count_fn)(SHOTS))):
            reset_cases.append({"source": f"ref_reset.py:{circ_fn}", "index": i, "num_qubits": qc.num_qubits,
                                "num_clbits": qc.num_clbits, "ops": qc.ops, "noise": [],
                                "probabilities": {str(int(k, 16)): v / SHOTS for k, v in ct.items()}})
    OUT.write_text(json.dumps({"shots": SHOTS, "cases": cases, "readout_cases": readout_cases,
                               "reset_cases": reset_cases}, indent=0))
    print(f"{len(cases)} + {len(readout_cases)} readout + {len(reset_cases)} reset cases -> {OUT}")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_DIR)
