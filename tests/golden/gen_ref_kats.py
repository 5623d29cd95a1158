"""Generate ref_kats.json: the reference's own known-answer tests for gates.

The reference's test suite holds hand-written circuits with exact target
statevectors, unitaries and counts in test/terra/reference/ref_1q_clifford.py,
ref_2q_clifford.py, ref_non_clifford.py and ref_rotation.py.  They build
their circuits with qiskit's QuantumCircuit, and qiskit is not installed
here.  This script puts a minimal recording stand-in for qiskit's circuit
builder in sys.modules.  It imports those four files from the reference
tree, calls every ``*_circuits_*`` function with final_measure=False and
the matching ``*_statevector_*``, ``*_unitary_*`` and ``*_counts_*``
functions, and writes each circuit (gate name, qubits, parameters) with its
targets.

Usage:  python tests/golden/gen_ref_kats.py [reference test dir]
(default: the reference checkout's test/terra/reference folder).
"""
from __future__ import annotations

import importlib.util
import json
import sys
import types
from pathlib import Path

import numpy as np

OUT = Path(__file__).resolve().parent / "ref_kats.json"
DEFAULT_DIR = Path("/root/reference/test/terra/reference")
FILES = ("ref_1q_clifford", "ref_2q_clifford", "ref_non_clifford", "ref_rotation")
SHOTS = 4096


class _Bit:
    def __init__(self, reg, index):
        self.reg, self.index = reg, index


class _Register:
    def __init__(self, size, name=None):
        self.size = int(size)
        self.name = name

    def __len__(self):
        return self.size

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [_Bit(self, j) for j in range(self.size)[i]]
        if i < 0:
            i += self.size
        if not 0 <= i < self.size:
            raise IndexError(i)
        return _Bit(self, i)

    def __iter__(self):
        return (_Bit(self, j) for j in range(self.size))


class QuantumRegister(_Register):
    pass


class ClassicalRegister(_Register):
    pass


# qiskit gate methods used by the four files: (number of qubit arguments, number of parameters)
_GATES = {
    "h": (1, 0), "x": (1, 0), "y": (1, 0), "z": (1, 0), "s": (1, 0), "sdg": (1, 0), "t": (1, 0), "tdg": (1, 0),
    "id": (1, 0), "rx": (1, 1), "ry": (1, 1), "rz": (1, 1), "cx": (2, 0), "cz": (2, 0), "swap": (2, 0),
    "ecr": (2, 0), "cp": (2, 1), "cu": (2, 4), "ccx": (3, 0), "cswap": (3, 0),
}
# number of leading control qubits of the controlled gates
_CONTROLS = {"cx": 1, "cz": 1, "cp": 1, "cu": 1, "ccx": 2, "cswap": 1}


class QuantumCircuit:
    """Records gates as (name, qubit indices, parameters).  A register
    argument broadcasts the gate over its qubits, as qiskit does."""

    def __init__(self, *regs, name=None):
        self.offsets, self.num_qubits = {}, 0
        for r in regs:
            if isinstance(r, QuantumRegister):
                self.offsets[id(r)] = self.num_qubits
                self.num_qubits += r.size
        self.ops = []

    def _targets(self, arg):
        if isinstance(arg, _Bit):
            return [self.offsets[id(arg.reg)] + arg.index]
        if isinstance(arg, QuantumRegister):
            return [self.offsets[id(arg)] + j for j in range(arg.size)]
        if isinstance(arg, (list, tuple)):
            return [q for a in arg for q in self._targets(a)]
        return [int(arg)]

    def _gate(self, name, nq, npar, args, ctrl_state=None):
        params, qargs = list(args[:npar]), args[npar:npar + nq]
        if len(qargs) != nq:
            raise TypeError(f"{name}: expected {nq} qubit arguments")
        lists = [self._targets(a) for a in qargs]
        width = max(len(x) for x in lists)
        for j in range(width):
            qs = [x[j] if len(x) > 1 else x[0] for x in lists]
            # an open control (ctrl_state bit i = 0 for control i) is the gate
            # conjugated by X on that control, as qiskit lowers it
            flips = []
            if ctrl_state is not None:
                state = int(ctrl_state, 2) if isinstance(ctrl_state, str) else int(ctrl_state)
                flips = [qs[i] for i in range(_CONTROLS[name]) if not (state >> i) & 1]
            self.ops.extend(["x", [q], []] for q in flips)
            self.ops.append([name, qs, [float(p) for p in params]])
            self.ops.extend(["x", [q], []] for q in flips)
        return self

    def __getattr__(self, name):
        if name in _GATES:
            nq, npar = _GATES[name]
            return lambda *args, ctrl_state=None, **kw: self._gate(name, nq, npar, args, ctrl_state)
        raise AttributeError(name)

    def barrier(self, *args, **kw):
        return self

    def measure(self, *args, **kw):
        raise AssertionError("circuits are generated with final_measure=False")

    def delay(self, duration, qarg=None, unit="dt"):
        for q in self._targets(qarg):
            self.ops.append(["delay", [q], []])
        return self

    def pauli(self, label, qargs):
        # PauliGate: label character -1-i acts on qargs[i]
        qs = self._targets(qargs)
        for i, q in enumerate(qs):
            ch = label[len(label) - 1 - i].lower()
            self.ops.append(["id" if ch == "i" else ch, [q], []])
        return self


def _install_stub():
    mod = types.ModuleType("qiskit")
    mod.QuantumRegister, mod.ClassicalRegister, mod.QuantumCircuit = QuantumRegister, ClassicalRegister, QuantumCircuit
    sys.modules["qiskit"] = mod


def _load(path: Path):
    spec = importlib.util.spec_from_file_location(path.stem, path)
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def _cplx(a):
    a = np.asarray(a, dtype=complex).reshape(-1)
    return [[float(z.real), float(z.imag)] for z in a]


def main(ref_dir: Path = DEFAULT_DIR):
    _install_stub()
    cases = []
    for fname in FILES:
        m = _load(ref_dir / f"{fname}.py")
        for attr in sorted(dir(m)):
            if "_circuits_" not in attr:
                continue
            stem, kind = attr.split("_circuits_")
            circuits = getattr(m, attr)(final_measure=False)
            targets = {}
            for t in ("statevector", "unitary", "counts"):
                f = getattr(m, f"{stem}_{t}_{kind}", None)
                if f is not None:
                    targets[t] = f(SHOTS, hex_counts=True) if t == "counts" else f()
            # circuits and targets pair by position up to the shorter list, as
            # the reference's compare_* helpers zip them (a few lists differ in length)
            for i, qc in enumerate(circuits):
                case = {"source": f"{fname}.py:{attr}", "index": i, "num_qubits": qc.num_qubits, "ops": qc.ops}
                if i < len(targets.get("statevector", ())):
                    case["statevector"] = _cplx(targets["statevector"][i])
                if i < len(targets.get("unitary", ())):
                    u = np.asarray(targets["unitary"][i], dtype=complex)
                    case["unitary"] = _cplx(u.reshape(-1, order="F"))  # column-major, as the engine's matrices
                if i < len(targets.get("counts", ())):
                    case["probabilities"] = {str(int(k, 16)): v / SHOTS for k, v in targets["counts"][i].items()}
                if len(case) > 4:
                    cases.append(case)
    OUT.write_text(json.dumps({"shots": SHOTS, "cases": cases}, indent=0))
    print(f"{len(cases)} cases -> {OUT}")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_DIR)
