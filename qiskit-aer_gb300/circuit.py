"""A minimal circuit builder (qiskit is not a dependency) whose instructions
assemble into the engine's op list the way ``aer_compiler._assemble_op``
(qiskit_aer/backends/aer_compiler.py:875-1020) assembles qiskit instructions
into AerCircuit ops: named gates, ``unitary``, ``diagonal``, ``superop``,
``kraus``, ``reset``, ``barrier``, ``measure`` and the save instructions
``save_statevector`` / ``save_statevector_dict`` / ``save_density_matrix``
/ ``save_unitary`` / ``save_probabilities`` / ``save_probabilities_dict`` /
``save_amplitudes`` / ``save_amplitudes_squared`` /
``save_expectation_value`` / ``save_expectation_value_variance``
(qiskit_aer/library/save_instructions/).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _capi as A


class ParameterExpression:
    """A real affine expression c0 + sum_p c_p * p over Parameters: the part of
    qiskit's ParameterExpression that parameter binding uses (the Python side
    of the reference evaluates each bound expression per binding,
    qiskit_aer/backends/aerbackend.py:96-126)."""

    __slots__ = ("_terms", "_const")

    def __init__(self, terms=None, const: float = 0.0):
        self._terms = dict(terms or {})
        self._const = float(const)

    @property
    def parameters(self) -> set:
        return {p for p, c in self._terms.items() if c != 0.0}

    @staticmethod
    def _coerce(x) -> "ParameterExpression":
        if isinstance(x, ParameterExpression):
            return x
        if np.ndim(x) != 0 or np.iscomplexobj(x):
            raise TypeError(f"cannot combine a parameter with {x!r}")
        return ParameterExpression({}, float(x))

    def _combine(self, other, sign: float) -> "ParameterExpression":
        o = self._coerce(other)
        terms = dict(self._terms)
        for p, c in o._terms.items():
            terms[p] = terms.get(p, 0.0) + sign * c
        return ParameterExpression(terms, self._const + sign * o._const)

    def _scale(self, k) -> "ParameterExpression":
        if isinstance(k, ParameterExpression):
            if k.parameters and self.parameters:
                raise TypeError("only affine parameter expressions are supported")
            if k.parameters:
                return k._scale(self._const)
            k = k._const
        k = float(k)
        return ParameterExpression({p: c * k for p, c in self._terms.items()}, self._const * k)

    def __add__(self, o): return self._combine(o, 1.0)
    def __radd__(self, o): return self._combine(o, 1.0)
    def __sub__(self, o): return self._combine(o, -1.0)
    def __rsub__(self, o): return self._coerce(o)._combine(self, -1.0)
    def __mul__(self, k): return self._scale(k)
    def __rmul__(self, k): return self._scale(k)
    def __truediv__(self, k): return self._scale(1.0 / float(k))
    def __neg__(self): return self._scale(-1.0)
    def __pos__(self): return self

    def bind(self, values: dict) -> "ParameterExpression | float":
        """Substitute the parameters found in `values`; a float once none is left."""
        terms, const = {}, self._const
        for p, c in self._terms.items():
            if p in values:
                const += c * float(values[p])
            else:
                terms[p] = c
        return ParameterExpression(terms, const) if any(c != 0.0 for c in terms.values()) else const

    def evaluate(self, binds: dict) -> np.ndarray:
        """Values of the expression for every binding: binds maps each of its
        parameters to an array of values (one per binding)."""
        out = None
        for p, c in self._terms.items():
            if c == 0.0:
                continue
            if p not in binds:
                raise ValueError(f"no values bound to parameter '{p.name}'")
            v = c * np.asarray(binds[p], dtype=np.float64)
            out = v if out is None else out + v
        if out is None:
            raise ValueError("the expression has no parameter")
        return out + self._const

    def __float__(self):
        if self.parameters:
            raise TypeError(f"unbound parameters: {sorted(p.name for p in self.parameters)}")
        return self._const

    def __repr__(self):
        parts = [f"{c:g}*{p.name}" for p, c in self._terms.items() if c != 0.0]
        if self._const or not parts:
            parts.append(f"{self._const:g}")
        return " + ".join(parts)


class Parameter(ParameterExpression):
    """A named circuit parameter (qiskit.circuit.Parameter); identity-hashed."""

    __slots__ = ("name",)

    def __init__(self, name: str):
        super().__init__({}, 0.0)
        self.name = str(name)
        self._terms[self] = 1.0

    __hash__ = object.__hash__

    def __eq__(self, other):
        return self is other

    def __repr__(self):
        return f"Parameter({self.name})"


def _param(x):
    """A gate parameter as stored: a float, or an expression with parameters."""
    if isinstance(x, ParameterExpression):
        return x if x.parameters else float(x)
    return float(x)


@dataclass
class Instruction:
    kind: str                      # "gate" | "unitary" | "diagonal" | "superop" | "kraus" | "reset" | "barrier" | "measure" | "save" | "set"
    name: str
    qubits: list
    params: list = field(default_factory=list)
    data: object = None            # matrix / diagonal / kraus list / save payload
    clbits: list = field(default_factory=list)
    # classical condition (clbits, value): applied only when the memory bits
    # clbits[i] equal bit i of value (Operations::Op conditional, checked by
    # ClassicalRegister::check_conditional before each op)
    condition: tuple | None = None


class QuantumCircuit:
    def __init__(self, num_qubits: int, num_clbits: int = 0, name: str = "circuit", metadata: dict | None = None):
        self.num_qubits = int(num_qubits)
        self.num_clbits = int(num_clbits)
        self.name = name
        self.metadata = dict(metadata or {})
        self.creg_name = "c"  # the classical register's name ("meas" after measure_all, as qiskit names it)
        self.data: list[Instruction] = []

    # ---- generic ----
    def append_gate(self, name: str, qubits, params=()):
        self.data.append(Instruction("gate", name, [int(q) for q in qubits], [_param(p) for p in params]))
        return self

    # ---- parameters ----
    @property
    def parameters(self) -> list:
        """The circuit's unbound parameters, sorted by name (qiskit's order)."""
        found = {}
        for ins in self.data:
            for p in ins.params:
                if isinstance(p, ParameterExpression):
                    for q in p.parameters:
                        found[id(q)] = q
        return sorted(found.values(), key=lambda q: q.name)

    @property
    def num_parameters(self) -> int:
        return len(self.parameters)

    def copy(self) -> "QuantumCircuit":
        out = QuantumCircuit(self.num_qubits, self.num_clbits, self.name, self.metadata)
        out.creg_name = self.creg_name
        out.data = [Instruction(i.kind, i.name, list(i.qubits), list(i.params), i.data, list(i.clbits), i.condition)
                    for i in self.data]
        return out

    def assign_parameters(self, values) -> "QuantumCircuit":
        """A copy with parameters replaced: values is a dict {Parameter: value}
        or a sequence in the order of `parameters`."""
        if not isinstance(values, dict):
            params = self.parameters
            values = list(values)
            if len(values) != len(params):
                raise ValueError(f"{len(values)} values for {len(params)} parameters")
            values = dict(zip(params, values))
        out = self.copy()
        for ins in out.data:
            ins.params = [p.bind(values) if isinstance(p, ParameterExpression) else p for p in ins.params]
        return out

    def unitary(self, mat, qubits, label="unitary"):
        self.data.append(Instruction("unitary", label, [int(q) for q in qubits], data=np.asarray(mat, dtype=complex)))
        return self

    def diagonal(self, diag, qubits):
        self.data.append(Instruction("diagonal", "diagonal", [int(q) for q in qubits], data=np.asarray(diag, dtype=complex)))
        return self

    def superop(self, mat, qubits):
        self.data.append(Instruction("superop", "superop", [int(q) for q in qubits], data=np.asarray(mat, dtype=complex)))
        return self

    def kraus(self, mats, qubits):
        self.data.append(Instruction("kraus", "kraus", [int(q) for q in qubits], data=[np.asarray(m, dtype=complex) for m in mats]))
        return self

    def reset(self, qubits):
        qubits = [qubits] if np.isscalar(qubits) else qubits
        self.data.append(Instruction("reset", "reset", [int(q) for q in qubits]))
        return self

    def barrier(self, *qubits):
        self.data.append(Instruction("barrier", "barrier", [int(q) for q in qubits]))
        return self

    def measure(self, qubits, clbits):
        qubits = [qubits] if np.isscalar(qubits) else qubits
        clbits = [clbits] if np.isscalar(clbits) else clbits
        self.num_clbits = max(self.num_clbits, max(clbits) + 1)
        self.data.append(Instruction("measure", "measure", [int(q) for q in qubits], clbits=[int(c) for c in clbits]))
        return self

    def measure_all(self):
        if self.num_clbits == 0:
            self.creg_name = "meas"
        return self.measure(list(range(self.num_qubits)), list(range(self.num_qubits)))

    def c_if(self, clbits, value: int):
        """Condition the last instruction on classical bits (qiskit's c_if on
        a register made of `clbits`, least significant first)."""
        clbits = [clbits] if np.isscalar(clbits) else clbits
        if not self.data:
            raise ValueError("c_if needs an instruction to condition")
        self.num_clbits = max(self.num_clbits, max(clbits) + 1)
        self.data[-1].condition = ([int(c) for c in clbits], int(value))
        return self

    def needs_shots(self, method: str = "statevector") -> bool:
        """True when measure sampling does not apply and every shot runs the
        circuit (Executor::check_measure_sampling_opt): a measurement followed
        by other ops, a classical condition, or, on a statevector, a reset or
        a Kraus channel."""
        seen_measure = False
        for ins in self.data:
            if ins.condition is not None:
                return True
            if ins.kind == "measure":
                seen_measure = True
            elif ins.kind not in ("save", "barrier") and seen_measure:  # a set after a measure too
                return True
            if method == "statevector" and ins.kind in ("reset", "kraus"):
                return True
        return False

    # ---- set instructions (qiskit_aer/library/set_instructions: SetStatevector,
    # SetDensityMatrix, SetUnitary; applied as the state's initialize_from_vector /
    # initialize_from_matrix, statevector_state.hpp:538-540,
    # densitymatrix_state.hpp:456-461) ----
    def set_statevector(self, state):
        v = np.asarray(state, dtype=complex).reshape(-1)
        if v.size != 1 << self.num_qubits:
            raise ValueError("The size of the statevector for the set_statevector instruction must be equal to "
                             "the number of qubits")
        self.data.append(Instruction("set", "statevector", list(range(self.num_qubits)), data=v))
        return self

    def set_density_matrix(self, state):
        m = np.asarray(state, dtype=complex)
        d = 1 << self.num_qubits
        if m.shape != (d, d):
            raise ValueError("The size of the density matrix for the set_density_matrix instruction must be "
                             "equal to the number of qubits")
        self.data.append(Instruction("set", "density_matrix", list(range(self.num_qubits)), data=m))
        return self

    def set_unitary(self, state):
        m = np.asarray(state, dtype=complex)
        d = 1 << self.num_qubits
        if m.shape != (d, d):
            raise ValueError("The size of the unitary matrix for the set_unitary instruction must be equal to "
                             "the number of qubits")
        self.data.append(Instruction("set", "unitary", list(range(self.num_qubits)), data=m))
        return self

    def save_state(self, label=None):
        """The method's own state (SaveState, qiskit_aer/library/save_instructions/
        save_state.py): the statevector, density matrix or unitary, saved
        under the method's name unless a label is given
        (statevector_state.hpp:597-615)."""
        self.data.append(Instruction("save", "state", [], data="_method_" if label is None else label))
        return self

    def save_statevector(self, label="statevector"):
        self.data.append(Instruction("save", "statevector", [], data=label))
        return self

    def save_density_matrix(self, label="density_matrix"):
        self.data.append(Instruction("save", "density_matrix", [], data=label))
        return self

    def save_unitary(self, label="unitary"):
        self.data.append(Instruction("save", "unitary", [], data=label))
        return self

    def save_probabilities(self, qubits=None, label="probabilities"):
        q = list(range(self.num_qubits)) if qubits is None else [int(x) for x in qubits]
        self.data.append(Instruction("save", "probabilities", q, data=label))
        return self

    def save_expectation_value(self, terms, label="expectation_value"):
        """terms: list of (coeff, label, qubits) — the (pauli, coeff) list
        SaveExpectationValue builds (save_expectation_value.py:61-68)."""
        self.data.append(Instruction("save", "expval", [], data=(label, list(terms))))
        return self

    def save_expectation_value_variance(self, terms, label="expectation_value_variance"):
        """[<O>, <O^2> - <O>^2] (SaveExpectationValueVariance,
        save_expectation_value.py:100-135)."""
        self.data.append(Instruction("save", "expval_var", [], data=(label, list(terms))))
        return self

    def save_amplitudes(self, params, label="amplitudes"):
        """Amplitudes of the listed basis states (statevector method,
        State::apply_save_amplitudes, statevector_state.hpp:654-679)."""
        self.data.append(Instruction("save", "amplitudes", [], data=(label, [int(i) for i in params])))
        return self

    def save_amplitudes_squared(self, params, label="amplitudes_squared"):
        self.data.append(Instruction("save", "amplitudes_squared", [], data=(label, [int(i) for i in params])))
        return self

    def save_probabilities_dict(self, qubits=None, label="probabilities_dict"):
        """Probabilities as {hex outcome: p}, entries above the chop threshold
        (save_probs_ket, statevector_state.hpp:575-588)."""
        q = list(range(self.num_qubits)) if qubits is None else [int(x) for x in qubits]
        self.data.append(Instruction("save", "probabilities_dict", q, data=label))
        return self

    def save_statevector_dict(self, label="statevector_dict"):
        self.data.append(Instruction("save", "statevector_dict", [], data=label))
        return self

    # ---- standard gates (names of the reference gate sets) ----
    def _g(name, nq, npar=0):
        def f(self, *args):
            params, qubits = args[:npar], args[npar:]
            if len(qubits) == 1 and not np.isscalar(qubits[0]):
                qubits = tuple(qubits[0])
            return self.append_gate(name, qubits, params)
        f.__name__ = name
        return f

    id = _g("id", 1); x = _g("x", 1); y = _g("y", 1); z = _g("z", 1); h = _g("h", 1)
    s = _g("s", 1); sdg = _g("sdg", 1); t = _g("t", 1); tdg = _g("tdg", 1); sx = _g("sx", 1); sxdg = _g("sxdg", 1)
    rx = _g("rx", 1, 1); ry = _g("ry", 1, 1); rz = _g("rz", 1, 1); p = _g("p", 1, 1); u1 = _g("u1", 1, 1)
    u2 = _g("u2", 1, 2); u3 = _g("u3", 1, 3); u = _g("u", 1, 3); r = _g("r", 1, 2)
    cx = _g("cx", 2); cy = _g("cy", 2); cz = _g("cz", 2); swap = _g("swap", 2); ecr = _g("ecr", 2)
    cp = _g("cp", 2, 1); crx = _g("crx", 2, 1); cry = _g("cry", 2, 1); crz = _g("crz", 2, 1)
    rxx = _g("rxx", 2, 1); ryy = _g("ryy", 2, 1); rzz = _g("rzz", 2, 1); rzx = _g("rzx", 2, 1)
    ccx = _g("ccx", 3); cswap = _g("cswap", 3); ccz = _g("ccz", 3)
    del _g

    def mcx(self, controls, target):
        return self.append_gate("mcx", list(controls) + [target])

    def mcp(self, lam, controls, target):
        return self.append_gate("mcp", list(controls) + [target], [lam])

    # ---- assembly ----
    def split_final(self):
        """Ops before the first measurement / save, the trailing measures, and
        the saves and set instructions in circuit order, each with the
        number of body ops before it (a sampleable circuit: measures only at
        the end, Executor::check_measure_sampling_opt)."""
        body, meas, saves = [], [], []
        for ins in self.data:
            if ins.kind == "measure":
                meas.append(ins)
            elif ins.kind in ("save", "set"):
                if ins.kind == "set" and meas:
                    raise ValueError("only final measurements are supported (no mid-circuit measure)")
                saves.append((len(body), ins))
            else:
                if meas:
                    raise ValueError("only final measurements are supported (no mid-circuit measure)")
                body.append(ins)
        return body, meas, saves


_PAULI_PRODUCT = {("X", "Y"): (1j, "Z"), ("Y", "Z"): (1j, "X"), ("Z", "X"): (1j, "Y"),
                  ("Y", "X"): (-1j, "Z"), ("Z", "Y"): (-1j, "X"), ("X", "Z"): (-1j, "Y")}


def _pauli_of(label: str, qubits) -> dict:
    """{qubit: 'X'|'Y'|'Z'} of a label read right to left onto qubits."""
    out = {}
    for j, q in enumerate(qubits):
        c = label[len(label) - 1 - j].upper()
        if c not in "IXYZ":
            raise ValueError(f"invalid Pauli label {label!r}")
        if c != "I":
            out[int(q)] = c
    return out


def _pauli_product(a: dict, b: dict):
    phase, out = 1 + 0j, dict(a)
    for q, pb in b.items():
        pa = out.get(q)
        if pa is None:
            out[q] = pb
        elif pa == pb:
            del out[q]
        else:
            ph, pc = _PAULI_PRODUCT[(pa, pb)]
            phase *= ph
            out[q] = pc
    return phase, out


def expval_params(terms, variance: bool = False):
    """The reference's expectation-value parameters (_expval_params,
    save_expectation_value.py:139-168): one entry per distinct Pauli, in
    first-seen order, with the sum of the real parts of its coefficients in
    O and, for the variance, in O.O (the Pauli products of every ordered pair
    of terms, phases folded into the coefficients).  Returns
    [((qubits, label), c_O, c_OO)] with label over the sorted qubits."""
    ops = [(complex(c), _pauli_of(lab, q)) for c, lab, q in terms]
    params = {}
    for c, d in ops:
        key = tuple(sorted(d.items()))
        c1, c2 = params.get(key, (0.0, 0.0))
        params[key] = (c1 + c.real, c2)
    if variance:
        for ca, da in ops:
            for cb, db in ops:
                ph, d = _pauli_product(da, db)
                key = tuple(sorted(d.items()))
                c1, c2 = params.get(key, (0.0, 0.0))
                params[key] = (c1, c2 + (ca * cb * ph).real)
    out = []
    for key, (c1, c2) in params.items():
        qubits = [q for q, _ in key]
        out.append(((qubits, "".join(p for _, p in reversed(key))), c1, c2))
    return out


class NativeCircuit:
    """The engine's op list (gbqv_circuit_t) built from instructions."""

    def __init__(self, num_qubits: int, instructions=()):
        self._L = A.lib()
        h = C.c_void_p()
        A.check(self._L.gbqv_circuit_create(int(num_qubits), C.byref(h)))
        self._h = h
        self.num_qubits = num_qubits
        self.param_slots = []  # (op index, parameter position, expression)
        for ins in instructions:
            self.add(ins)

    def bind(self, binds: dict, nbind: int) -> None:
        """Runtime parameter binding (gbqv_circuit_bind_param): every
        parameterised gate parameter gets its value for each of the nbind
        bindings; binds maps each Parameter to nbind values."""
        for op_index, pos, expr in self.param_slots:
            v = np.ascontiguousarray(np.broadcast_to(expr.evaluate(binds), (nbind,)), dtype=np.float64)
            if v.shape != (nbind,):
                raise ValueError("every parameter needs one value per binding")
            A.check(self._L.gbqv_circuit_bind_param(self._h, op_index, pos, nbind, v.ctypes.data_as(A.dp)))

    def close(self):
        if getattr(self, "_h", None):
            self._L.gbqv_circuit_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def add(self, ins: Instruction):
        q, qp, k = A.qubits_arg(ins.qubits)
        L = self._L
        if ins.kind == "gate":
            vals = []
            for pos, p in enumerate(ins.params):
                if isinstance(p, ParameterExpression):
                    # placeholder until bind(): the op's index is the current op count
                    self.param_slots.append((self.num_ops(), pos, p))
                    vals.append(0.0)
                else:
                    vals.append(float(p))
            pa = np.ascontiguousarray(np.asarray(vals, dtype=np.float64))
            A.check(L.gbqv_circuit_gate(self._h, ins.name.encode(), qp, k, pa.ctypes.data_as(A.dp), pa.size))
        elif ins.kind == "unitary":
            m, mp = A.cmat_arg(ins.data)
            A.check(L.gbqv_circuit_unitary(self._h, qp, k, mp))
        elif ins.kind == "diagonal":
            m, mp = A.cmat_arg(np.asarray(ins.data).reshape(-1))
            A.check(L.gbqv_circuit_diagonal(self._h, qp, k, mp))
        elif ins.kind == "superop":
            m, mp = A.cmat_arg(ins.data)
            A.check(L.gbqv_circuit_superop(self._h, qp, k, mp))
        elif ins.kind == "kraus":
            flat = np.concatenate([np.asarray(x, dtype=complex).reshape(-1, order="F") for x in ins.data])
            m, mp = A.cmat_arg(flat)
            A.check(L.gbqv_circuit_kraus(self._h, qp, k, len(ins.data), mp))
        elif ins.kind == "reset":
            A.check(L.gbqv_circuit_reset(self._h, qp, k))
        elif ins.kind == "barrier":
            A.check(L.gbqv_circuit_barrier(self._h, qp, k))
        else:
            raise ValueError(f"cannot assemble {ins.kind}")

    def num_ops(self) -> int:
        n = C.c_int()
        A.check(self._L.gbqv_circuit_num_ops(self._h, C.byref(n)))
        return n.value

    def ops(self):
        """[(type, name, qubits)] of the current op list."""
        out = []
        for i in range(self.num_ops()):
            t, nq = C.c_int(), C.c_int()
            qb = (C.c_uint64 * 64)()
            name = C.create_string_buffer(64)
            A.check(self._L.gbqv_circuit_op_info(self._h, i, C.byref(t), C.byref(nq), qb, 64, name, 64))
            out.append((t.value, name.value.decode(), [int(qb[j]) for j in range(nq.value)]))
        return out

    def op_matrix(self, i: int) -> np.ndarray:
        t, name, q = self.ops()[i]
        k = len(q)
        size = {1: 1 << (2 * k), 2: 1 << k, 3: 1 << (4 * k)}.get(t, 1 << (2 * k))
        out = np.empty(size, dtype=np.complex128)
        A.check(self._L.gbqv_circuit_op_matrix(self._h, i, out.ctypes.data_as(A.vp), size))
        return out

    def fuse(self, config: "A.FusionConfig"):
        applied = C.c_int()
        name = C.create_string_buffer(16)
        A.check(self._L.gbqv_circuit_fuse(self._h, C.byref(config), C.byref(applied), name, 16))
        return bool(applied.value), name.value.decode()
