"""Adjoint-method gradients of Pauli-Hamiltonian expectation values.

``ExpvalGrad`` runs the engine's ``gbqv_adjoint_expval_grad`` (forward pass,
lam = H psi in one multi-term Pauli pass, then a reverse sweep that
uncomputes psi and lam gate by gate; two state buffers, no stored
intermediate states).  ``expval`` is its ``torch.autograd.Function`` face:
``loss = expval(theta, ansatz, hamiltonian)`` and ``loss.backward()`` fills
``theta.grad``.  Parameter shift and central finite differences, the
references the gradient is checked against, run on the same engine.

The reference has no gradient code; the expectation value it is checked
against is Aer's ``save_expval`` (src/simulators/state.hpp:416-447).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _capi as A
from .circuit import Instruction, NativeCircuit
from .qubitvector import QubitVector

GENERATOR_GATES = ("rx", "ry", "rz", "rxx", "ryy", "rzz", "rzx")


@dataclass
class Hamiltonian:
    """sum_t coeffs[t] * P_t; term t = (qubits, label) with label[k-1-i] on qubits[i]."""
    terms: list
    coeffs: np.ndarray

    def arrays(self):
        qs, offs, labels = [], [0], []
        for q, lab in self.terms:
            qs.extend(int(x) for x in q)
            offs.append(len(qs))
            labels.append(lab.encode())
        qa = np.ascontiguousarray(np.asarray(qs, dtype=np.uint64))
        oa = (C.c_int * len(offs))(*offs)
        la = (C.c_char_p * len(labels))(*labels)
        ca = np.ascontiguousarray(np.asarray(self.coeffs, dtype=np.float64))
        return qa, oa, la, ca


class Ansatz:
    """A gate list whose rotation gates may read a parameter.

    ``gates``: list of (name, qubits, param_index or None, fixed_params)."""

    def __init__(self, num_qubits: int, gates):
        self.num_qubits = num_qubits
        self.gates = list(gates)
        self.num_params = 1 + max((g[2] for g in self.gates if g[2] is not None), default=-1)
        self._native = NativeCircuit(num_qubits)
        for name, q, pi, fixed in self.gates:
            params = list(fixed) if fixed else ([0.0] if pi is not None else [])
            self._native.add(Instruction("gate", name, list(q), params))
        self._param_of_op = (C.c_int * len(self.gates))(*[(-1 if g[2] is None else g[2]) for g in self.gates])

    def instructions(self, theta):
        out = []
        for name, q, pi, fixed in self.gates:
            params = [float(theta[pi])] if pi is not None else list(fixed or [])
            out.append(Instruction("gate", name, list(q), params))
        return out


def hardware_efficient_ansatz(num_qubits: int, layers: int):
    """layers x (RY(theta) and RZ(theta) on every qubit, then a linear CX ladder)."""
    gates, p = [], 0
    for _ in range(layers):
        for q in range(num_qubits):
            gates.append(("ry", [q], p, None))
            p += 1
        for q in range(num_qubits):
            gates.append(("rz", [q], p, None))
            p += 1
        for q in range(num_qubits - 1):
            gates.append(("cx", [q, q + 1], None, None))
    return Ansatz(num_qubits, gates)


def random_hamiltonian(num_qubits: int, nterms: int, rng, min_weight=1, max_weight=4):
    terms = []
    for _ in range(nterms):
        w = int(rng.integers(min_weight, max_weight + 1))
        q = sorted(int(x) for x in rng.choice(num_qubits, size=w, replace=False))
        terms.append((q, "".join(rng.choice(list("XYZ"), size=w))))
    return Hamiltonian(terms, rng.normal(size=nterms))


class Engine:
    """A statevector handle reused across evaluations (one HBM allocation)."""

    def __init__(self, num_qubits: int, precision: str = "double"):
        self.qv = QubitVector(num_qubits, precision)

    def close(self):
        self.qv.close()

    def energy_and_grad(self, ansatz: Ansatz, theta, ham: Hamiltonian):
        theta = np.ascontiguousarray(np.asarray(theta, dtype=np.float64))
        qa, oa, la, ca = ham.arrays()
        e = C.c_double()
        g = np.zeros(ansatz.num_params, dtype=np.float64)
        L = self.qv._L
        A.check(L.gbqv_adjoint_expval_grad(self.qv.handle, ansatz._native.handle, ansatz._param_of_op,
                                           theta.ctypes.data_as(A.dp), theta.size, len(ham.terms),
                                           qa.ctypes.data_as(A.u64p), oa, la, ca.ctypes.data_as(A.dp), C.byref(e),
                                           g.ctypes.data_as(A.dp)), self.qv.handle)
        return e.value, g

    def energy(self, ansatz: Ansatz, theta, ham: Hamiltonian) -> float:
        """E(theta) by one forward pass: Aer's Fusion pass (statevector
        defaults) and the cache-blocked runs, as the adjoint's forward pass."""
        nc = NativeCircuit(ansatz.num_qubits, ansatz.instructions(theta))
        L = self.qv._L
        cfg = A.FusionConfig()
        A.check(L.gbqv_fusion_default_config(0, C.byref(cfg)))
        nc.fuse(cfg)
        self.qv.initialize()
        A.check(L.gbqv_set_blocking(self.qv.handle, 1), self.qv.handle)
        A.check(L.gbqv_execute(self.qv.handle, nc.handle), self.qv.handle)
        _, total = self.qv.expval_pauli_many(ham.terms, ham.coeffs)
        return total

    def param_shift_grad(self, ansatz: Ansatz, theta, ham: Hamiltonian, indices=None):
        """(E(theta + pi/2 e_i) - E(theta - pi/2 e_i)) / 2 per parameter i."""
        theta = np.asarray(theta, dtype=np.float64)
        idx = range(ansatz.num_params) if indices is None else indices
        out = {}
        for i in idx:
            tp, tm = theta.copy(), theta.copy()
            tp[i] += np.pi / 2
            tm[i] -= np.pi / 2
            out[i] = 0.5 * (self.energy(ansatz, tp, ham) - self.energy(ansatz, tm, ham))
        return out

    def finite_diff_grad(self, ansatz: Ansatz, theta, ham: Hamiltonian, indices, h=1e-5):
        theta = np.asarray(theta, dtype=np.float64)
        out = {}
        for i in indices:
            tp, tm = theta.copy(), theta.copy()
            tp[i] += h
            tm[i] -= h
            out[i] = (self.energy(ansatz, tp, ham) - self.energy(ansatz, tm, ham)) / (2 * h)
        return out


def _torch_function():
    import torch

    class ExpvalGrad(torch.autograd.Function):
        """loss = <psi(theta)|H|psi(theta)>; the adjoint gradient is computed in
        the same engine call and returned by backward()."""

        @staticmethod
        def forward(ctx, theta, engine, ansatz, ham):
            e, g = engine.energy_and_grad(ansatz, theta.detach().cpu().numpy(), ham)
            ctx.save_for_backward(torch.as_tensor(g, dtype=theta.dtype, device=theta.device))
            return theta.new_tensor(e)

        @staticmethod
        def backward(ctx, grad_out):
            (g,) = ctx.saved_tensors
            return grad_out * g, None, None, None

    return ExpvalGrad


_EXPVAL = None


def expval(theta, engine: Engine, ansatz: Ansatz, ham: Hamiltonian):
    """torch.autograd entry point: differentiable <H> of the ansatz at theta."""
    global _EXPVAL
    if _EXPVAL is None:
        _EXPVAL = _torch_function()
    return _EXPVAL.apply(theta, engine, ansatz, ham)
