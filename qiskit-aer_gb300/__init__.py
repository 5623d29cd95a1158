"""GB300-native statevector / density-matrix engine with Qiskit Aer's qreg
surface.

Package layout:
  csrc/           CUDA kernels (sm_103a) + C++ host code behind the C ABI
                  declared in include/gbqv.h (built into libgbqv.so)
  _capi.py        ctypes binding of that ABI
  qubitvector.py  QubitVector / DensityMatrix (the reference's qreg surface)
  circuit.py      instruction list -> engine op list
  noise.py        noise channels as superoperators
  simulator.py    AerSimulator-shaped run() with fusion, sampling, saves
  adjoint.py      adjoint-method gradients behind torch.autograd
  autotune.py     schedule autotuner (execution form, batch team split)
"""
from ._capi import GBQVError, lib
from .circuit import NativeCircuit, Parameter, ParameterExpression, QuantumCircuit
from .noise import (NoiseModel, QuantumError, ReadoutError, amplitude_damping_error, coherent_unitary_error,
                    depolarizing_error, kraus_error, mixed_unitary_error, pauli_error, phase_amplitude_damping_error,
                    phase_damping_error, reset_error, thermal_relaxation_error)
from .qubitvector import DensityMatrix, QubitVector, UnitaryMatrix
from .simulator import AerSimulator, Result, uniforms
from . import adjoint, autotune, batched
from .primitives import EstimatorV2, SamplerV2

__all__ = [
    "AerSimulator", "adjoint", "autotune", "batched", "DensityMatrix", "EstimatorV2", "SamplerV2", "GBQVError", "NativeCircuit", "NoiseModel",
    "Parameter", "ParameterExpression", "QuantumCircuit",
    "QuantumError", "QubitVector", "Result", "UnitaryMatrix", "amplitude_damping_error", "depolarizing_error", "lib",
    "phase_amplitude_damping_error", "uniforms", "coherent_unitary_error", "kraus_error", "mixed_unitary_error",
    "pauli_error", "phase_damping_error", "reset_error", "thermal_relaxation_error", "ReadoutError",
]


def build(force: bool = False):
    """Compile libgbqv.so in tree (nvcc, sm_103a)."""
    from . import _build

    return _build.build(force=force)
