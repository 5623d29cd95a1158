"""C-ABI checks that need no GPU: the library builds, loads and exports every
function include/gbqv.h declares; host-only entry points behave."""
import re
from pathlib import Path

import numpy as np
import pytest

from _pkg import ROOT, pkg

HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b((?:gbqv|aer)_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = pkg().lib()
    missing = [f for f in declared_functions() if not hasattr(L, f)]
    assert not missing, f"missing exports: {missing}"
    assert len(declared_functions()) >= 60


def test_version_and_device_count():
    L = pkg().lib()
    assert L.gbqv_version() == 10000
    assert L.gbqv_device_count() >= 0


def test_uniform_stream_matches_reference_rng():
    a = np.load(ROOT / "tests" / "golden" / "rng_cases.npz")
    for key in a.files:
        seed = int(key.split("_", 1)[1])
        np.testing.assert_array_equal(pkg().uniforms(seed, 1000), a[key])


def test_create_without_gpu_fails_cleanly():
    P = pkg()
    if P.lib().gbqv_device_count() > 0:
        pytest.skip("a GPU is visible")
    with pytest.raises(P.GBQVError) as e:
        P.QubitVector(4)
    assert e.value.code in (3, 4)


def test_bad_arguments_are_errors_not_crashes():
    import ctypes as C
    P = pkg()
    L = P.lib()
    h = C.c_void_p()
    assert L.gbqv_create(4, 7, 0, C.byref(h)) == 1          # bad precision
    assert b"precision" in L.gbqv_last_error(None)
    assert L.gbqv_create(0, 1, 0, C.byref(h)) == 1          # bad size
    assert L.gbqv_norm(None, None) == 1                       # null handle
    c = P.NativeCircuit(3)
    with pytest.raises(P.GBQVError):
        c.add(P.circuit.Instruction("gate", "cx", [0, 3]))    # qubit out of range
    with pytest.raises(P.GBQVError):
        c.add(P.circuit.Instruction("gate", "cx", [1, 1]))    # repeated qubit
    with pytest.raises(P.GBQVError):
        c.add(P.circuit.Instruction("gate", "nosuchgate", [0]))
