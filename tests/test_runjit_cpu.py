"""The specialised register-tile runs (gbqv_set_run_jit): the source
generator's kernel for a synthetic run that uses every op kind compiles with
NVRTC for sm_103a, in complex64 and complex128 (host only, no GPU); the
option reaches the simulator and rejects bad values."""
import ctypes as C

import pytest

from _pkg import pkg


@pytest.mark.parametrize("dbl", [0, 1])
def test_specialised_run_source_compiles(dbl):
    L = pkg().lib()
    buf = C.create_string_buffer(1 << 16)
    rc = L.gbqv_run_jit_compile_check(dbl, buf, len(buf))
    if rc != 0 and b"not available" in buf.value:  # pragma: no cover - NVRTC missing
        pytest.skip("NVRTC is not available")
    assert rc == 0, buf.value.decode()


def test_runtime_compile_option():
    P = pkg()
    sim = P.AerSimulator(runtime_compile=2)
    assert sim.options["runtime_compile"] == 2
    sim.set_options(runtime_compile=0)
    assert sim.options["runtime_compile"] == 0
    with pytest.raises(ValueError, match="runtime_compile"):
        sim.set_options(runtime_compile=3)
