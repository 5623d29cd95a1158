"""The C++ QubitVector adapter (include/gbqv_qubitvector.hpp) compiles with
-Wall -Wextra -Werror against include/gbqv.h, its three classes instantiate
in full, it links against libgbqv.so, and a failing C-ABI call surfaces as
the reference's exception type (std::runtime_error for a CUDA error, here the
missing GPU) instead of crossing the ABI."""
import pytest

from adapter_build import build_driver, run_driver


def test_adapter_compiles_links_and_translates_errors(tmp_path):
    exe = build_driver(tmp_path)
    rc, out, err = run_driver(exe, "sv c128 4\nnorm\nend\n", timeout=120)
    if rc == 0:  # a GPU is present: the state was created and the norm read
        assert out.startswith("norm 1")
    else:
        assert rc == 3, (rc, out, err)
        assert out.startswith("runtime_error:"), out


def test_adapter_driver_rejects_bad_input(tmp_path):
    exe = build_driver(tmp_path)
    rc, _, _ = run_driver(exe, "", timeout=60)
    assert rc == 2
