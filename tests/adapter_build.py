"""Compiles tests/adapter_driver.cpp (the C++ QubitVector adapter of
include/gbqv_qubitvector.hpp over libgbqv.so) with g++ into a temporary
directory; shared by the CPU and GPU adapter tests."""
import shutil
import subprocess
from pathlib import Path

from _pkg import ROOT, pkg


def cuda_lib_dir() -> Path:
    nvcc = shutil.which("nvcc")
    home = Path(nvcc).resolve().parent.parent if nvcc else Path("/usr/local/cuda")
    return home / "lib64"


def build_driver(tmp: Path) -> Path:
    pkg().build()
    lib = ROOT / "qiskit-aer_gb300"
    out = tmp / "adapter_driver"
    cmd = ["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "adapter_driver.cpp"), "-o", str(out), "-L", str(lib), "-lgbqv",
           f"-Wl,-rpath,{lib}", "-L", str(cuda_lib_dir()), f"-Wl,-rpath,{cuda_lib_dir()}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise AssertionError(f"adapter driver failed to compile:\n{r.stdout}\n{r.stderr}")
    return out


def run_driver(exe: Path, text: str, timeout: float = 300.0):
    r = subprocess.run([str(exe)], input=text, capture_output=True, text=True, timeout=timeout)
    return r.returncode, r.stdout, r.stderr
