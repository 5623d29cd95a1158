"""Build recipe of libgbqv.so (the engine) — nvcc for sm_103a only, in tree.

Each translation unit under csrc/ compiles in parallel to an object in
_build/, then one link makes ``libgbqv.so`` next to this file.  Rebuilds
only when a source or header is newer than the library.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libgbqv.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
GEN = BUILD / "gen"
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", str(INCLUDE), "-I", str(CSRC), "-I", str(GEN)]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-I", str(INCLUDE), "-I", str(CSRC)]


def _cuda_home() -> Path:
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    return Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))


def _sources():
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def _compile(src: Path) -> Path:
    obj = BUILD / (src.name + ".o")
    cuda = _cuda_home()
    if src.suffix == ".cu":
        cmd = [str(cuda / "bin" / "nvcc"), *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *CXX_FLAGS, "-I", str(cuda / "include"), "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def _generate() -> None:
    """gbqv_runreg_dev_src.inc: the texts of csrc/gbqv_fpair.cuh and
    csrc/gbqv_runreg_dev.cuh as C++ strings, which the specialised
    register-tile runs hand to NVRTC."""
    GEN.mkdir(parents=True, exist_ok=True)
    out = "// generated from csrc/gbqv_fpair.cuh and csrc/gbqv_runreg_dev.cuh by _build.py\n"
    for name, var in (("gbqv_fpair.cuh", "kFpairSrc"), ("gbqv_runreg_dev.cuh", "kRunRegDevSrc")):
        text = (CSRC / name).read_text()
        assert ")GBQVDEV\"" not in text
        out += "static const char " + var + "[] = R\"GBQVDEV(" + text + ")GBQVDEV\";\n"
    (GEN / "gbqv_runreg_dev_src.inc").write_text(out)


def build(force: bool = False, verbose: bool = False) -> Path:
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    _generate()
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    cuda = _cuda_home()
    cmd = [str(cuda / "bin" / "nvcc"), *ARCH, "-shared", "-o", str(LIB) + ".tmp", *map(str, objs),
           "-lcudart", "-ldl", "-L", str(cuda / "lib64")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(str(LIB) + ".tmp", LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
