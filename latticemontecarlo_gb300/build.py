"""Build recipe of the native library (CUDA kernels for sm_103a + C ABI).

Produces ``latticemontecarlo_gb300/liblmc_gb300.so`` in-tree with nvcc (device
code, ``-gencode arch=compute_103a,code=sm_103a``) and g++ (host code), compiled
in parallel. No CMake, no PyTorch extension machinery: the library exports a
plain C ABI (``include/lmc_gb300.h``).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "liblmc_gb300.so"
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def cuda_home() -> Path:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and (Path(cand) / "bin" / "nvcc").exists():
            return Path(cand)
    nvcc = shutil.which("nvcc")
    if nvcc:
        return Path(nvcc).resolve().parent.parent
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


HOST = PKG / "host"
EXE = PKG / "bin" / "lmc_gb300"


def _has_zlib() -> bool:
    proc = subprocess.run(["g++", "-x", "c++", "-E", "-"], input="#include <zlib.h>\n", capture_output=True, text=True)
    return proc.returncode == 0


def build_host(verbose: bool = False, force: bool = False) -> Path:
    """The C++ host mirror (lmc_host.cpp) and the `lmc_gb300 -p param.txt` executable,
    linked against liblmc_gb300.so (rpath to the package directory)."""
    sources = [HOST / "lmc_host.cpp", HOST / "main.cpp"]
    inputs = sources + [HOST / "lmc_host.hpp", ROOT / "include" / "lmc_gb300.h", LIB]
    if EXE.exists() and not force and EXE.stat().st_mtime >= max(p.stat().st_mtime for p in inputs):
        return EXE
    EXE.parent.mkdir(exist_ok=True)
    libs = ["-lz"] if _has_zlib() else []
    tmp = EXE.with_suffix(".tmp")
    _run(["g++", "-O2", "-std=c++17", "-Wall", "-I", str(HOST), *map(str, sources), "-o", str(tmp), "-L", str(PKG),
          "-llmc_gb300", "-Wl,-rpath,$ORIGIN/..", *libs])
    os.replace(tmp, EXE)
    if verbose:
        print(f"built {EXE}", file=sys.stderr)
    return EXE


def build(verbose: bool = False, force: bool = False) -> Path:
    cuda = cuda_home()
    nvcc = str(cuda / "bin" / "nvcc")
    obj = PKG / "_build"
    obj.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    headers = list(CSRC.glob("*.h*")) + list(CSRC.glob("*.cuh")) + [ROOT / "include" / "lmc_gb300.h"]
    newest_input = max(p.stat().st_mtime for p in sources + headers)
    if LIB.exists() and not force and LIB.stat().st_mtime >= newest_input:
        return LIB
    jobs = []
    objects = []
    for src in sources:
        out = obj / (src.stem + ".o")
        objects.append(str(out))
        if src.suffix == ".cu":
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-v" if verbose else "-O3",
                   "-I", str(CSRC), "-c", str(src), "-o", str(out)]
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", str(cuda / "include"), "-I", str(CSRC),
                   "-c", str(src), "-o", str(out)]
        jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
        list(ex.map(_run, jobs))
    tmp = LIB.with_suffix(".so.tmp")
    _run(["g++", "-shared", "-o", str(tmp), *objects, "-L", str(cuda / "lib64"), "-lcudart",
          f"-Wl,-rpath,{cuda / 'lib64'}"])
    os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    build_host(verbose="-v" in sys.argv, force="-f" in sys.argv)
