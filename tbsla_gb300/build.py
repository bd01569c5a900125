"""Builds libtbsla_gb300.so in-tree for sm_103a, and the driver programs
(tbsla_gb300/apps) into tbsla_gb300/bin.

``python -m tbsla_gb300.build`` or ``tbsla_gb300.build.build()``.  CUDA
sources go through nvcc with ``-gencode arch=compute_103a,code=sm_103a``, C++
sources through g++; translation units compile in parallel and only when a
source or header is newer than the library.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtbsla_gb300.so")
INCLUDE = os.path.join(ROOT, "include")
APPS = os.path.join(HERE, "apps")
BIN = os.path.join(HERE, "bin")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-fopenmp", f"-I{INCLUDE}"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-Wall", f"-I{INCLUDE}"]


def _nvcc() -> str:
    for c in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build tbsla_gb300")


def sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")) +
                  glob.glob(os.path.join(CSRC, "dropin", "*.cpp")))


def _deps() -> list[str]:
    return (sources() + glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(CSRC, "dropin", "*.h")) + glob.glob(os.path.join(INCLUDE, "**", "*.h*"),
                                                                       recursive=True) + [__file__])


def apps() -> list[str]:
    """The driver programs (tbsla_gb300/apps/*.cpp), built into tbsla_gb300/bin."""
    return sorted(glob.glob(os.path.join(APPS, "*.cpp")))


def app_path(name: str) -> str:
    return os.path.join(BIN, name)


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    if not all(os.path.getmtime(d) <= t for d in _deps()):
        return False
    for src in apps():
        exe = app_path(os.path.splitext(os.path.basename(src))[0])
        if not os.path.exists(exe) or os.path.getmtime(exe) < max(t, os.path.getmtime(src)):
            return False
    return True


def _build_app(src: str) -> str:
    exe = app_path(os.path.splitext(os.path.basename(src))[0])
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-Wall", f"-I{INCLUDE}", f"-I{APPS}", src,
           f"-L{HERE}", "-ltbsla_gb300", "-Wl,-rpath,$ORIGIN/..", "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return exe


def _obj(src: str) -> str:
    rel = os.path.relpath(src, CSRC).replace(os.sep, "__")
    return os.path.join(BUILD, rel + ".o")


def _compile(src: str) -> str:
    obj = _obj(src)
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj]
    else:
        cmd = [os.environ.get("CXX", "g++")] + CXX_FLAGS + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    """Compiles the library if needed and returns its path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=max(2, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB + ".tmp"
    cuda_lib = os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "lib64")
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp", f"-L{cuda_lib}",
                                                              "-lcublas", f"-Xlinker=-rpath={cuda_lib}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    os.makedirs(BIN, exist_ok=True)
    with ThreadPoolExecutor(max_workers=max(2, len(apps()))) as ex:
        list(ex.map(_build_app, apps()))
    if verbose:
        print(f"built {LIB} and {len(apps())} driver programs in {BIN}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
