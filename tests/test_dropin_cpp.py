"""The drop-in C++ API (include/tbsla/cpp/*.hpp, the C_CPP_* ABI in
include/tbsla/cpp/*.h) and the exports of the C ABI (include/tbsla_gb300.h).

CPU: every function the C headers declare is exported by the library; the
C++ test program compiles and links against the drop-in headers; and, where
TBSLA's sources are present, the reference's own test programs
(src/cpp/tests/*.cpp, the ones its CMakeLists registers as tests) compile and
link unchanged against the drop-in headers and library.
GPU: the C++ test program (tests/cpp/test_dropin.cpp) runs: known answers,
closed-form cdiag products and a_axpx_ for every format, exact cross-format
cqmat products, PageRank / personalized PageRank across formats, binary and
Matrix Market round trips, the C_CPP_* ABI.
"""
from __future__ import annotations

import ctypes
import glob
import os
import re
import shutil
import subprocess

import pytest

from oracle.oracle import reference_sources

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(ROOT, "include")
_REF_SRC = reference_sources()
REFERENCE_TESTS = os.path.join(_REF_SRC, "tests") if _REF_SRC else ""

C_HEADERS = [os.path.join(INCLUDE, "tbsla_gb300.h")] + sorted(glob.glob(os.path.join(INCLUDE, "tbsla", "cpp", "*.h")))


def declared_functions(path: str) -> list[str]:
    """Names of the functions a C header declares (static inline ones aside)."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    text = re.sub(r"//[^\n]*", " ", text)
    names = re.findall(r"^\s*(?!static)[A-Za-z_][\w\s\*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M)
    return sorted({n for n in names if n not in ("if", "return", "sizeof")})


def _compile_cpp(src: str, out: str, lib_dir: str) -> subprocess.CompletedProcess:
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O2", "-Wall", f"-I{INCLUDE}", src, f"-L{lib_dir}",
           "-ltbsla_gb300", f"-Wl,-rpath,{lib_dir}", "-o", out]
    return subprocess.run(cmd, capture_output=True, text=True)


@pytest.mark.parametrize("header", C_HEADERS, ids=os.path.basename)
def test_c_headers_are_exported(capi, header):
    L = capi.lib()
    names = declared_functions(header)
    assert names, header
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, f"{os.path.basename(header)} declares unexported {missing}"


def test_dropin_program_builds(capi, tmp_path):
    lib_dir = os.path.dirname(capi.LIB_PATH)
    r = _compile_cpp(os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp"), str(tmp_path / "t"), lib_dir)
    assert r.returncode == 0, r.stderr


def _registered_reference_tests() -> list[str]:
    cm = os.path.join(REFERENCE_TESTS, "CMakeLists.txt")
    if not os.path.exists(cm):
        return []
    exe = dict(re.findall(r"add_executable\((\w+)\s+(\w+\.cpp)\)", open(cm).read()))
    tested = re.findall(r"add_test\(\w+\s+(\w+)\)", open(cm).read())
    return sorted({exe[t] for t in tested if t in exe})


REFERENCE_APPS = os.path.join(_REF_SRC, "apps") if _REF_SRC else ""


def _reference_apps() -> list[str]:
    if not os.path.isdir(REFERENCE_APPS):
        return []
    return sorted(f for f in os.listdir(REFERENCE_APPS) if f.endswith(".cpp"))


@pytest.mark.skipif(not os.path.isdir(REFERENCE_APPS), reason="TBSLA sources not present")
@pytest.mark.parametrize("src", _reference_apps() or ["none"])
def test_reference_apps_compile_against_dropin(capi, tmp_path, src):
    """The reference's driver programs (src/cpp/apps/*.cpp: tbsla_perf,
    tbsla_page_rank, ...) build unchanged against the drop-in headers
    (InputParser.hpp, split.hpp, cpuset_to_cstr.hpp, tbsla/Configs.h among
    them) and the library."""
    lib_dir = os.path.dirname(capi.LIB_PATH)
    r = _compile_cpp(os.path.join(REFERENCE_APPS, src), str(tmp_path / "t"), lib_dir)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TESTS), reason="TBSLA sources not present")
def test_reference_input_parser_test_passes(capi, tmp_path):
    """The reference's command-line parser test (src/cpp/tests/input_parser.cpp)
    runs against the drop-in's InputParser (no GPU involved) and exits 0."""
    lib_dir = os.path.dirname(capi.LIB_PATH)
    exe = str(tmp_path / "input_parser")
    r = _compile_cpp(os.path.join(REFERENCE_TESTS, "input_parser.cpp"), exe, lib_dir)
    assert r.returncode == 0, r.stderr[-2000:]
    assert subprocess.run([exe], timeout=60).returncode == 0


def test_driver_utilities(capi, tmp_path):
    """split, cpuset_to_cstr and InputParser of the drop-in on known answers
    (the behaviour of src/cpp/utils/split.cpp, cpuset_to_cstr.cpp and
    InputParser.cpp)."""
    lib_dir = os.path.dirname(capi.LIB_PATH)
    exe = str(tmp_path / "utils_check")
    r = _compile_cpp(os.path.join(ROOT, "tests", "cpp", "utils_check.cpp"), exe, lib_dir)
    assert r.returncode == 0, r.stderr[-2000:]
    run = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0, run.stdout + run.stderr


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TESTS), reason="TBSLA sources not present")
@pytest.mark.parametrize("src", _registered_reference_tests() or ["none"])
def test_reference_tests_compile_against_dropin(capi, tmp_path, src):
    lib_dir = os.path.dirname(capi.LIB_PATH)
    r = _compile_cpp(os.path.join(REFERENCE_TESTS, src), str(tmp_path / "t"), lib_dir)
    assert r.returncode == 0, r.stderr[-2000:]


@pytest.mark.gpu
def test_dropin_program_runs_on_gpu(gpu, tmp_path):
    lib_dir = os.path.dirname(gpu.LIB_PATH)
    exe = str(tmp_path / "test_dropin")
    r = _compile_cpp(os.path.join(ROOT, "tests", "cpp", "test_dropin.cpp"), exe, lib_dir)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=600)
    fails = [l for l in run.stdout.splitlines() if l.startswith("FAIL")]
    assert run.returncode == 0 and "OK 0" in run.stdout, "\n".join(fails[:40]) + run.stderr[-2000:]


def test_driver_programs_build(capi):
    """build() compiles the driver programs (tbsla_gb300/apps) next to the
    library; run without their required flags they print the reference
    drivers' usage errors and exit 1 (no GPU needed for that)."""
    from tbsla_gb300 import build
    for name, msg in (("tbsla_perf", "A file format has to be given"),
                      ("tbsla_page_rank", "A matrix file has to be given")):
        exe = build.app_path(name)
        assert os.path.exists(exe), exe
        r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
        assert r.returncode == 1 and msg in r.stderr, (name, r.returncode, r.stderr)
