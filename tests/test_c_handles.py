"""The C handles (C_CPP_Matrix*_*, C_CPP_Vector_*) against the reference's own,
on the CPU: tests/cpp/c_handles.c is built once against the drop-in headers
and library and once against the reference's C headers and sources
(oracle/_ref/libtbsla_ref_c.so, compiled from them by oracle/Makefile where
they are present); both runs must print the same text (stdout and the
matrices' prints, capacities included) and write the same files.  Products
are left out: the drop-in's run on the GPU."""
import os
import subprocess

import pytest

from oracle.oracle import reference_sources

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_REF_SRC = reference_sources()
REF_C_INCLUDE = os.path.join(_REF_SRC, "interface", "c", "include") if _REF_SRC else ""
REF_LIB_DIR = os.path.join(ROOT, "oracle", "_ref")


def _build(src, include, lib_dir, lib, out):
    cmd = [os.environ.get("CC", "gcc"), "-std=gnu11", "-O1", "-Wall", f"-I{include}", src, f"-L{lib_dir}",
           f"-l{lib}", f"-Wl,-rpath,{lib_dir}", "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def _run(prog, d):
    os.makedirs(d)
    r = subprocess.run([prog, d], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    files = {f: open(os.path.join(d, f), "rb").read() for f in sorted(os.listdir(d))}
    return r.stdout, r.stderr, files


def test_c_handles_behave_as_the_reference(capi, ref, tmp_path):
    if not (os.path.isdir(REF_C_INCLUDE) and os.path.exists(os.path.join(REF_LIB_DIR, "libtbsla_ref_c.so"))):
        pytest.skip("the reference's C handles are not built on this host")
    src = os.path.join(ROOT, "tests", "cpp", "c_handles.c")
    ours, theirs = str(tmp_path / "ours"), str(tmp_path / "ref")
    _build(src, os.path.join(ROOT, "include"), os.path.dirname(capi.LIB_PATH), "tbsla_gb300", ours)
    _build(src, REF_C_INCLUDE, REF_LIB_DIR, "tbsla_ref_c", theirs)
    out_o, err_o, files_o = _run(ours, str(tmp_path / "d_ours"))
    out_r, err_r, files_r = _run(theirs, str(tmp_path / "d_ref"))
    assert out_o == out_r
    assert err_o == err_r
    assert sorted(files_o) == sorted(files_r) and len(files_r) == 11
    for name, data in files_r.items():
        assert files_o[name] == data, name
