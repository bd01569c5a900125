"""Shared fixtures.

Markers: ``gpu`` -- needs a CUDA device (the parity tests proper, run through
the C ABI); everything else runs on a CPU-only host.
"""
from __future__ import annotations

import ctypes
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU; runs the CUDA path through the C ABI")


def gpu_count() -> int:
    for name in ("libcudart.so", "libcudart.so.13", "libcuda.so.1"):
        try:
            L = ctypes.CDLL(name)
        except OSError:
            continue
        n = ctypes.c_int(0)
        if name.startswith("libcuda."):
            if L.cuInit(0) != 0 or L.cuDeviceGetCount(ctypes.byref(n)) != 0:
                return 0
        elif L.cudaGetDeviceCount(ctypes.byref(n)) != 0:
            return 0
        return n.value
    return 0


@pytest.fixture(scope="session")
def capi():
    from tbsla_gb300 import build, capi as c
    build.build()
    c.lib()
    return c


@pytest.fixture(scope="session")
def gpu(capi):
    if gpu_count() == 0:
        pytest.fail("no CUDA device visible: the gpu tests need one")
    return capi


@pytest.fixture(scope="session")
def orc():
    from oracle.oracle import Oracle, build
    build(ref=False)
    return Oracle()


@pytest.fixture(scope="session")
def ref():
    from oracle.oracle import Reference, build, reference_available, reference_sources
    if reference_sources():
        build(ref=True)
    if not reference_available():
        pytest.skip("reference build oracle/_ref not present on this host")
    r = Reference()
    r.set_threads(1)
    return r


@pytest.fixture(scope="session")
def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)


def fnv(a: np.ndarray) -> str:
    from oracle.oracle import Oracle
    return f"{Oracle().fnv1a(np.ascontiguousarray(a)):016x}"


def assert_close(y, yref, scale=None, rtol=1e-12, what=""):
    """|y - yref| <= rtol * scale componentwise, scale defaulting to |yref|
    (use sum_j |a_ij x_j| for sums with cancellation)."""
    y = np.asarray(y, np.float64)
    yref = np.asarray(yref, np.float64)
    assert y.shape == yref.shape, f"{what}: shape {y.shape} vs {yref.shape}"
    s = np.abs(yref) if scale is None else np.asarray(scale)
    bad = np.abs(y - yref) > rtol * s + 1e-300
    if bad.any():
        i = int(np.argmax(bad))
        raise AssertionError(f"{what}: {int(bad.sum())} entries off, first at {i}: {y[i]!r} vs {yref[i]!r} "
                             f"(scale {s[i]!r})")
