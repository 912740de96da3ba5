"""Shared test set-up: the `gpu` marker, in-tree builds, fixture loading.

CPU tests (-m "not gpu") exercise the oracle against the reference's golden
data, the host logic of the C library (table parsing, sampling) and its
exported symbols; GPU tests compare the CUDA path with the oracle.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
# the reference tree (only the CPU tests that read it as text use it)
REFERENCE = os.environ.get("DNSMC_REFERENCE", "/root/reference")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def _ensure_built():
    from dnsmc_gb300 import build as pkg_build
    from oracle import build as orc_build
    if not os.path.exists(pkg_build.lib_path()):
        pkg_build.build()
    if not os.path.exists(orc_build.lib_path()):
        orc_build.build(with_ref=False)


_ensure_built()


def golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name)) as d:
        return {k: d[k] for k in d.files}


@pytest.fixture(scope="session")
def particle_tables():
    return golden("particle_tables.npz")


@pytest.fixture(scope="session")
def ck_tables():
    return golden("ck_tables.npz")


@pytest.fixture(scope="session")
def resfortm():
    return golden("resfortm.npz")


def has_gpu() -> bool:
    try:
        import ctypes
        rt = None
        for name in ("libcudart.so", "libcudart.so.13", "libcuda.so.1"):
            try:
                rt = ctypes.CDLL(name)
                break
            except OSError:
                continue
        if rt is None:
            return False
        if hasattr(rt, "cuInit"):
            return rt.cuInit(0) == 0
        n = ctypes.c_int()
        return rt.cudaGetDeviceCount(ctypes.byref(n)) == 0 and n.value > 0
    except Exception:
        return False
