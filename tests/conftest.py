"""Shared fixtures for the mwblas test suite.

Markers: `gpu` marks tests that need a CUDA device (run with -m gpu).
The CPU oracle (oracle/) is the checker; the library under test is
epblas-parallel_gb300/libmwblas_gb300.so, always called through its C ABI.
"""
from __future__ import annotations

import importlib.util
import json
import os
import zlib
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "epblas-parallel_gb300")
GOLDEN = os.path.join(ROOT, "tests", "golden", "ref_vectors.npz")


def load_module(name, path):
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


mwb = load_module("mwblas", os.path.join(PKG, "mwblas.py"))
orc = load_module("oracle", os.path.join(ROOT, "oracle", "oracle.py"))
build_mod = load_module("mwblas_build", os.path.join(PKG, "build.py"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


def _gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def oracle():
    orc.build()
    return orc.Oracle()


@pytest.fixture(scope="session")
def golden():
    z = np.load(GOLDEN)
    meta = json.loads(bytes(z["meta_json"]).decode())
    return z, meta


@pytest.fixture(scope="session")
def libpath():
    return build_mod.build()


@pytest.fixture(scope="session")
def lib(libpath):
    """The GPU library. GPU tests fail loudly if it cannot run on a device."""
    return mwb.MWBlas(libpath)


@pytest.fixture(scope="session")
def gpu(lib):
    if not _gpu_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    import torch
    torch.cuda.init()
    return lib


@pytest.fixture
def rng(request):
    seed = zlib.crc32(request.node.name.encode())   # stable across processes
    return np.random.default_rng(seed)


def ref_library():
    """The reference built from its own sources (only where they exist)."""
    p = os.path.join(ROOT, "oracle", "_ref", "libmwblas_ref.so")
    return mwb.MWBlas(p, extensions=False) if os.path.exists(p) else None
