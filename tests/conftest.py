"""Shared fixtures. GPU tests are marked `gpu`; everything else runs on CPU
through a host-only context (AQUA_DEVICE_HOST_ONLY) and the CPU oracle."""
from __future__ import annotations

import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "aqua-engine_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session", autouse=True)
def built():
    sys.path.insert(0, ROOT)
    import __graft_entry__

    __graft_entry__.build()
    yield


@pytest.fixture(scope="session")
def host_ctx(built):
    import aqua

    ctx = aqua.Context(device=aqua_host_only())
    yield ctx
    ctx.close()


@pytest.fixture(scope="session")
def gpu_ctx(built):
    import aqua

    ctx = aqua.Context(device=0)
    yield ctx
    ctx.close()


def aqua_host_only() -> int:
    return -2  # AQUA_DEVICE_HOST_ONLY


def random_rays(n: int, lo: float, hi: float, seed: int, tmin: float = 0.0):
    import numpy as np

    rng = np.random.default_rng(seed)
    rays = np.zeros((n, 8), np.float32)
    rays[:, 0:3] = rng.uniform(lo, hi, (n, 3))
    rays[:, 3] = tmin
    rays[:, 4:7] = rng.normal(size=(n, 3))
    rays[:, 7] = np.inf
    return rays
