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


def reference_scene(name: str):
    """Path of one of the reference project's scene files, or None.

    Looked up in $AQUA_REFERENCE_DIR/scenes (a checkout of the reference),
    then in tests/golden/reference_scenes (the staged living-room copy, see
    tests/golden/stage_reference_scenes.py), then in tests/golden/cbox (the
    committed Cornell scene)."""
    dirs = []
    env = os.environ.get("AQUA_REFERENCE_DIR")
    if env:
        dirs.append(os.path.join(env, "scenes"))
    dirs += [os.path.join(GOLDEN, "reference_scenes"), os.path.join(GOLDEN, "cbox")]
    for d in dirs:
        p = os.path.join(d, name)
        if os.path.exists(p):
            return p
    return None


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
