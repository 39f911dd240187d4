"""The C ABI: libaqua.so exports every symbol include/aqua.h declares, the
ctypes binding declares the same set, and struct sizes match the header's
layout rules. No GPU needed."""
from __future__ import annotations

import ctypes
import os
import re
import subprocess

import pytest

import aqua

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "aqua.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"AQUA_API\s+[\w\s\*]+?\b(aqua_\w+)\s*\(", text)))


def test_header_declares_the_expected_surface():
    names = declared_symbols()
    for n in ("aqua_create", "aqua_destroy", "aqua_last_error", "aqua_load_scene_json",
              "aqua_make_procedural_scene", "aqua_load_integrator_json", "aqua_trace", "aqua_render",
              "aqua_render_batch", "aqua_scene_free"):
        assert n in names


def test_library_exports_every_declared_symbol():
    lib = aqua.load_library()
    for n in declared_symbols():
        assert hasattr(lib, n), n
    out = subprocess.run(["nm", "-D", "--defined-only", aqua.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (aqua_\w+)", out))
    assert set(declared_symbols()) <= exported
    # nothing but the ABI is exported from the library's own code
    assert {s for s in exported if s.startswith("aqua_")} == set(declared_symbols())


def test_binding_declares_every_symbol():
    assert sorted(n for n, _, _ in aqua.SIGNATURES) == declared_symbols()


def test_struct_layouts():
    assert ctypes.sizeof(aqua.Ray) == 32
    assert ctypes.sizeof(aqua.Hit) == 16
    assert ctypes.sizeof(aqua.Material) == 32
    assert ctypes.sizeof(aqua.Light) == 56
    assert ctypes.sizeof(aqua.IntegratorCfg) == 56


def test_status_strings_and_version():
    lib = aqua.load_library()
    assert lib.aqua_version() == 200  # four-wide BVH export layout
    assert lib.aqua_status_string(0) == b"ok"
    assert lib.aqua_status_string(4) == b"missing asset"
    assert lib.aqua_status_string(99) == b"unknown status"


def test_null_arguments_are_rejected():
    lib = aqua.load_library()
    assert lib.aqua_create(None, None) == aqua.ERR_INVALID_ARG
    assert lib.aqua_last_error(None) == b"out is NULL"
    assert lib.aqua_render(None, None, None, None, None, 0, None) == aqua.ERR_INVALID_ARG
    with aqua.Context(device=-2) as c:
        assert lib.aqua_load_scene_json(c.handle, None, 0, None) == aqua.ERR_INVALID_ARG
        assert b"non-NULL" in lib.aqua_last_error(c.handle)
    lib.aqua_destroy(None)  # no-op


def test_defaults_follow_integrator_json():
    c = aqua.IntegratorCfg()
    aqua.load_library().aqua_integrator_defaults(ctypes.byref(c))
    # scenes/integrator.json:3-7
    assert (c.spp, c.batch_size, c.max_depth, c.training_iters) == (4, 512, 5, 2048)
    assert abs(c.learning_rate - 1e-3) < 1e-9
