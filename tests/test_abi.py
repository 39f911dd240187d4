"""The C ABI: libaqua.so exports every symbol include/aqua.h declares, the
ctypes binding declares the same set, and struct sizes match the header's
layout rules. No GPU needed."""
from __future__ import annotations

import ctypes
import json
import os
import re
import subprocess
import sys

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
    assert ctypes.sizeof(aqua.Material) == 64
    assert ctypes.sizeof(aqua.Light) == 56
    assert ctypes.sizeof(aqua.IntegratorCfg) == 64


def test_status_strings_and_version():
    lib = aqua.load_library()
    assert lib.aqua_version() == 300  # 64-byte aqua_material with the Principled lobes
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


NULL_CHILD = r'''
import sys, json, ctypes as C
sys.path.insert(0, sys.argv[1])
import aqua
lib = aqua.load_library()
ctx = aqua.Context(device=-2)
out = {}
for mode in ("null_ctx", "host_ctx"):
    for name, res, args in aqua.SIGNATURES:
        if name in ("aqua_version", "aqua_render_noalloc_max_pixels", "aqua_status_string", "aqua_last_error"):
            continue
        vals = [0 if a in (C.c_int, C.c_int32, C.c_uint32, C.c_uint64, C.c_size_t) else None for a in args]
        takes_ctx = bool(args) and args[0] is aqua._P and name not in ("aqua_destroy", "aqua_nrc_defaults")
        if mode == "host_ctx" and takes_ctx:
            vals[0] = ctx.handle
        r = getattr(lib, name)(*vals)
        out[mode + ":" + name] = r
print(json.dumps(out))
'''


def test_every_entry_point_survives_null_arguments(built):
    """Each entry point called with NULL pointers and zero sizes, once with a
    NULL context and once with a host-only one: status calls return an error
    (freeing or destroying NULL is a no-op that succeeds), the *_defaults
    and destroy calls return quietly, and nothing crashes (child process)."""
    r = subprocess.run([sys.executable, "-c", NULL_CHILD, os.path.join(ROOT, "aqua-engine_gb300")],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    got = json.loads(r.stdout.strip().splitlines()[-1])
    noops = {"host_ctx:aqua_scene_free", "host_ctx:aqua_nrc_destroy"}
    for key, st in got.items():
        name = key.split(":")[1]
        if name in ("aqua_destroy", "aqua_integrator_defaults", "aqua_tuning_defaults", "aqua_nrc_defaults"):
            assert st is None, key
        elif name == "aqua_workspace_bytes":
            assert st == 0, key
        elif key in noops:
            assert st == aqua.OK, key
        else:
            assert st not in (None, aqua.OK), key
            if key.startswith("null_ctx:"):
                assert st == aqua.ERR_INVALID_ARG, key
