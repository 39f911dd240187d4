"""The Rust binding rust/src/ffi.rs (the `src/ffi.rs` a maintainer of the
reference crate adds) against include/aqua.h, and the ctypes binding's struct
layouts against the header. No Rust compiler exists here, so the check is
textual: every entry point with the same parameter and return types (pointer
constness included), every struct field for field, every constant with the
same value. No GPU needed."""
from __future__ import annotations

import ctypes
import os
import re

import pytest

import aqua

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "aqua.h")
FFI = os.path.join(ROOT, "rust", "src", "ffi.rs")

# scalar spellings -> one canonical name per ABI type
C_BASE = {"int32_t": "i32", "int": "i32", "aqua_status": "i32", "uint32_t": "u32", "uint64_t": "u64",
          "size_t": "usize", "float": "f32", "double": "f64", "uint8_t": "u8", "uint16_t": "u16",
          "char": "c_char", "void": "void"}
RUST_BASE = {"c_int": "i32", "aqua_status": "i32", "c_void": "void"}
SIZE = {"i32": 4, "u32": 4, "f32": 4, "u64": 8, "usize": 8, "f64": 8, "u8": 1, "u16": 2}


# ---------------------------------------------------------------- C side
def c_text() -> str:
    t = open(HEADER).read()
    t = re.sub(r"/\*.*?\*/", " ", t, flags=re.S)
    return re.sub(r"//[^\n]*", " ", t)


def c_type(s: str):
    s = " ".join(s.replace("*", " * ").split())
    if s.endswith("*"):
        inner = s[:-1].strip()
        if "*" not in inner and inner.startswith("const "):
            return ("*const", c_type(inner[len("const "):]))
        return ("*mut", c_type(inner))
    s = s.replace("const ", "").strip()
    return C_BASE.get(s, s)


def c_functions() -> dict:
    out = {}
    for ret, name, params in re.findall(r"AQUA_API\s+([^;{}]*?)\b(aqua_\w+)\s*\(([^)]*)\)\s*;", c_text()):
        ps = [p.strip() for p in params.split(",") if p.strip() and p.strip() != "void"]
        types = []
        for p in ps:
            m = re.match(r"^(.*?[\s\*])(\w+)$", p)
            assert m, (name, p)
            types.append(c_type(m.group(1)))
        out[name] = (c_type(ret), types)
    return out


def c_structs() -> dict:
    out = {}
    for name, body, alias in re.findall(r"typedef\s+struct\s+(\w+)\s*\{(.*?)\}\s*(\w+)\s*;", c_text(), flags=re.S):
        assert name == alias
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"^(\w+)\s*(\**)\s*(.*)$", decl)
            base, stars, rest = m.group(1), m.group(2), m.group(3)
            for d in rest.split(","):
                d = d.strip()
                dm = re.match(r"^(\**)\s*(\w+)\s*(?:\[(\d+)\])?$", d)
                assert dm, (name, d)
                t = c_type(base + "*" * (len(stars) + len(dm.group(1))))
                if dm.group(3):
                    t = ("arr", t, int(dm.group(3)))
                fields.append((dm.group(2), t))
        out[name] = fields
    return out


def c_constants() -> dict:
    t = c_text()
    out = {}
    for body in re.findall(r"enum\s*\w*\s*\{(.*?)\}", t, flags=re.S):
        for item in body.split(","):
            m = re.match(r"^\s*(AQUA_\w+)\s*=\s*(.+?)\s*$", item, flags=re.S)
            if m:
                out[m.group(1)] = eval(re.sub(r"(\d+)u\b", r"\1", m.group(2)))
    for name, val in re.findall(r"#define\s+(AQUA_\w+)\s+(\(?-?\d+\)?)\s*$", t, flags=re.M):
        out[name] = eval(val)
    return out


# ---------------------------------------------------------------- Rust side
def rust_text() -> str:
    blocks = [open(FFI).read()]
    ffi = [b for b in blocks if 'extern "C"' in b and "pub struct aqua_stats" in b]
    assert len(ffi) == 1, "rust/src/ffi.rs is the complete binding"
    return re.sub(r"//[^\n]*", " ", ffi[0])


def rust_type(s: str):
    s = " ".join(s.split())
    if s.startswith("*const "):
        return ("*const", rust_type(s[len("*const "):]))
    if s.startswith("*mut "):
        return ("*mut", rust_type(s[len("*mut "):]))
    m = re.match(r"^\[(\w+);\s*(\d+)\]$", s)
    if m:
        return ("arr", rust_type(m.group(1)), int(m.group(2)))
    return RUST_BASE.get(s, s)


def rust_functions() -> dict:
    out = {}
    block = re.search(r'extern "C"\s*\{(.*)\}', rust_text(), flags=re.S).group(1)
    for name, params, ret in re.findall(r"pub fn (aqua_\w+)\s*\((.*?)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        types = []
        for p in [p for p in params.split(",") if p.strip()]:
            pname, ptype = p.split(":", 1)
            types.append(rust_type(ptype))
        out[name] = (rust_type(ret) if ret.strip() else "void", types)
    return out


def rust_structs() -> dict:
    text = rust_text()
    out = {}
    for attrs, name, body in re.findall(r"((?:#\[[^\]]*\]\s*)*)pub struct (\w+)\s*\{(.*?)\}", text, flags=re.S):
        assert "#[repr(C)]" in attrs, f"{name} must be #[repr(C)]"
        fields = []
        for f in [f.strip() for f in re.split(r",(?![^\[]*\])", body) if f.strip()]:
            m = re.match(r"^(pub\s+)?(?:r#)?(\w+)\s*:\s*(.+)$", f, flags=re.S)
            assert m, (name, f)
            fields.append((m.group(2), rust_type(m.group(3)), bool(m.group(1))))
        out[name] = fields
    return out


def rust_constants() -> dict:
    out = {}
    for name, val in re.findall(r"pub const (AQUA_\w+)\s*:\s*\w+\s*=\s*([^;]+);", rust_text()):
        out[name] = eval(val)
    return out


# ---------------------------------------------------------------- tests
def test_rust_binding_declares_every_entry_point_with_header_types():
    c, r = c_functions(), rust_functions()
    assert sorted(r) == sorted(c), (set(c) ^ set(r))
    for name, (ret, params) in c.items():
        assert r[name][0] == ret, (name, "return", r[name][0], ret)
        assert len(r[name][1]) == len(params), (name, "arity")
        for i, (rt, ct) in enumerate(zip(r[name][1], params)):
            assert rt == ct, (name, i, rt, ct)


def test_rust_binding_structs_match_header_field_for_field():
    c, r = c_structs(), rust_structs()
    opaque = {n for n, f in r.items() if f and all(not pub for _, _, pub in f)}
    assert opaque == {"aqua_ctx", "aqua_scene", "aqua_nrc"}
    assert sorted(set(r) - opaque) == sorted(c)
    for name, fields in c.items():
        assert [(n, t) for n, t, _ in r[name]] == fields, name


def test_rust_binding_constants_match_header_values():
    c, r = c_constants(), rust_constants()
    assert sorted(r) == sorted(c), (set(c) ^ set(r))
    for k, v in c.items():
        assert r[k] == v, k


def c_layout(fields):
    """Offsets and size of a C struct under the x86-64 / AArch64 LP64 rules."""
    def size_align(t):
        if isinstance(t, tuple) and t[0] == "arr":
            s, a = size_align(t[1])
            return s * t[2], a
        if isinstance(t, tuple):
            return 8, 8
        return SIZE[t], SIZE[t]

    off, align, offsets = 0, 1, {}
    for n, t in fields:
        s, a = size_align(t)
        off = (off + a - 1) // a * a
        offsets[n] = off
        off += s
        align = max(align, a)
    return offsets, (off + align - 1) // align * align


CTYPES = {"aqua_options": aqua.Options, "aqua_ray": aqua.Ray, "aqua_hit": aqua.Hit,
          "aqua_trace_counts": aqua.TraceCounts, "aqua_integrator_cfg": aqua.IntegratorCfg,
          "aqua_tuning": aqua.Tuning, "aqua_stats": aqua.Stats, "aqua_scene_info": aqua.SceneInfo,
          "aqua_camera": aqua.Camera, "aqua_material": aqua.Material, "aqua_light": aqua.Light,
          "aqua_job": aqua.Job, "aqua_batch_stats": aqua.BatchStats, "aqua_nrc_cfg": aqua.NrcCfg}


@pytest.mark.parametrize("name", sorted(CTYPES))
def test_ctypes_structs_match_header_layout(name):
    fields = c_structs()[name]
    cls = CTYPES[name]
    assert [f[0] for f in cls._fields_] == [n for n, _ in fields]
    offsets, size = c_layout(fields)
    assert ctypes.sizeof(cls) == size
    for n, off in offsets.items():
        assert getattr(cls, n).offset == off, (name, n)


def test_every_header_struct_has_a_ctypes_mirror():
    assert sorted(CTYPES) == sorted(c_structs())
