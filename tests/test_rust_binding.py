"""The Rust binding a maintainer of the reference crate would add
(rust/isosurface-gpu-sys, rust/isosurface/src/gpu) cannot be compiled here:
there is no Rust toolchain.  These CPU tests keep it honest against the C
header instead: every function of include/isosurface_gpu.h is declared in
the extern block with the same parameter names, matching types and the same
return type; the #[repr(C)] structures have the header's fields in order;
the status, flag and placer constants have the header's values; and the
program ops the Rust lowering emits are the header's op codes."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "isosurface_gpu.h")
SYS = os.path.join(ROOT, "rust", "isosurface-gpu-sys", "src", "lib.rs")
LOWER = os.path.join(ROOT, "rust", "isosurface", "src", "gpu", "lower.rs")
GPU_MOD = os.path.join(ROOT, "rust", "isosurface", "src", "gpu", "mod.rs")

# C type -> Rust type, as the binding spells them
C2R = {
    "iso_status": "IsoStatus", "int": "c_int", "uint32_t": "u32", "uint64_t": "u64", "int64_t": "i64",
    "size_t": "usize", "float": "f32", "double": "f64", "void": "c_void", "char": "c_char", "uint8_t": "u8",
    "iso_ctx": "IsoCtx", "iso_program": "IsoProgram", "iso_batch": "IsoBatch", "iso_mlp": "IsoMlp",
    "iso_mesh_info": "IsoMeshInfo", "iso_chunk_desc": "IsoChunkDesc", "iso_surrogate_stats": "IsoSurrogateStats",
    "iso_mesh_distance_result": "IsoMeshDistanceResult",
}


def _c_type_to_rust(t):
    """'const iso_program* const*' -> '*const *const IsoProgram' and so on."""
    t = t.replace("struct ", "").strip()
    m = re.match(r"^(const\s+)?(\w+)\s*(.*)$", t)
    const_base, base, stars = m.group(1) is not None, m.group(2), m.group(3).replace(" ", "")
    out = C2R[base]
    levels = stars.split("*")[:-1] if stars else []
    # levels[i] is the qualifier text before the (i+1)-th star ("" or "const")
    for i, qual in enumerate(levels):
        pointee_const = const_base if i == 0 else qual == "const"
        out = ("*const " if pointee_const else "*mut ") + out
    return out


def _header_functions():
    s = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for ret, name, args in re.findall(r"^ISO_API\s+([^;(]+?)\s*\b(iso_\w+)\s*\(([^;]*?)\)\s*;", s,
                                      flags=re.S | re.M):
        params = []
        args = " ".join(args.split())
        if args != "void":
            for p in args.split(","):
                m = re.match(r"^(.*?)(\w+)$", p.strip())
                params.append((m.group(2), _c_type_to_rust(m.group(1))))
        out[name] = (params, _c_type_to_rust(" ".join(ret.split())))
    return out


def _rust_functions():
    s = open(SYS).read()
    block = s[s.index('extern "C" {'):]
    out = {}
    for name, args, ret in re.findall(r"pub fn (iso_\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", block, flags=re.S):
        params = []
        for p in " ".join(args.split()).split(","):
            p = p.strip()
            if p:
                n, t = p.split(":", 1)
                params.append((n.strip(), t.strip()))
        out[name] = (params, ret.strip() if ret else "()")
    return out


def test_every_header_function_is_declared_alike():
    h, r = _header_functions(), _rust_functions()
    assert len(h) > 50
    assert sorted(h) == sorted(r)
    for name, (params, ret) in h.items():
        assert r[name][0] == params, name
        assert r[name][1] == ret, name


def _header_structs():
    s = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for body, name in re.findall(r"typedef struct \w+ \{(.*?)\}\s*(\w+);", s, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            ctype, names = decl.split(" ", 1)
            for n in names.split(","):
                fields.append((n.strip(), C2R[ctype]))
        out[C2R[name]] = fields
    return out


def test_structures_match():
    s = open(SYS).read()
    for name, fields in _header_structs().items():
        m = re.search(r"pub struct %s \{(.*?)\}" % name, s, flags=re.S)
        assert m, name
        got = re.findall(r"pub (\w+): (\w+),", m.group(1))
        assert got == fields, name
        assert "#[repr(C)]" in s[: m.start()].rsplit("}", 1)[-1], name


def test_constants_match():
    h = dict(re.findall(r"#define (ISO_\w+) (\d+)u?\b", open(HEADER).read()))
    r = dict(re.findall(r"pub const (ISO_\w+): \w+ = (\d+);", open(SYS).read()))
    assert len(r) >= 25
    for name, value in r.items():
        assert h[name] == value, name
    for name in h:
        if name.startswith(("ISO_ERR_", "ISO_FLAG_", "ISO_PLACER_", "ISO_STAGE_")) or name == "ISO_OK":
            assert name in r, name


def test_lowering_op_codes_match_the_program_format():
    table = dict((name, int(code, 16)) for code, name in
                 re.findall(r"\*\s+(0x[0-9A-F]{2}) (\w+)", open(HEADER).read()))
    assert table["SPHERE"] == 0x10 and table["CD_END"] == 0x41
    codes = dict((name, int(v, 16)) for name, v in re.findall(r"const OP_(\w+): u32 = (0x[0-9A-F]+);",
                                                               open(LOWER).read()))
    assert codes
    for name, v in codes.items():
        assert table[name] == v, name
    assert "0x314F_5349" in open(LOWER).read()  # "ISO1", the header's magic


@pytest.mark.parametrize("fn", ["marching_cubes", "dual_contouring", "linear_hashed_marching_cubes",
                                "point_cloud", "extended_marching_cubes"])
def test_wrappers_cover_the_reference_extractors(fn):
    src = open(GPU_MOD).read()
    assert re.search(r"pub fn %s<" % fn, src), fn
