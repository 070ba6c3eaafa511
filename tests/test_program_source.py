"""The CUDA C the library compiles per general program (csrc/jit.cu), on
the CPU: iso_program_source needs no device, and NVRTC compiles for sm_103a
without one.  Every general test program's module must compile (the culled
sampler's two kernels, the full field's, and DualContouring's placement
with the program's normals written out unless it holds a central
difference), and the generated evaluators must walk the program's ops as
the interpreter does (one statement per primitive, operator and point map);
sphere sets are not compiled."""
import ctypes

import numpy as np
import pytest

from isosurface_gb300 import scenes
from isosurface_gb300 import source as S
from isosurface_gb300.scenes import SplitMix64

ISO_OK, ISO_ERR_UNSUPPORTED = 0, 9


def _lib():
    from isosurface_gb300._capi import lib
    try:
        return lib()
    except Exception as exc:  # the library is not built here
        pytest.skip("library not loadable: %s" % exc)


def _source(data):
    L = _lib()
    need = ctypes.c_size_t()
    st = L.iso_program_source(data, len(data), None, 0, ctypes.byref(need))
    if st != ISO_OK:
        return st, None
    buf = ctypes.create_string_buffer(need.value)
    assert L.iso_program_source(data, len(data), buf, need.value, ctypes.byref(need)) == ISO_OK
    return ISO_OK, buf.value.decode()


def _nvrtc():
    for name in ("libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                 "/usr/local/cuda/lib64/libnvrtc.so"):
        try:
            return ctypes.CDLL(name)
        except OSError:
            continue
    pytest.skip("no libnvrtc")


def _compile(src):
    n = _nvrtc()
    prog = ctypes.c_void_p()
    assert n.nvrtcCreateProgram(ctypes.byref(prog), src.encode(), b"iso_program.cu", 0, None, None) == 0
    opts = [b"--gpu-architecture=sm_103a", b"--fmad=false", b"--std=c++17", b"-default-device"]
    arr = (ctypes.c_char_p * len(opts))(*opts)
    rc = n.nvrtcCompileProgram(prog, len(opts), arr)
    size = ctypes.c_size_t()
    n.nvrtcGetProgramLogSize(prog, ctypes.byref(size))
    log = ctypes.create_string_buffer(size.value + 1)
    n.nvrtcGetProgramLog(prog, log)
    cubin = ctypes.c_size_t()
    if rc == 0:
        n.nvrtcGetCUBINSize(prog, ctypes.byref(cubin))
    n.nvrtcDestroyProgram(ctypes.byref(prog))
    return rc, cubin.value, log.value.decode(errors="replace")


def _general():
    rng = SplitMix64(5)

    def rigid(src):
        from isosurface_gb300.scenes import random_rotation
        return S.Rigid(src, rng.uniforms(3, -0.1, 0.1), random_rotation(rng))

    return {
        "csg": scenes.csg(),
        "csg7": scenes.csg(seed=7),
        "box": S.unit_to_cube(S.RectangularPrism((0.5, 0.3, 0.7))),
        "cylinder": S.unit_to_cube(S.Cylinder(0.4, 0.6)),
        "intersection": S.unit_to_cube(S.Intersection(S.Sphere(0.8), S.RectangularPrism((0.6, 0.6, 0.6)))),
        "smooth": S.unit_to_cube(S.SmoothUnion(S.Translate(S.Sphere(0.3), (0.2, 0, 0)),
                                               S.Translate(S.Sphere(0.3), (-0.2, 0, 0)), 0.1)),
        "central_difference": S.unit_to_cube(S.CentralDifference(
            S.Union(S.Difference(S.Sphere(0.25), S.RectangularPrism((0.2, 0.2, 0.2))), S.Cylinder(0.02, 0.25)))),
        "nested": S.unit_to_cube(S.Difference(S.Union(rigid(S.Torus(0.5, 0.1)), rigid(S.Sphere(0.4))),
                                              S.Intersection(rigid(S.RectangularPrism((0.3, 0.2, 0.6))),
                                                             S.Cylinder(0.2, 0.9)))),
        # a flat union of translated primitives (compiled for the full field)
        "flat": S.unit_to_cube(S.Union(S.Translate(S.Sphere(0.3), (0.1, 0, 0)),
                                       S.Translate(S.RectangularPrism((0.2, 0.2, 0.2)), (-0.3, 0, 0)))),
    }


@pytest.mark.parametrize("name", sorted(_general()))
def test_generated_module_compiles(name):
    src = _general()[name]
    data = bytes(S.lower(src))
    st, text = _source(data)
    assert st == ISO_OK, st
    at = text.index("struct JitEval")
    body = text[at:text.index("prunable", at)]
    ops = np.frombuffer(data[16:16 + 4 * int(np.frombuffer(data[4:8], np.uint32)[0])], np.uint32) & 0xFF
    prims = int(np.isin(ops, [0x10, 0x11, 0x12, 0x13]).sum())
    binary = int(np.isin(ops, [0x20, 0x21, 0x22, 0x23]).sum())
    maps = int(np.isin(ops, [0x01, 0x02, 0x03]).sum())
    assert body.count("const float val") == prims + binary
    assert body.count("const V3 pt") == maps
    for kernel in ("iso_jit_classify", "iso_jit_rows", "iso_jit_field"):
        assert 'extern "C" __global__ void __launch_bounds__(256) %s(' % kernel in text
    # the normals are written out too (DualContouring's placement kernel),
    # except through a central difference, which the interpreter keeps
    has_cd = bool(np.isin(ops, [0x40]).any())
    assert ("struct JitHermite" in text) == (not has_cd)
    assert ("iso_jit_dc_place" in text) == (not has_cd)
    if not has_cd:
        h = text[text.index("struct JitHermite"):]
        h = h[:h.index("iso_jit_dc_place")]
        assert h.count("const float hval") == prims + binary
        assert h.count("const V3 hnrm") == prims + binary
    rc, cubin, log = _compile(text)
    assert rc == 0 and cubin > 0, log


def test_uncompiled_forms_are_reported():
    rng = np.random.default_rng(1)
    sph = rng.uniform(-0.8, 0.8, size=(12, 4)).astype(np.float32)
    sph[:, 3] = np.abs(sph[:, 3]) * 0.3 + 0.05
    for src in (S.unit_to_cube(S.SphereSet(sph)), S.unit_to_cube(S.SphereSet(sph, smooth_k=0.05))):
        assert _source(bytes(S.lower(src)))[0] == ISO_ERR_UNSUPPORTED
    assert _source(b"\x00" * 8)[0] == 5  # ISO_ERR_BAD_PROGRAM
