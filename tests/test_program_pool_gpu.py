"""Programs uploaded and destroyed around every extraction, as a binding's
extract() does: a context keeps the device blocks of destroyed programs and
hands them to the next uploads, and an extraction recorded as a CUDA graph
replays for a program uploaded again with the same contents into the same
block.  Checked here: alternating programs through the reused blocks give
each program's own mesh (never a replay of the other's recording); host
delivery through a re-uploaded program is right; a program destroyed after
its context is freed safely."""
import ctypes

import numpy as np
import pytest

import oracle
from isosurface_gb300 import Context, Program, scenes
from isosurface_gb300 import source as S
from isosurface_gb300._capi import MeshInfo, check, lib

pytestmark = pytest.mark.gpu

SIZE = 97


def _want(src):
    return oracle.Program(S.lower(src)).marching_cubes(SIZE)


def test_alternating_reuploads_extract_their_own_meshes():
    c = Context(0)
    srcs = {"sphere": scenes.sphere(), "csg": scenes.csg(), "torus": scenes.bench_torus()}
    want = {k: _want(v) for k, v in srcs.items()}
    order = ["sphere", "sphere", "sphere", "csg", "csg", "csg", "sphere", "csg", "torus", "torus", "torus", "sphere",
             "sphere"]
    for name in order:
        p = Program(c, srcs[name])
        got = c.download(c.mc_extract(p, SIZE))
        p.close()
        assert np.array_equal(got.vertices.reshape(-1), want[name].vertices.reshape(-1)), name
        assert np.array_equal(got.indices, want[name].indices), name
    c.close()


@pytest.mark.parametrize("flags", [0, 4])  # ISO_FLAG_HOST_COPY: delivery by copy after the extraction
def test_reuploaded_program_delivers_to_host_buffers(flags):
    c = Context(0)
    src = scenes.csg()
    want = _want(src)
    data = bytes(S.lower(src))
    nv, nt = len(want.vertices), len(want.indices) // 3
    v = np.zeros(3 * nv + 64, np.float32)
    i = np.zeros(3 * nt + 64, np.uint32)
    # page-locked, so that without ISO_FLAG_HOST_COPY the kernels write them
    check(lib().iso_host_register(v.ctypes.data_as(ctypes.c_void_p), v.nbytes))
    check(lib().iso_host_register(i.ctypes.data_as(ctypes.c_void_p), i.nbytes))
    f32p, u32p = ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint32)
    for _ in range(5):
        ph = ctypes.c_void_p()
        check(lib().iso_program_create(c.h, data, len(data), ctypes.byref(ph)), c.h)
        mi = MeshInfo()
        v[:] = 0
        i[:] = 0
        check(lib().iso_mc_extract_host(c.h, ph, SIZE, flags, v.ctypes.data_as(f32p), v.size, i.ctypes.data_as(u32p),
                                        i.size, ctypes.byref(mi)), c.h)
        lib().iso_program_destroy(ph)
        assert (mi.num_vertices, mi.num_triangles) == (nv, nt)
        assert np.array_equal(v[:3 * nv], want.vertices.reshape(-1))
        assert np.array_equal(i[:3 * nt], want.indices)
    lib().iso_host_unregister(v.ctypes.data_as(ctypes.c_void_p))
    lib().iso_host_unregister(i.ctypes.data_as(ctypes.c_void_p))
    c.close()


def test_program_destroyed_after_its_context():
    c = Context(0)
    p = Program(c, scenes.sphere())
    c.mc_extract(p, 17)
    c.close()
    p.close()  # the context is gone: the block is freed, not pooled
    c2 = Context(0)
    got = c2.download(c2.mc_extract(scenes.sphere(), SIZE))
    assert np.array_equal(got.indices, _want(scenes.sphere()).indices)
    c2.close()
