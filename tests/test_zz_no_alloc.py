"""iso_mc_extract_field_noalloc: marching cubes for callers that cannot call
cudaMalloc / cudaFree (memory owned by the host application's allocator or
budget, per-frame loops that cannot take the implicit synchronisation of
those calls).  Its scratch is a fixed device array inside the library; the
caller passes the field and the output buffers.

Checked here through the C ABI against the allocating entry point
(iso_mc_extract_field) and against the oracle's MarchingCubes, on two calls
in a row, which must both match them exactly (the parity bar of the
marching-cubes tests: byte-identical meshes).
The second call also shows that leftovers in the shared scratch array from
the first call do not leak into the result.  This file is collected last on
purpose, and passes alone in a fresh process as well as after the others."""
import ctypes

import numpy as np
import pytest

import oracle
from isosurface_gb300 import scenes
from isosurface_gb300 import source as S
from isosurface_gb300._capi import MeshInfo, lib

pytestmark = pytest.mark.gpu

ISO_OK, ISO_ERR_INVALID_ARG, ISO_ERR_CAPACITY, ISO_ERR_TOO_LARGE = 0, 1, 2, 8


def _field(ctx, source, size):
    import torch
    pitch = size + 3
    field = torch.empty((size + 1) * size * pitch, dtype=torch.float32, device="cuda")
    ctx.sample_grid(source, size, field.data_ptr(), pitch)
    return field, pitch


def _noalloc(field, size, pitch, vcap, tcap):
    import torch
    verts = torch.zeros(max(vcap, 1) * 3, dtype=torch.float32, device="cuda")
    idx = torch.zeros(max(tcap, 1) * 3, dtype=torch.int32, device="cuda")
    info = MeshInfo()
    torch.cuda.synchronize()
    st = lib().iso_mc_extract_field_noalloc(ctypes.c_void_p(field.data_ptr()), size, size, size + 1, pitch,
                                            ctypes.c_void_p(verts.data_ptr()), vcap,
                                            ctypes.c_void_p(idx.data_ptr()), tcap, None, ctypes.byref(info))
    return st, info, verts, idx


@pytest.mark.parametrize("name,size", [("csg", 65), ("sphere_union", 97)])
def test_noalloc_matches_allocating_entry_point_twice(ctx, name, size):
    source = getattr(scenes, name)()
    field, pitch = _field(ctx, source, size)
    ref_info = ctx.mc_extract_field(field.data_ptr(), size, size, size + 1, pitch)
    ref = ctx.download(ref_info)
    nv, nt = ref_info.num_vertices, ref_info.num_triangles
    assert nt > 0
    want = oracle.Program(S.lower(source)).marching_cubes(size)
    assert np.array_equal(ref.vertices, want.vertices) and np.array_equal(ref.indices, want.indices)
    for _ in range(2):
        st, info, verts, idx = _noalloc(field, size, pitch, nv, nt)
        assert st == ISO_OK
        assert (info.num_vertices, info.num_triangles) == (nv, nt)
        got_v = verts[: 3 * nv].cpu().numpy().reshape(-1, 3)
        got_i = idx[: 3 * nt].cpu().numpy().view(np.uint32)
        assert np.array_equal(got_v, ref.vertices) and np.array_equal(got_v, want.vertices)
        assert np.array_equal(got_i, ref.indices) and np.array_equal(got_i, want.indices)


def test_noalloc_reports_sizes_and_limits(ctx):
    size = 33
    field, pitch = _field(ctx, scenes.sphere(), size)
    st, info, _, _ = _noalloc(field, size, pitch, 0, 0)
    assert st == ISO_ERR_CAPACITY and info.num_triangles > 0 and info.num_vertices > 0
    # a grid whose scratch exceeds the fixed array is refused before any work
    info = MeshInfo()
    st = lib().iso_mc_extract_field_noalloc(ctypes.c_void_p(field.data_ptr()), 1025, 1025, 1026, 1025, None, 0,
                                            None, 0, None, ctypes.byref(info))
    assert st == ISO_ERR_TOO_LARGE
    # a grid taller than the launch grid allows is refused up front
    info = MeshInfo()
    st = lib().iso_mc_extract_field_noalloc(ctypes.c_void_p(field.data_ptr()), 2, 2, 65537, 2, None, 0,
                                            None, 0, None, ctypes.byref(info))
    assert st == ISO_ERR_INVALID_ARG
