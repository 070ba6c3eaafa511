"""Failure handling: under an injected allocation failure (a host-side fake
of a failed cudaMalloc, iso_debug_fail_allocation) every extractor reports
ISO_ERR_OUT_OF_MEMORY and the same context then extracts the right mesh; a
bounded device-side wait that is made to run out (iso_debug_scan_timeout)
reports ISO_ERR_TIMEOUT and the next call extracts the right mesh.  Nothing
faults, traps or hangs on the device."""
import numpy as np
import pytest

import oracle
from isosurface_gb300 import Context, IsoError, scenes
from isosurface_gb300 import source as S

pytestmark = pytest.mark.gpu

OUT_OF_MEMORY = 7
TIMEOUT = 4


def _extract(c, kind, src):
    if kind == "lhmc":
        return c.lhmc_extract(src, 5, keys=True)
    if kind == "mc":
        return c.mc_extract(src, 65)
    if kind == "dc":
        return c.dc_extract(src, 33)
    if kind == "point_cloud":
        return c.point_cloud_extract(src, 33)
    return c.emc_extract(src, 33)[0]


def _reference(kind, src):
    p = oracle.Program(S.lower(src))
    return {"mc": lambda: p.marching_cubes(65), "dc": lambda: p.dual_contouring(33),
            "lhmc": lambda: p.lhmc(5), "point_cloud": lambda: p.point_cloud(33),
            "emc": lambda: p.extended_marching_cubes(33)}[kind]()


@pytest.mark.parametrize("kind", ["mc", "dc", "lhmc", "point_cloud", "emc"])
def test_allocation_failure_is_reported_and_the_context_recovers(kind):
    src = S.Translate(S.Sphere(0.3), (0.5, 0.5, 0.5)) if kind == "emc" else scenes.sphere()
    ref = _reference(kind, src)
    failures = 0
    for after in range(6):
        c = Context(0)
        try:
            c.debug_fail_allocation(after)
            try:
                _extract(c, kind, src)
            except IsoError as e:
                assert e.status == OUT_OF_MEMORY
                failures += 1
            c.debug_fail_allocation(-1)
            if kind == "lhmc":
                # the reference's order is HashMap order: triangle sets keyed
                # by MortonKey pairs, positions per key within 2 ulps
                from test_lhmc_gpu import _compare
                _compare(c.download(_extract(c, kind, src), keys=True), ref, 5)
            else:
                m = c.download(_extract(c, kind, src))
                assert np.array_equal(m.vertices, ref.vertices)
                assert np.array_equal(m.indices, ref.indices)
        finally:
            c.close()
    assert failures > 0


def test_lookback_wait_gives_up_and_the_next_call_recovers(ctx):
    """A bounded device-side wait that runs out: with iso_debug_scan_timeout
    the look-back scan's first block never publishes its status, the blocks
    behind it poll it 256 times, give up and flag it, and the call returns
    ISO_ERR_TIMEOUT.  The next call, with the hook off, extracts the oracle's
    mesh.  Every wait is bounded, so nothing hangs."""
    import ctypes

    import torch

    from isosurface_gb300._capi import MeshInfo, lib
    size = 65
    src = scenes.csg()
    pitch = size + 3
    field = torch.empty((size + 1) * size * pitch, dtype=torch.float32, device="cuda")
    ctx.sample_grid(src, size, field.data_ptr(), pitch)
    want = oracle.Program(S.lower(src)).marching_cubes(size)
    nv, nt = len(want.vertices), len(want.indices) // 3
    verts = torch.zeros(3 * nv, dtype=torch.float32, device="cuda")
    idx = torch.zeros(3 * nt, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()

    def call():
        info = MeshInfo()
        st = lib().iso_mc_extract_field_noalloc(ctypes.c_void_p(field.data_ptr()), size, size, size + 1, pitch,
                                                ctypes.c_void_p(verts.data_ptr()), nv,
                                                ctypes.c_void_p(idx.data_ptr()), nt, None, ctypes.byref(info))
        return st, info

    lib().iso_debug_scan_timeout(1)
    try:
        st, _ = call()
    finally:
        lib().iso_debug_scan_timeout(0)
    assert st == TIMEOUT
    st, info = call()
    assert st == 0 and (info.num_vertices, info.num_triangles) == (nv, nt)
    assert np.array_equal(verts.cpu().numpy().reshape(-1, 3), want.vertices)
    assert np.array_equal(idx.cpu().numpy().view(np.uint32), want.indices)
