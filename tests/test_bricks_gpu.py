"""Culled sampling for the extractors (iso_sample_grid_near, the batch
sampler): sign bits everywhere, values wherever marching cubes can read them.

Against the full sampler (iso_sample_grid, itself pinned to the oracle in
test_mc_gpu.py) on the same program and size:
  * every sign bit is equal (bits past the last sample of a row clear);
  * every value written is bit-identical, and every end of an edge whose
    signs differ (the only values marching cubes reads) is written;
  * the culling is real: far from the surface values are left unwritten;
and the meshes extracted through the culled sampler equal the meshes of the
full field byte for byte.  Programs: the MarchingCubes test sources, random
chunk scenes (unions of translated primitives, which also prune primitives
per sub-brick) and a domain map with a large scale."""
import numpy as np
import pytest

from isosurface_gb300 import scenes
from isosurface_gb300 import source as S
from isosurface_gb300.scenes import SplitMix64

from test_mc_gpu import _sources

pytestmark = pytest.mark.gpu


def _programs():
    out = dict(_sources())
    rng = SplitMix64(2024)
    for i in range(4):
        out["chunk%d" % i] = scenes.chunk_scene(rng)
    out["scaled_domain"] = S.DomainMap(S.Union(S.Translate(S.Sphere(300.0), (100.0, 0.0, 0.0)),
                                               S.Translate(S.Torus(250.0, 60.0), (-120.0, 50.0, 0.0))),
                                       scale=(1000.0, 1000.0, 1000.0), offset=(-500.0, -500.0, -500.0))
    out["csg_rigid"] = scenes.csg(seed=7)
    # unions of translated primitives past 32 (64-bit keep masks) and past 64
    # (no pruning, classification only)
    for n in (40, 70):
        r = np.random.default_rng(n)
        prims = [S.Translate(S.Sphere(float(r.uniform(0.05, 0.2))) if i % 2 else
                             S.RectangularPrism(tuple(float(x) for x in r.uniform(0.03, 0.15, 3))),
                             tuple(float(x) for x in r.uniform(-0.8, 0.8, 3))) for i in range(n)]
        u = prims[0]
        for q in prims[1:]:
            u = S.Union(u, q)
        out["prims%d" % n] = S.unit_to_cube(u)
    return out


# programs on the culled general path whose surface is small against the grid
CULLED = {"box", "csg", "csg_rigid", "cylinder", "intersection", "prim_union", "scaled_domain", "smooth", "sphere",
          "torus", "central_difference"}


def _pack(inside, W):
    import torch
    nz, ny, nx = inside.shape
    pad = torch.zeros((nz, ny, 32 * W), dtype=torch.int64, device=inside.device)
    pad[:, :, :nx] = inside.to(torch.int64)
    weights = torch.bitwise_left_shift(torch.ones(32, dtype=torch.int64, device=inside.device),
                                       torch.arange(32, device=inside.device))
    return (pad.view(nz, ny, W, 32) * weights).sum(-1)


def _crossing_ends(inside):
    import torch
    need = torch.zeros_like(inside)
    for axis in (0, 1, 2):
        n = inside.shape[axis]
        a = inside.narrow(axis, 0, n - 1)
        b = inside.narrow(axis, 1, n - 1)
        d = a != b
        need.narrow(axis, 0, n - 1).logical_or_(d)
        need.narrow(axis, 1, n - 1).logical_or_(d)
    return need


# below about one tile of 4 layers x 32 rows per SM (here 17 and 65) the
# library takes the plain sampler; 161 and 200 take the culled one
@pytest.mark.parametrize("name", sorted(_programs()))
@pytest.mark.parametrize("size", [17, 65, 161, 200])
def test_near_sampling_matches_full(ctx, name, size):
    import torch
    src = _programs()[name]
    pitch = size + 3
    W = (size + 31) // 32
    full = torch.empty(((size + 1) * size * pitch,), dtype=torch.float32, device="cuda")
    ctx.sample_grid(src, size, full.data_ptr(), pitch)
    near = torch.full_like(full, float("nan"))
    bits = torch.full(((size + 1) * size * W,), -1, dtype=torch.int32, device="cuda")
    ctx.sample_grid_near(src, size, near.data_ptr(), pitch, bits.data_ptr())
    f = full.view(size + 1, size, pitch)[:, :, :size]
    g = near.view(size + 1, size, pitch)[:, :, :size]
    assert not torch.isnan(f).any()
    inside = ~(f > 0)
    want_bits = _pack(inside, W)
    got_bits = bits.view(size + 1, size, W).to(torch.int64) & 0xFFFFFFFF
    assert torch.equal(got_bits, want_bits)
    written = ~torch.isnan(g)
    assert torch.equal(f.view(torch.int32)[written], g.view(torch.int32)[written])
    need = _crossing_ends(inside)
    assert bool(written[need].all()), int((need & ~written).sum())
    if size == 200 and name in CULLED:
        # far from the surface nothing is evaluated
        assert float(written.float().mean()) < 0.5


@pytest.mark.parametrize("name", ["csg", "prim_union", "smooth", "central_difference", "chunk1", "scaled_domain"])
def test_culled_mesh_equals_full_field_mesh(ctx, name):
    import torch
    src = _programs()[name]
    size = 161
    pitch = size
    full = torch.empty(((size + 1) * size * pitch,), dtype=torch.float32, device="cuda")
    ctx.sample_grid(src, size, full.data_ptr(), pitch)
    want = ctx.download(ctx.mc_extract_field(full.data_ptr(), size, size, size + 1, pitch))
    got = ctx.download(ctx.mc_extract(src, size))
    assert np.array_equal(got.vertices, want.vertices)
    assert np.array_equal(got.indices, want.indices)


@pytest.mark.parametrize("name", ["csg", "prim_union", "chunk2", "prims40", "prims70"])
def test_culled_mesh_equals_oracle(ctx, name):
    import oracle
    src = _programs()[name]
    want = oracle.Program(S.lower(src)).marching_cubes(161)
    got = ctx.download(ctx.mc_extract(src, 161, keys=True), keys=True)
    assert np.array_equal(got.keys, want.keys)
    assert np.array_equal(got.indices, want.indices)
    assert np.array_equal(got.vertices, want.vertices)


@pytest.mark.parametrize("name", sorted(_programs()))
def test_lipschitz_bound_holds(ctx, name):
    """The bound the culling relies on, checked on random pairs of nearby
    points: |f(a) - f(b)| <= lip |a - b| (up to f32 rounding)."""
    src = _programs()[name]
    lip = ctx.lipschitz(src)
    assert lip > 0
    rng = np.random.default_rng(3)
    a = rng.uniform(0.0, 1.0, size=(20000, 3)).astype(np.float32)
    b = (a + rng.normal(0.0, 0.01, size=a.shape)).astype(np.float32)
    fa = ctx.sample_points(src, a).astype(np.float64)
    fb = ctx.sample_points(src, b).astype(np.float64)
    dist = np.linalg.norm(a.astype(np.float64) - b.astype(np.float64), axis=1)
    slack = 1e-5 * (1.0 + np.maximum(np.abs(fa), np.abs(fb)))
    assert np.all(np.abs(fa - fb) <= lip * dist * (1 + 1e-4) + slack)


def test_compiled_evaluator_matches_interpreter(ctx):
    """General programs are sampled by a kernel compiled for them (NVRTC);
    with compilation switched off the interpreter runs instead, and the
    sign bits and every value both write are identical."""
    import torch
    from isosurface_gb300._capi import lib
    progs = _programs()
    for name in ("csg", "csg_rigid", "smooth", "central_difference", "intersection", "cylinder", "box"):
        assert ctx.compiled(progs[name]), name
    # sphere sets, and flat unions of translated primitives (pruned per sub-brick by the interpreter)
    for name in ("sphere_set", "smooth_set", "prim_union", "chunk0", "prims40", "scaled_domain"):
        assert not ctx.compiled(progs[name]), name
    size, pitch = 200, 203
    W = (size + 31) // 32
    for name in ("csg", "smooth", "central_difference"):
        out = []
        for enable in (1, 0):
            lib().iso_jit_enable(enable)
            try:
                f = torch.full(((size + 1) * size * pitch,), float("nan"), dtype=torch.float32, device="cuda")
                b = torch.zeros(((size + 1) * size * W,), dtype=torch.int32, device="cuda")
                ctx.sample_grid_near(progs[name], size, f.data_ptr(), pitch, b.data_ptr())
                out.append((f.view(torch.int32).clone(), b.clone()))
            finally:
                lib().iso_jit_enable(1)
        assert torch.equal(out[0][1], out[1][1]), name
        assert torch.equal(out[0][0], out[1][0]), name  # the same samples written, the same bits


@pytest.mark.parametrize("name", ["csg", "csg_rigid", "smooth", "central_difference", "prim_union", "prims40",
                                  "prims70", "scaled_domain", "chunk0", "sphere_set"])
def test_compiled_full_field_matches_interpreter_and_oracle(ctx, name):
    """iso_sample_grid runs the program's compiled full-field kernel (every
    general program, flat unions of translated primitives included; sphere
    sets stay interpreted): the field is bit-identical to the interpreter's
    and to the oracle's at every sample."""
    import torch
    import oracle
    from isosurface_gb300._capi import lib
    src = _programs()[name]
    size, pitch = 97, 101
    out = []
    for enable in (1, 0):
        lib().iso_jit_enable(enable)
        try:
            f = torch.full(((size + 1) * size * pitch,), float("nan"), dtype=torch.float32, device="cuda")
            ctx.sample_grid(src, size, f.data_ptr(), pitch)
            out.append(f.view(size + 1, size, pitch)[:, :, :size].cpu().numpy())
        finally:
            lib().iso_jit_enable(1)
    assert np.array_equal(out[0].view(np.uint32), out[1].view(np.uint32)), name
    assert np.array_equal(out[0], oracle.Program(S.lower(src)).sample_grid(size)), name


def test_toggling_compilation_reruns_recorded_extractions(ctx):
    """A recorded extraction holds the sampler kernels of the setting it was
    recorded with: switching compilation off and on again must not replay
    the other setting's recording, and every mesh is the same."""
    from isosurface_gb300._capi import lib
    src = _programs()["csg"]
    size = 161
    want = None
    try:
        for enable in (1, 1, 1, 0, 0, 0, 1, 1):  # repeats record and replay each setting
            lib().iso_jit_enable(enable)
            launches0 = ctx.kernel_launches
            got = ctx.download(ctx.mc_extract(src, size))
            assert ctx.kernel_launches > launches0
            if want is None:
                want = got
            assert np.array_equal(got.vertices, want.vertices)
            assert np.array_equal(got.indices, want.indices)
    finally:
        lib().iso_jit_enable(1)
