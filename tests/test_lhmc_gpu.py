"""GPU parity of LinearHashedMarchingCubes against the oracle.

The reference walks its primal-vertex HashMap in RandomState order, so its
output order is not defined; the comparison is on the triangle set keyed by
MortonKey pairs (index_cache.rs:63-73) with winding preserved, and on vertex
positions per key (within 2 ulps: a vertex shared by two cubes may be
computed from either end of its edge)."""
import numpy as np
import pytest

import oracle
from isosurface_gb300 import scenes
from isosurface_gb300 import source as S

pytestmark = pytest.mark.gpu


def _tri_keys(mesh):
    k = (mesh.keys[:, 0].astype(np.uint64) << np.uint64(32)) | mesh.keys[:, 1].astype(np.uint64)
    return k[mesh.indices.reshape(-1, 3)]


def _compare(got, want, max_depth):
    gt, wt = _tri_keys(got), _tri_keys(want)
    assert len(gt) == len(wt)
    gs = gt[np.lexsort(gt.T[::-1])]
    ws = wt[np.lexsort(wt.T[::-1])]
    assert np.array_equal(gs, ws)
    gk = (got.keys[:, 0] << np.uint64(32)) | got.keys[:, 1]
    wk = (want.keys[:, 0].astype(np.uint64) << np.uint64(32)) | want.keys[:, 1].astype(np.uint64)
    assert len(np.unique(gk)) == len(gk)
    go, wo = np.argsort(gk), np.argsort(wk)
    assert np.array_equal(gk[go], wk[wo])
    # 1e-5 of the finest cell, but at least 2 ulps of the [0,1] coordinates:
    # which cube interpolates a shared edge first (and so in which direction)
    # follows the reference's HashMap order, so it varies run to run there too
    cell = 1.0 / (1 << max_depth)
    tol = max(1e-5 * cell, 2 * float(np.spacing(np.float32(1.0))))
    assert np.max(np.abs(got.vertices[go] - want.vertices[wo])) <= tol


@pytest.mark.parametrize("name,src", [
    ("sphere", scenes.sphere()),
    ("csg", scenes.csg()),
    ("torus_bench", scenes.bench_torus()),
    ("box", S.unit_to_cube(S.RectangularPrism((0.5, 0.3, 0.4)))),
    ("sphere_union", scenes.sphere_union()),
])
@pytest.mark.parametrize("max_depth", [2, 4, 6])
def test_lhmc_triangle_sets(ctx, name, src, max_depth):
    want = oracle.Program(S.lower(src)).lhmc(max_depth)
    assert want.stale_corners == 0
    info = ctx.lhmc_extract(src, max_depth, keys=True)
    assert ctx.lhmc_stale_corners == 0
    got = ctx.download(info, keys=True)
    _compare(got, want, max_depth)


def test_lhmc_reference_bench_depth7(ctx):
    """benches/isosurface.rs: LinearHashedMarchingCubes::new(7) on Torus(0.25, 0.1)."""
    src = scenes.bench_torus()
    want = oracle.Program(S.lower(src)).lhmc(7)
    got = ctx.download(ctx.lhmc_extract(src, 7, keys=True), keys=True)
    _compare(got, want, 7)


def test_lhmc_csg_depth8(ctx):
    """The LinearHashedMarchingCubes workload: depth 8 on the rigid-transformed CSG scene."""
    src = scenes.csg()
    want = oracle.Program(S.lower(src)).lhmc(8)
    got = ctx.download(ctx.lhmc_extract(src, 8, keys=True), keys=True)
    assert len(want.triangles) > 10000
    _compare(got, want, 8)


def test_lhmc_deterministic(ctx):
    src = scenes.csg()
    a = ctx.download(ctx.lhmc_extract(src, 6, keys=True), keys=True)
    b = ctx.download(ctx.lhmc_extract(src, 6, keys=True), keys=True)
    assert np.array_equal(a.indices, b.indices) and np.array_equal(a.vertices, b.vertices)


def test_lhmc_reference_style_api(ctx):
    from isosurface_gb300 import IndexedVertices, LinearHashedMarchingCubes, Sampler
    v, i = [], []
    LinearHashedMarchingCubes(5, context=ctx).extract(Sampler(scenes.sphere()), IndexedVertices(v, i))
    want = oracle.Program(S.lower(scenes.sphere())).lhmc(5)
    assert len(i) == len(want.indices) and len(v) == 3 * len(want.vertices)


def test_lhmc_interleaved_normals(ctx):
    src = scenes.csg()
    plain = ctx.download(ctx.lhmc_extract(src, 6))
    got = ctx.download(ctx.lhmc_extract(src, 6, normals=True))
    assert np.array_equal(got.vertices[:, :3], plain.vertices)
    assert np.array_equal(got.indices, plain.indices)
    o = oracle.Program(S.lower(src))
    assert np.array_equal(got.vertices[:, 3:], o.sample_normal(plain.vertices))


def test_lhmc_repeated_extractions_replay(ctx):
    """The same (program, depth) twice in a row is recorded as one CUDA graph
    with its counts; replays must give the eager run's bytes, also after
    another program in between and with keys."""
    src = scenes.csg()
    prog = ctx.program(src)
    first = ctx.download(ctx.lhmc_extract(prog, 6))
    for _ in range(4):  # eager, eager + record, replay, replay
        got = ctx.download(ctx.lhmc_extract(prog, 6))
        assert np.array_equal(got.vertices, first.vertices)
        assert np.array_equal(got.indices, first.indices)
    ctx.lhmc_extract(scenes.sphere(), 6)
    for _ in range(3):
        got = ctx.download(ctx.lhmc_extract(prog, 6, keys=True), keys=True)
        assert np.array_equal(got.vertices, first.vertices)
        assert np.array_equal(got.indices, first.indices)
    want = oracle.Program(S.lower(src)).lhmc(6)
    assert len(got.indices) == len(want.indices)
