"""GPU parity of the source evaluator, the grid sampler and MarchingCubes
against the oracle (CPU restatement of the reference), through the C ABI.

Parity bar: bit-exact.  The library reproduces MarchingCubes::extract's
IndexedVertices output byte for byte: same vertex order (first use in (z,y,x)
cell order), same positions, same index buffer."""
import json
import os

import numpy as np
import pytest

import oracle
from isosurface_gb300 import IsoError, scenes
from isosurface_gb300 import source as S

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _normalised(n):
    n = np.asarray(n, np.float32)
    l = np.float32(np.sqrt(np.float32(np.float32(n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])))
    return n / l


def test_reference_kats_on_gpu(ctx):
    """The reference's primitive known answers for values and normals,
    evaluated by the device VM (the Directed `sample_vector` answers belong
    to ExtendedMarchingCubes, which the oracle alone evaluates)."""
    for kat in json.load(open(os.path.join(GOLDEN, "kats.json"))):
        src = S.from_spec(kat["source"])
        if kat["kind"] == "scalar":
            v = ctx.sample_points(src, [kat["point"]])
            assert v[0] == np.float32(kat["expected"]), kat
        elif kat["kind"] == "normal":
            _, n = ctx.sample_points(src, [kat["point"]], normals=True)
            assert np.array_equal(_normalised(n[0]), np.asarray(kat["expected"], np.float32)), kat


def _sources():
    rng = np.random.default_rng(5)
    sph = rng.uniform(-0.8, 0.8, size=(20, 4)).astype(np.float32)
    sph[:, 3] = np.abs(sph[:, 3]) * 0.3 + 0.05
    return {
        "sphere": scenes.sphere(),
        "box": S.unit_to_cube(S.RectangularPrism((0.5, 0.3, 0.7))),
        "cylinder": S.unit_to_cube(S.Cylinder(0.4, 0.6)),
        "torus": scenes.bench_torus(),
        "csg": scenes.csg(),
        "intersection": S.unit_to_cube(S.Intersection(S.Sphere(0.8), S.RectangularPrism((0.6, 0.6, 0.6)))),
        "smooth": S.unit_to_cube(S.SmoothUnion(S.Translate(S.Sphere(0.3), (0.2, 0, 0)),
                                               S.Translate(S.Sphere(0.3), (-0.2, 0, 0)), 0.1)),
        "central_difference": S.unit_to_cube(S.CentralDifference(
            S.Union(S.Difference(S.Sphere(0.25), S.RectangularPrism((0.2, 0.2, 0.2))), S.Cylinder(0.02, 0.25)))),
        "sphere_set": S.unit_to_cube(S.SphereSet(sph)),
        "smooth_set": S.unit_to_cube(S.SphereSet(sph, smooth_k=0.05)),
        "set_nodomain": S.SphereSet(sph * np.float32([0.5, 0.5, 0.5, 0.5]) + np.float32([0.5, 0.5, 0.5, 0])),
        # a left fold of unions over translated primitives: compiled to a flat list on the device
        "prim_union": S.unit_to_cube(S.Union(S.Union(S.Union(
            S.Translate(S.Sphere(0.3), (0.2, -0.1, 0.05)), S.Translate(S.RectangularPrism((0.2, 0.3, 0.15)), (-0.3, 0.2, 0.1))),
            S.Translate(S.Torus(0.3, 0.08), (0.05, 0.35, -0.3))), S.Translate(S.Cylinder(0.12, 0.4), (-0.2, -0.4, 0.2)))),
    }


@pytest.mark.parametrize("name", sorted(_sources()))
def test_point_values_and_normals_bit_exact(ctx, name):
    src = _sources()[name]
    pts = np.random.default_rng(11).uniform(-0.1, 1.1, size=(4096, 3)).astype(np.float32)
    o = oracle.Program(S.lower(src))
    v, n = ctx.sample_points(src, pts, normals=True)
    assert np.array_equal(v, o.sample_scalar(pts))
    assert np.array_equal(n, o.sample_normal(pts))


@pytest.mark.parametrize("name", sorted(_sources()))
@pytest.mark.parametrize("size", [2, 5, 17, 40])
def test_mesh_bytes_identical(ctx, name, size):
    src = _sources()[name]
    o = oracle.Program(S.lower(src))
    want = o.marching_cubes(size)
    info = ctx.mc_extract(src, size, keys=True)
    got = ctx.download(info, keys=True)
    assert info.num_cells == (size - 1) * (size - 1) * size
    assert np.array_equal(got.keys, want.keys)
    assert np.array_equal(got.indices, want.indices)
    assert np.array_equal(got.vertices, want.vertices)


@pytest.mark.parametrize("name", ["sphere", "csg", "sphere_set", "torus"])
def test_cases_and_field_bit_exact(ctx, name):
    import torch
    src = _sources()[name]
    o = oracle.Program(S.lower(src))
    size = 33
    assert np.array_equal(ctx.mc_cases(src, size), o.mc_cases(size))
    pitch = 40
    field = torch.full(((size + 1) * size * pitch,), float("nan"), dtype=torch.float32, device="cuda")
    ctx.sample_grid(src, size, field.data_ptr(), pitch)
    got = field.view(size + 1, size, pitch)[:, :, :size].cpu().numpy()
    assert np.array_equal(got, o.sample_grid(size))


def test_c1_sphere_64(ctx):
    """64^3 cells over [-1,1]^3, sphere r=0.75: the reference's own CPU case."""
    src = scenes.sphere()
    want = oracle.Program(S.lower(src)).marching_cubes(65)
    got = ctx.download(ctx.mc_extract(src, 65, keys=True), keys=True)
    assert np.array_equal(got.vertices, want.vertices)
    assert np.array_equal(got.indices, want.indices)


def test_bench_torus_128(ctx):
    """The reference benchmark's MarchingCubes::new(128) on Torus(0.25, 0.1)."""
    src = scenes.bench_torus()
    want = oracle.Program(S.lower(src)).marching_cubes(128)
    got = ctx.download(ctx.mc_extract(src, 128))
    assert np.array_equal(got.vertices, want.vertices)
    assert np.array_equal(got.indices, want.indices)


def test_sphere_union_129(ctx):
    src = scenes.sphere_union()
    want = oracle.Program(S.lower(src)).marching_cubes(129)
    got = ctx.download(ctx.mc_extract(src, 129))
    assert np.array_equal(got.vertices, want.vertices)
    assert np.array_equal(got.indices, want.indices)


def test_extract_from_caller_field(ctx):
    import torch
    src = scenes.csg()
    o = oracle.Program(S.lower(src))
    size = 33
    g = torch.from_numpy(o.sample_grid(size)).cuda().contiguous()
    info = ctx.mc_extract_field(g.data_ptr(), size, size, size + 1, size)
    got = ctx.download(info)
    want = o.marching_cubes(size)
    assert np.array_equal(got.vertices, want.vertices)
    assert np.array_equal(got.indices, want.indices)


def test_full_size_512_parity(ctx):
    """The bench workload whole: MarchingCubes::new(513) on the seeded
    64-sphere union (512 x 512 x 513 cells).  Every cell's case equals the
    oracle's classification, and the vertex, index and lattice-edge key
    buffers equal the oracle's traversal of the whole grid byte for byte.
    The two oracle passes (about half a minute each on one core) run on
    host threads while the GPU extracts."""
    from concurrent.futures import ThreadPoolExecutor
    src = scenes.sphere_union()
    size = 513
    o = oracle.Program(S.lower(src))
    with ThreadPoolExecutor(2) as pool:
        f_mesh = pool.submit(o.marching_cubes, size)
        f_cases = pool.submit(o.mc_cases, size)
        info = ctx.mc_extract(src, size, keys=True)
        got = ctx.download(info, keys=True)
        cases = ctx.mc_cases(src, size)
        want_cases = f_cases.result()
        want = f_mesh.result()
    assert info.num_cells == (size - 1) ** 2 * size
    assert np.array_equal(cases.reshape(-1), want_cases.reshape(-1))
    assert info.num_triangles > 2_000_000
    assert np.array_equal(got.vertices, want.vertices)
    assert np.array_equal(got.indices, want.indices)
    assert np.array_equal(got.keys[:, 0], want.keys[:, 0])


def test_degenerate_sizes_and_errors(ctx):
    src = scenes.sphere()
    info = ctx.mc_extract(src, 1)
    assert info.num_vertices == 0 and info.num_triangles == 0
    with pytest.raises(IsoError):
        ctx.mc_extract(src, 0)
    for empty in (S.Sphere(-1.0), S.Sphere(10.0)):
        info = ctx.mc_extract(empty, 17)
        assert info.num_vertices == 0 and info.num_triangles == 0
    with pytest.raises(IsoError):
        ctx.program(b"ISO1" + b"\0" * 12)


def test_reference_style_api(ctx):
    """MarchingCubes::new(n).extract(&Sampler::new(&source), &mut IndexedVertices)."""
    from isosurface_gb300 import IndexedVertices, MarchingCubes, Sampler
    vertices, indices = [], []
    MarchingCubes(33, context=ctx).extract(Sampler(scenes.sphere()), IndexedVertices(vertices, indices))
    want = oracle.Program(S.lower(scenes.sphere())).marching_cubes(33)
    assert np.array_equal(np.asarray(vertices, np.float32), want.vertices.reshape(-1))
    assert np.array_equal(np.asarray(indices, np.uint32), want.indices)


@pytest.mark.parametrize("name", ["sphere", "csg", "torus", "smooth", "central_difference", "sphere_set"])
def test_mc_interleaved_normals(ctx, name):
    """IndexedInterleavedNormals (extractor.rs:97-127): each vertex followed
    by source.sample_normal(vertex), bit for bit as the oracle."""
    src = _sources()[name]
    want = oracle.Program(S.lower(src)).marching_cubes(33, normals=True)
    got = ctx.download(ctx.mc_extract(src, 33, normals=True))
    assert got.vertices.shape == (len(want.vertices), 6)
    assert np.array_equal(got.vertices[:, :3], want.vertices)
    assert np.array_equal(got.vertices[:, 3:], want.normals)
    assert np.array_equal(got.indices, want.indices)
    # the next plain extraction is 3 floats per vertex again
    plain = ctx.download(ctx.mc_extract(src, 33))
    assert plain.vertices.shape == (len(want.vertices), 3)


def test_reference_style_normals_sink(ctx):
    from isosurface_gb300 import IndexedInterleavedNormals, MarchingCubes, OnlyInterleavedNormals, Sampler
    src = scenes.csg()
    want = oracle.Program(S.lower(src)).marching_cubes(21, normals=True)
    v, i = [], []
    MarchingCubes(21, context=ctx).extract(Sampler(src), IndexedInterleavedNormals(v, i, src))
    inter = np.concatenate([want.vertices, want.normals], 1).reshape(-1)
    assert np.array_equal(np.asarray(v, np.float32), inter)
    assert np.array_equal(np.asarray(i, np.uint32), want.indices)
    v2 = []
    MarchingCubes(21, context=ctx).extract(Sampler(src), OnlyInterleavedNormals(v2, src))
    assert np.array_equal(np.asarray(v2, np.float32), inter)


@pytest.mark.parametrize("name", sorted(_sources()))
@pytest.mark.parametrize("size", [1, 2, 5, 17, 40])
def test_point_cloud_bytes_identical(ctx, name, size):
    """PointCloud::extract (point_cloud.rs:50-63): active-cell centres in
    traversal order."""
    src = _sources()[name]
    want = oracle.Program(S.lower(src)).point_cloud(size)
    info = ctx.point_cloud_extract(src, size)
    got = ctx.download(info)
    assert info.num_triangles == 0 and info.num_cells == want.cells
    assert np.array_equal(got.vertices, want.vertices)


def test_point_cloud_full_size_and_normals(ctx):
    src = scenes.sphere_union()
    o = oracle.Program(S.lower(src))
    want = o.point_cloud(129)
    got = ctx.download(ctx.point_cloud_extract(src, 129, normals=True))
    assert np.array_equal(got.vertices[:, :3], want.vertices)
    assert np.array_equal(got.vertices[:, 3:], o.sample_normal(want.vertices))
    # 512^3: count and a slab of centres against the oracle's cases
    info = ctx.point_cloud_extract(src, 513)
    cases = ctx.mc_cases(src, 513)
    assert info.num_vertices == int(np.count_nonzero((cases != 0) & (cases != 255)))


def test_point_cloud_reference_style_api(ctx):
    from isosurface_gb300 import OnlyVertices, PointCloud, Sampler
    v = []
    PointCloud(33, context=ctx).extract(Sampler(scenes.bench_torus()), OnlyVertices(v))
    want = oracle.Program(S.lower(scenes.bench_torus())).point_cloud(33)
    assert np.array_equal(np.asarray(v, np.float32), want.vertices.reshape(-1))


@pytest.mark.parametrize("size", [33, 129])
def test_sphere_union_near_only_values(ctx, size):
    """MarchingCubes on a sphere union samples signs everywhere but exact
    values only within one lattice step of the surface; fill the context's
    field with another source's values first so a missing value cannot pass
    by coincidence."""
    for src in (scenes.sphere_union(), S.unit_to_cube(S.SphereSet(
            np.array([[0.1, -0.2, 0.05, 0.5], [-0.3, 0.3, -0.1, 0.35], [0.35, 0.25, 0.3, 0.2]], np.float32)))):
        ctx.mc_extract(scenes.bench_torus(), size)  # generic sampler: writes every value
        got = ctx.download(ctx.mc_extract(src, size))
        want = oracle.Program(S.lower(src)).marching_cubes(size)
        assert np.array_equal(got.vertices, want.vertices)
        assert np.array_equal(got.indices, want.indices)


def test_repeated_extractions_replay_the_recorded_graph(ctx):
    """A (program, size) extracted twice in a row is recorded as one CUDA graph
    and replayed afterwards: replays give the same bytes as the eager run,
    also after other extractions, a keys flag change and a buffer regrowth
    (which must force a new recording rather than a stale replay)."""
    src = scenes.sphere_union()
    want = oracle.Program(S.lower(src)).marching_cubes(97)
    prog = ctx.program(src)

    def check(keys=False):
        got = ctx.download(ctx.mc_extract(prog, 97, keys=keys), keys=keys)
        assert np.array_equal(got.vertices, want.vertices)
        assert np.array_equal(got.indices, want.indices)
        if keys:
            assert np.array_equal(got.keys, want.keys)

    for _ in range(4):  # eager, eager + record, replay, replay
        check()
    launches = ctx.kernel_launches
    check()
    assert ctx.kernel_launches > launches  # replays still count their kernels
    ctx.mc_extract(scenes.bench_torus(), 97)  # another program in between
    check()
    check()
    for _ in range(3):
        check(keys=True)
    check()
    # a much larger mesh regrows the context's buffers; the recorded graph
    # must not write into the freed ones
    ctx.mc_extract(src, 301)
    for _ in range(3):
        check()


def test_1024_cubed_block_emit_fallback(ctx):
    """new(1025): 3.2e9 lattice edges do not fit the 32-bit edge map, so the
    block emit resolves owners itself (on near-surface sampled values).  A
    middle slab of cell layers must equal the oracle's traversal of that slab,
    and every vertex must be used once per distinct lattice edge."""
    src = scenes.sphere_union()
    size = 1025
    info = ctx.mc_extract(src, size, keys=True)
    got = ctx.download(info, keys=True)
    cases = ctx.mc_cases(src, size)
    tri_count = np.array(json.load(open(os.path.join(GOLDEN, "mc_tables.json")))["TRIANGLE_CONNECTION"])
    ntri = (tri_count[:, 0::3][:, :5] >= 0).sum(1)
    per_layer = ntri[cases.reshape(size, -1)].sum(1)
    del cases
    assert per_layer.sum() == info.num_triangles
    z0, z1 = 511, 513
    t0, t1 = int(per_layer[:z0].sum()), int(per_layer[:z1].sum())
    want = oracle.Program(S.lower(src)).marching_cubes_slab(size, z0, z1)
    assert np.array_equal(got.keys[:, 0][got.indices[3 * t0:3 * t1]], want.keys[:, 0][want.indices])
    gv = got.vertices[got.indices[3 * t0:3 * t1]]
    wv = want.vertices[want.indices]
    assert np.max(np.abs(gv - wv)) <= 1e-5 / (size - 1)
    # every vertex is used and every key is distinct
    assert len(np.unique(got.indices)) == info.num_vertices
    assert len(np.unique(got.keys[:, 0])) == info.num_vertices


def _pinned(n, dtype):
    import torch
    return torch.empty(n, dtype=dtype, pin_memory=True)


def test_extract_into_host_buffers(ctx):
    """iso_mc_extract_host: page-locked buffers are filled by the extraction
    kernels themselves (eager, recording and replayed runs), pageable ones by
    a copy; both give the oracle's bytes, and the mesh stays on the device."""
    import torch
    src = scenes.sphere_union()
    size = 161
    want = oracle.Program(S.lower(src)).marching_cubes(size)
    nv, nt = len(want.vertices), len(want.indices) // 3
    prog = ctx.program(src)
    pv, pi = _pinned(3 * nv + 7, torch.float32), _pinned(3 * nt + 5, torch.int32)
    for _ in range(4):  # eager, eager + record, replay, replay
        pv.fill_(-1.0)
        pi.fill_(-1)
        info = ctx.mc_extract_host(prog, size, pv, pi)
        assert (info.num_vertices, info.num_triangles) == (nv, nt)
        assert np.array_equal(pv.numpy()[:3 * nv].reshape(-1, 3), want.vertices)
        assert np.array_equal(pi.numpy()[:3 * nt].view(np.uint32), want.indices)
        assert (pv.numpy()[3 * nv:] == -1.0).all() and (pi.numpy()[3 * nt:] == -1).all()
    on_dev = ctx.download(info)
    assert np.array_equal(on_dev.vertices, want.vertices) and np.array_equal(on_dev.indices, want.indices)
    # other page-locked buffers after the recording: no replay into the old ones
    qv, qi = _pinned(3 * nv, torch.float32), _pinned(3 * nt, torch.int32)
    pv.fill_(-1.0)
    for _ in range(3):
        ctx.mc_extract_host(prog, size, qv, qi)
        assert np.array_equal(qv.numpy().reshape(-1, 3), want.vertices)
        assert np.array_equal(qi.numpy().view(np.uint32), want.indices)
    assert (pv.numpy() == -1.0).all()
    # pageable numpy buffers take the copy path
    v = np.zeros((nv, 3), np.float32)
    i = np.zeros(3 * nt, np.uint32)
    ctx.mc_extract_host(prog, size, v, i)
    assert np.array_equal(v, want.vertices) and np.array_equal(i, want.indices)


def test_extract_into_host_buffers_too_small(ctx):
    """Buffers one element short: ISO_ERR_CAPACITY, nothing written, the
    sizes reported and the mesh downloadable afterwards."""
    import ctypes

    import torch
    from isosurface_gb300._capi import MeshInfo, lib
    src = scenes.sphere_union()
    size = 97
    want = oracle.Program(S.lower(src)).marching_cubes(size)
    nv, nt = len(want.vertices), len(want.indices) // 3
    prog = ctx.program(src)
    for short_v in (True, False):
        pv = _pinned(3 * nv - (1 if short_v else 0), torch.float32).fill_(7.0)
        pi = _pinned(3 * nt - (0 if short_v else 1), torch.int32).fill_(7)
        for _ in range(3):
            info = MeshInfo()
            st = lib().iso_mc_extract_host(ctx.h, prog.h, size, 0, ctypes.c_void_p(pv.data_ptr()), pv.numel(),
                                           ctypes.c_void_p(pi.data_ptr()), pi.numel(), ctypes.byref(info))
            assert st == 2  # ISO_ERR_CAPACITY
            assert (info.num_vertices, info.num_triangles) == (nv, nt)
            assert (pv.numpy() == 7.0).all() and (pi.numpy() == 7).all()
        got = ctx.download(info)
        assert np.array_equal(got.vertices, want.vertices) and np.array_equal(got.indices, want.indices)


def test_extract_into_host_buffers_with_normals(ctx):
    import torch
    src = scenes.csg()
    size = 65
    want = oracle.Program(S.lower(src)).marching_cubes(size, normals=True)
    nv, nt = len(want.vertices), len(want.indices) // 3
    pv, pi = _pinned(6 * nv, torch.float32), _pinned(3 * nt, torch.int32)
    info = ctx.mc_extract_host(src, size, pv, pi, normals=True)
    assert (info.num_vertices, info.num_triangles) == (nv, nt)
    got = pv.numpy().reshape(-1, 6)
    assert np.array_equal(got[:, :3], want.vertices) and np.array_equal(got[:, 3:], want.normals)
    assert np.array_equal(pi.numpy().view(np.uint32), want.indices)


def test_extract_into_registered_numpy_buffers(ctx):
    """Ordinary host arrays page-locked with iso_host_register take the
    direct path and give the oracle's bytes; registering twice is refused."""
    import ctypes

    from isosurface_gb300._capi import lib
    src = scenes.sphere_union()
    size = 129
    want = oracle.Program(S.lower(src)).marching_cubes(size)
    v = np.zeros((len(want.vertices) + 3, 3), np.float32)
    i = np.zeros(len(want.indices) + 8, np.uint32)
    for a in (v, i):
        assert lib().iso_host_register(ctypes.c_void_p(a.ctypes.data), a.nbytes) == 0
    try:
        assert lib().iso_host_register(ctypes.c_void_p(v.ctypes.data), v.nbytes) == 1
        for _ in range(3):
            info = ctx.mc_extract_host(src, size, v, i)
            assert np.array_equal(v[:info.num_vertices], want.vertices)
            assert np.array_equal(i[:3 * info.num_triangles], want.indices)
    finally:
        for a in (v, i):
            assert lib().iso_host_unregister(ctypes.c_void_p(a.ctypes.data)) == 0
    assert lib().iso_host_unregister(ctypes.c_void_p(v.ctypes.data)) == 1


def test_extract_into_host_buffers_257(ctx):
    """Delivery to page-locked buffers at 257^3 (16K segments, several
    resolve steps per thread): eager, recorded and replayed runs give the
    oracle's bytes."""
    import torch
    src = scenes.sphere_union()
    size = 257
    want = oracle.Program(S.lower(src)).marching_cubes(size)
    nv, nt = len(want.vertices), len(want.indices) // 3
    prog = ctx.program(src)
    pv, pi = _pinned(3 * nv, torch.float32), _pinned(3 * nt, torch.int32)
    for _ in range(4):
        pv.fill_(0.0)
        pi.fill_(0)
        info = ctx.mc_extract_host(prog, size, pv, pi)
        assert (info.num_vertices, info.num_triangles) == (nv, nt)
        assert np.array_equal(pv.numpy().reshape(-1, 3), want.vertices)
        assert np.array_equal(pi.numpy().view(np.uint32), want.indices)
    got = ctx.download(info)
    assert np.array_equal(got.indices, want.indices)
