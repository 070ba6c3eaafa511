"""GPU parity of DualContouring (MinimiseQEF and ParticleBasedMinimisation
placers) against the oracle, through the C ABI.

The required bar is DC vertex positions within 1e-4 of a cell; the library follows the
reference's f32 and f64 operation order (the SVD of src/math/svd.rs included),
so the tests assert the stricter byte-identical output and report the
position difference if that ever fails."""
import numpy as np
import pytest

import oracle
from isosurface_gb300 import scenes
from isosurface_gb300 import source as S

pytestmark = pytest.mark.gpu


def _sources():
    return {
        "sphere": scenes.sphere(),
        "csg": scenes.csg(),
        "box": S.unit_to_cube(S.RectangularPrism((0.45, 0.3, 0.6))),
        "torus": S.unit_to_cube(S.Torus(0.5, 0.2)),
        "cylinder": S.unit_to_cube(S.Cylinder(0.4, 0.5)),
        "central_difference": S.unit_to_cube(S.CentralDifference(
            S.Intersection(S.Sphere(0.8), S.RectangularPrism((0.6, 0.6, 0.6))))),
    }


def _compare(got, want, size):
    assert np.array_equal(got.keys, want.keys)
    assert np.array_equal(got.indices, want.indices)
    diff = np.max(np.abs(got.vertices - want.vertices)) if len(want.vertices) else 0.0
    assert diff <= 1e-4 / (size - 1), diff
    assert np.array_equal(got.vertices, want.vertices), "positions within tolerance but not identical: %g" % diff


@pytest.mark.parametrize("placer", [0, 1])
@pytest.mark.parametrize("name", sorted(_sources()))
@pytest.mark.parametrize("size", [3, 9, 33])
def test_dc_bytes_identical(ctx, name, size, placer):
    src = _sources()[name]
    want = oracle.Program(S.lower(src)).dual_contouring(size, placer=placer)
    info = ctx.dc_extract(src, size, placer=placer, keys=True)
    got = ctx.download(info, keys=True)
    assert info.num_triangles == len(want.triangles)
    _compare(got, want, size)


@pytest.mark.parametrize("name", ["sphere", "torus", "central_difference", "box"])
def test_dc_culled_sampling_161(ctx, name):
    """A grid large enough for the culled sampler (values only near the
    surface): the dual values of skipped corners are never read as values."""
    src = _sources()[name]
    want = oracle.Program(S.lower(src)).dual_contouring(161, placer=0)
    got = ctx.download(ctx.dc_extract(src, 161, keys=True), keys=True)
    _compare(got, want, 161)


def test_dc_csg_257(ctx):
    """The DualContouring workload: 256^3 cells, rigid-transformed CSG scene,
    analytic-gradient normals, MinimiseQEF."""
    src = scenes.csg()
    want = oracle.Program(S.lower(src)).dual_contouring(257, placer=0)
    got = ctx.download(ctx.dc_extract(src, 257, keys=True), keys=True)
    assert len(want.triangles) > 10000
    _compare(got, want, 257)


def test_dc_reference_style_api(ctx):
    from isosurface_gb300 import DualContouring, IndexedVertices, ParticleBasedMinimisation, Sampler
    v, i = [], []
    DualContouring(17, ParticleBasedMinimisation(), context=ctx).extract(Sampler(scenes.csg()), IndexedVertices(v, i))
    want = oracle.Program(S.lower(scenes.csg())).dual_contouring(17, placer=1)
    assert np.array_equal(np.asarray(i, np.uint32), want.indices)
    assert np.array_equal(np.asarray(v, np.float32), want.vertices.reshape(-1))


def test_dc_small_sizes(ctx):
    for size in (1, 2):
        info = ctx.dc_extract(scenes.sphere(), size)
        assert info.num_triangles == 0


@pytest.mark.parametrize("placer", [0, 1])
def test_dc_interleaved_normals(ctx, placer):
    """DualContouring into IndexedInterleavedNormals: the DC mesh plus
    sample_normal at each placed vertex, bit for bit."""
    src = scenes.csg()
    o = oracle.Program(S.lower(src))
    want = o.dual_contouring(33, placer)
    got = ctx.download(ctx.dc_extract(src, 33, placer, normals=True))
    assert np.array_equal(got.vertices[:, :3], want.vertices)
    assert np.array_equal(got.vertices[:, 3:], o.sample_normal(want.vertices))
    assert np.array_equal(got.indices, want.indices)


@pytest.mark.parametrize("placer", [0, 1])
@pytest.mark.parametrize("name", ["csg", "torus", "cylinder", "box", "central_difference"])
def test_dc_compiled_and_interpreted_normals(ctx, name, placer):
    """DualContouring's placement runs the program's compiled normals when
    compilation is on (iso_jit_dc_place; a central difference stays with the
    interpreter), the interpreter's eval_hermite when it is off: both meshes
    equal the oracle's byte for byte."""
    from isosurface_gb300._capi import lib
    src = _sources()[name]
    size = 33
    want = oracle.Program(S.lower(src)).dual_contouring(size, placer=placer)
    for enable in (1, 0):
        lib().iso_jit_enable(enable)
        try:
            got = ctx.download(ctx.dc_extract(src, size, placer=placer, keys=True), keys=True)
        finally:
            lib().iso_jit_enable(1)
        _compare(got, want, size)
