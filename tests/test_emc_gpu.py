"""GPU parity of ExtendedMarchingCubes (iso_emc_extract) against the oracle,
through the C ABI: bit-exact vertices and indices, the same number of rotated
edges, the normals sink, and the errors the entry point raises.

The kernels' per-item code is also checked on the host by test_emc_host.py;
these tests run the kernels themselves."""
import numpy as np
import pytest

import oracle
from isosurface_gb300 import ExtendedMarchingCubes, IndexedVertices, IsoError
from isosurface_gb300 import source as S

from emc_scenes import FIXED, random_scenes

pytestmark = pytest.mark.gpu


def _gpu(ctx, src, n, normals=False):
    info, flips = ctx.emc_extract(src, n, normals=normals)
    m = ctx.download(info)
    return m, flips, info


@pytest.mark.parametrize("name", sorted(FIXED))
@pytest.mark.parametrize("size", [2, 3, 16, 33, 65])
def test_emc_matches_oracle(ctx, name, size):
    src = FIXED[name]
    o = oracle.Program(S.lower(src)).extended_marching_cubes(size)
    m, flips, info = _gpu(ctx, src, size)
    assert info.num_cells == (size - 1) ** 2 * size
    assert np.array_equal(m.vertices, o.vertices)
    assert np.array_equal(m.indices, o.indices)
    assert flips == o.flips


def test_emc_random_csg(ctx):
    for n, src in random_scenes(23, 40):
        o = oracle.Program(S.lower(src)).extended_marching_cubes(n)
        m, flips, _ = _gpu(ctx, src, n)
        assert np.array_equal(m.vertices, o.vertices) and np.array_equal(m.indices, o.indices)
        assert flips == o.flips


def test_emc_normals(ctx):
    src = FIXED["cube"]
    o = oracle.Program(S.lower(src)).extended_marching_cubes(33, normals=True)
    m, _, _ = _gpu(ctx, src, 33, normals=True)
    assert m.vertices.shape[1] == 6
    assert np.array_equal(m.vertices[:, :3], o.vertices)
    assert np.array_equal(m.vertices[:, 3:], o.normals)


def test_emc_reference_api(ctx):
    """ExtendedMarchingCubes::new(n).extract(&sampler, &mut IndexedVertices)."""
    src = FIXED["difference"]
    vertices, indices = [], []
    ExtendedMarchingCubes(17, context=ctx).extract(S.Sampler(src), IndexedVertices(vertices, indices))
    o = oracle.Program(S.lower(src)).extended_marching_cubes(17)
    assert np.array_equal(np.asarray(vertices, np.float32).reshape(-1, 3), o.vertices)
    assert np.array_equal(np.asarray(indices, np.uint32), o.indices)


@pytest.mark.parametrize("src", [S.SmoothUnion(S.Sphere(0.2), S.Translate(S.Sphere(0.2), (0.1, 0.0, 0.0)), 0.05),
                                 S.Rigid(S.Sphere(0.3), (0.5, 0.5, 0.5), np.eye(3, dtype=np.float32)),
                                 S.SphereSet(np.array([[0.5, 0.5, 0.5, 0.3]], np.float32))])
def test_emc_rejects_sources_without_directed_metric(ctx, src):
    with pytest.raises(IsoError):
        ctx.emc_extract(src, 9)


def test_emc_size_bounds(ctx):
    info, flips = ctx.emc_extract(FIXED["sphere"], 1)
    assert info.num_vertices == 0 and info.num_triangles == 0 and flips == 0
    with pytest.raises(IsoError):
        ctx.emc_extract(FIXED["sphere"], 514)
