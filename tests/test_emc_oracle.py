"""CPU tests of the oracle's ExtendedMarchingCubes (src/extended_marching_cubes.rs)
and of the Directed metric it samples (src/distance.rs:72-104).

The reference has no test of ExtendedMarchingCubes, so the oracle is pinned
by the Directed known answers of the primitives' own tests (test_oracle.py
runs them with the scalar and normal ones), by the EDGE_LOOPS table checked
against the fixture, and by what the algorithm guarantees:

* a smooth surface sampled finely spawns no feature, and the mesh is then
  marching cubes' mesh with the same connectivity, its vertices placed by
  the exact axis distances (on the sphere to ~1e-6 of a cell);
* on a cube (where the reference's box normal, the cardinal axis of the
  largest component, is the face normal) every feature vertex lands on a
  crease and exactly eight on the corners;
* every mesh is closed, edge-manifold and consistently oriented, with
  marching cubes' Euler characteristic, and no flip meets a face another
  flip rewrote (so the result does not depend on the order of the
  reference's HashSet).
"""
import json
import os
import sys

import numpy as np
import pytest

import oracle
from isosurface_gb300 import source as S

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
NO_KEY = np.uint64(0xFFFFFFFFFFFFFFFF)


def _manifold(tris):
    """(#undirected edges, #edges not shared by exactly two triangles, #directed duplicates)"""
    e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]])
    directed = e[:, 0].astype(np.int64) << 32 | e[:, 1].astype(np.int64)
    undirected = np.minimum(e[:, 0], e[:, 1]).astype(np.int64) << 32 | np.maximum(e[:, 0], e[:, 1]).astype(np.int64)
    u, c = np.unique(undirected, return_counts=True)
    return len(u), int(np.sum(c != 2)), len(directed) - len(np.unique(directed))


def _centred(src):
    return S.Translate(src, (0.5, 0.5, 0.5))


def test_edge_loops_table():
    """EDGE_LOOPS reaches the oracle's header entry for entry, and its loops
    cover each case's crossing edges."""
    t = json.load(open(os.path.join(HERE, "golden", "mc_tables.json")))
    sys.path.insert(0, os.path.join(ROOT, "isosurface_gb300", "csrc"))
    try:
        import gen_mc_tables
    finally:
        sys.path.pop(0)
    assert gen_mc_tables.check_edge_loops(t) == [167, 181, 229]
    text = open(os.path.join(ROOT, "oracle", "ref_tables.h")).read()
    body = text[text.index("EDGE_LOOPS[256][17]"):]
    body = body[body.index("{") + 1: body.index("};")]
    vals = [int(v) for v in body.replace("{", " ").replace("}", " ").replace(",", " ").split()]
    assert vals == sum(t["EDGE_LOOPS"], [])


@pytest.mark.parametrize("size", [16, 33, 65])
def test_emc_smooth_sphere_is_mc_with_exact_crossings(size):
    p = oracle.Program(S.lower(_centred(S.Sphere(0.3))))
    e = p.extended_marching_cubes(size)
    m = p.marching_cubes(size)
    assert e.features == 0 and e.flips == 0
    assert np.array_equal(e.indices, m.indices) and np.array_equal(e.keys, m.keys)
    assert e.cells == m.cells == (size - 1) ** 2 * size
    radial = np.abs(np.linalg.norm(e.vertices.astype(np.float64) - 0.5, axis=1) - 0.3) * (size - 1)
    assert radial.max() < 1e-5


@pytest.mark.parametrize("half", [0.27, 0.3])
@pytest.mark.parametrize("size", [16, 33])
def test_emc_cube_features_on_creases(half, size):
    p = oracle.Program(S.lower(_centred(S.RectangularPrism((half, half, half)))))
    m = p.extended_marching_cubes(size)
    feat = np.all(m.keys == NO_KEY, axis=1)
    assert feat.sum() == m.features > 0 and m.conflicts == 0 and m.flips >= m.features
    cell = 1.0 / (size - 1)
    assert np.abs(p.sample_scalar(m.vertices)).max() < 1e-5 * cell
    planes = (np.abs(np.abs(m.vertices - 0.5) - np.float32(half)) < 1e-5).sum(axis=1)
    assert np.all(planes[feat] >= 2)
    assert np.sum(planes[feat] == 3) == 8
    ne, bad, dup = _manifold(m.triangles)
    assert bad == 0 and dup == 0 and len(m.vertices) - ne + len(m.triangles) == 2
    # the flips turn the creases into mesh edges between feature vertices
    t = m.triangles
    e = np.concatenate([t[:, [0, 1]], t[:, [1, 2]], t[:, [2, 0]]])
    assert np.sum(feat[e[:, 0]] & feat[e[:, 1]]) > 0


@pytest.mark.parametrize("name", ["box", "cylinder", "torus", "csg"])
@pytest.mark.parametrize("size", [16, 33])
def test_emc_meshes_closed_and_oriented(name, size):
    src = {"box": S.RectangularPrism((0.31, 0.23, 0.17)),
           "cylinder": S.Cylinder(0.27, 0.21),
           "torus": S.Torus(0.25, 0.1),
           "csg": S.Difference(S.Sphere(0.3), S.RectangularPrism((0.26, 0.26, 0.26)))}[name]
    p = oracle.Program(S.lower(_centred(src)))
    e = p.extended_marching_cubes(size)
    m = p.marching_cubes(size)
    assert e.conflicts == 0
    ne, bad, dup = _manifold(e.triangles)
    assert bad == 0 and dup == 0
    mne, _, _ = _manifold(m.triangles)
    assert len(e.vertices) - ne + len(e.triangles) == len(m.vertices) - mne + len(m.triangles)
    # a feature cell replaces its triangles by fans around one new vertex
    assert len(e.vertices) == len(m.vertices) + e.features


def test_emc_normals_sink():
    """IndexedInterleavedNormals: the source's normal at every vertex,
    feature vertices included."""
    p = oracle.Program(S.lower(_centred(S.RectangularPrism((0.27, 0.27, 0.27)))))
    m = p.extended_marching_cubes(16, normals=True)
    assert m.features > 0
    assert np.array_equal(m.normals, p.sample_normal(m.vertices))


@pytest.mark.parametrize("src", [S.SmoothUnion(S.Sphere(0.2), S.Translate(S.Sphere(0.2), (0.1, 0.0, 0.0)), 0.05),
                                 S.Rigid(S.Sphere(0.3), (0.0, 0.0, 0.0), np.eye(3, dtype=np.float32))])
def test_emc_needs_directed_metric(src):
    """The reference defines sample_vector for its primitives and CSG only."""
    p = oracle.Program(S.lower(_centred(src)))
    assert not p.has_vector
    with pytest.raises(ValueError):
        p.extended_marching_cubes(8)


def test_emc_result_does_not_depend_on_flip_order():
    """The reference rotates its feature edges in HashSet order (random per
    run); any order gives the same mesh."""
    from emc_scenes import random_scenes
    for n, src in random_scenes(5, 25):
        p = oracle.Program(S.lower(src))
        base = p.extended_marching_cubes(n)
        for seed in (1, 2, 3):
            m = p.extended_marching_cubes(n, flip_order_seed=seed)
            assert m.flips == base.flips
            assert np.array_equal(m.indices, base.indices) and np.array_equal(m.vertices, base.vertices)
