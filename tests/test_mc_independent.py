"""Second, independent restatements of MarchingCubes::extract, of
DualContouring's traversal, of PointCloud, of LinearHashedMarchingCubes and
of ExtendedMarchingCubes in plain Python, for small grids, checked against the oracle (byte for byte;
LHMC as triangle sets, its reference output being in HashMap order) (which the
GPU library is checked against).  It follows the reference's own structure
rather than the oracle's: PrimalGrid::traverse (src/traversal/primal_grid.rs:
39-89) over tuples, classify_corners / find_edge_crossings / march_cube
(src/marching_cubes_impl.rs:26-117) over the tables as the reference declares
them (tests/golden/mc_tables.json), and MeshTopologyBuilder with an
IndexCache dict keyed by GridKey (src/mesh.rs:225-260, src/index_cache.rs:
17-61).  Field values come from the oracle's evaluator, which the
reference's known-answer tests pin; every f32 operation is done in numpy
float32 in the reference's order."""
import json
import os

import numpy as np
import pytest

import oracle
from isosurface_gb300 import scenes
from isosurface_gb300 import source as S

F = np.float32
T = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "mc_tables.json")))
CORNERS = [tuple(c) for c in T["CORNERS"]]
EDGE_CONNECTION = [tuple(e) for e in T["EDGE_CONNECTION"]]
EDGE_CROSSING_MASK = T["EDGE_CROSSING_MASK"]
TRIANGLE_CONNECTION = T["TRIANGLE_CONNECTION"]


def marching_cubes(prog, size):
    one_over_size = F(1.0) / F(size - 1)
    pts = np.array([(x, y, z) for z in range(size + 1) for y in range(size) for x in range(size)], np.float32)
    pos = pts * one_over_size  # x as f32 * one_over_size, per component
    val = prog.sample_scalar(pos)
    at = lambda x, y, z: (z * size + y) * size + x
    vertices, indices, cache = [], [], {}
    for z in range(size):
        for y in range(size - 1):
            for x in range(size - 1):
                keys = [(x + c[0], y + c[1], z + c[2]) for c in CORNERS]
                corners = [pos[at(*k)] for k in keys]
                values = [val[at(*k)] for k in keys]
                cube = 0
                for i in range(8):  # classify_corners: bit i when !(v > 0)
                    if not values[i] > F(0.0):
                        cube |= 1 << i
                verts = [None] * 12
                for i in range(12):  # find_edge_crossings + Signed::find_crossing_point
                    if EDGE_CROSSING_MASK[cube] & (1 << i):
                        u, v = EDGE_CONNECTION[i]
                        a, b = values[u], values[v]
                        delta = F(b - a)
                        t = F(0.5) if delta == F(0.0) else F(-a / delta)
                        verts[i] = corners[u] * F(F(1.0) - t) + corners[v] * t
                row = TRIANGLE_CONNECTION[cube]
                for k in range(0, 15, 3):  # march_cube
                    if row[k] < 0:
                        break
                    for e in row[k:k + 3]:
                        u, v = EDGE_CONNECTION[e]
                        key = tuple(sorted((keys[u], keys[v])))  # GridKey::new
                        if key not in cache:
                            cache[key] = len(cache)
                            vertices.append(verts[e])
                        indices.append(cache[key])
    return np.array(vertices, np.float32).reshape(-1, 3), np.array(indices, np.uint32)


@pytest.mark.parametrize("name", ["sphere", "csg", "torus", "union"])
@pytest.mark.parametrize("size", [2, 5, 12, 21])
def test_independent_restatement_matches_oracle(name, size):
    src = {"sphere": scenes.sphere(), "csg": scenes.csg(),
           "torus": S.Translate(S.Torus(0.25, 0.1), (0.5, 0.5, 0.5)),
           "union": scenes.sphere_union(count=8)}[name]
    prog = oracle.Program(S.lower(src))
    v, i = marching_cubes(prog, size)
    m = prog.marching_cubes(size)
    assert np.array_equal(v, m.vertices)
    assert np.array_equal(i, m.indices)
    if size == 12:
        assert len(i) > 30  # a real surface, not an empty mesh


def _normalised_or_zero(n):
    """Vec3::normalised (vector.rs:468-478) or zero, in f32."""
    n = np.asarray(n, np.float32)
    ln = np.sqrt(F(F(n[0] * n[0] + n[1] * n[1]) + n[2] * n[2]))
    if abs(ln) < F(1.1920929e-07):
        return np.zeros(3, np.float32)
    return n / ln


def dual_contouring(prog, size, placer):
    """DualContouring::extract (src/dual_contouring.rs:65-105) over
    DualGrid::traverse (src/traversal/dual_grid.rs:52-95): each primal cell's
    dual vertex (placed when the cell is active, else the cell centre) and
    value, then marching cubes on every dual cube once its far corner's cell
    is reached.  Feature placement is the oracle's (place_feature)."""
    one_over_size = F(1.0) / F(size - 1)
    m = size - 1
    pts = np.array([(x, y, z) for z in range(size + 1) for y in range(size) for x in range(size)], np.float32)
    pos = pts * one_over_size
    val = prog.sample_scalar(pos)
    at = lambda x, y, z: (z * size + y) * size + x
    duals = [[None] * (m * m), [None] * (m * m)]
    vertices, indices, cache = [], [], {}
    half = F(0.5)
    for z in range(size):
        for y in range(m):
            for x in range(m):
                keys = [(x + c[0], y + c[1], z + c[2]) for c in CORNERS]
                corners = np.array([pos[at(*k)] for k in keys], np.float32)
                values = [val[at(*k)] for k in keys]
                cube = sum(1 << i for i in range(8) if not values[i] > F(0.0))
                if cube in (0, 255):
                    vertex = corners[0] * F(F(1.0) - half) + corners[6] * half  # Vec3::lerp
                else:
                    normals = np.array([_normalised_or_zero(prog.sample_normal(c)[0]) for c in corners], np.float32)
                    vertex, _ = oracle.place_feature(corners, normals, placer)
                value = F(F(F(1.0) - half) * values[0]) + F(half * values[6])  # Signed::lerp
                duals[z % 2][y * m + x] = (np.asarray(vertex, np.float32), value)
                if x > 0 and y > 0 and z > 0:
                    bx, by, bz = x - 1, y - 1, z - 1
                    dkeys = [(bx + c[0], by + c[1], bz + c[2]) for c in CORNERS]
                    d = [duals[(bz + c[2]) % 2][(by + c[1]) * m + bx + c[0]] for c in CORNERS]
                    dc = [e[0] for e in d]
                    dv = [e[1] for e in d]
                    c2 = sum(1 << i for i in range(8) if not dv[i] > F(0.0))
                    verts = [None] * 12
                    for i in range(12):
                        if EDGE_CROSSING_MASK[c2] & (1 << i):
                            u, v = EDGE_CONNECTION[i]
                            delta = F(dv[v] - dv[u])
                            t = F(0.5) if delta == F(0.0) else F(-dv[u] / delta)
                            verts[i] = dc[u] * F(F(1.0) - t) + dc[v] * t
                    row = TRIANGLE_CONNECTION[c2]
                    for k in range(0, 15, 3):
                        if row[k] < 0:
                            break
                        for e in row[k:k + 3]:
                            u, v = EDGE_CONNECTION[e]
                            key = tuple(sorted((dkeys[u], dkeys[v])))
                            if key not in cache:
                                cache[key] = len(cache)
                                vertices.append(verts[e])
                            indices.append(cache[key])
    return np.array(vertices, np.float32).reshape(-1, 3), np.array(indices, np.uint32)


@pytest.mark.parametrize("placer", [0, 1])
@pytest.mark.parametrize("size", [3, 9, 14])
def test_independent_dual_contouring_matches_oracle(placer, size):
    prog = oracle.Program(S.lower(scenes.csg()))
    v, i = dual_contouring(prog, size, placer)
    m = prog.dual_contouring(size, placer)
    assert np.array_equal(v, m.vertices)
    assert np.array_equal(i, m.indices)
    if size == 14:
        assert len(i) > 30


@pytest.mark.parametrize("size", [2, 7, 16])
def test_independent_point_cloud_matches_oracle(size):
    """PointCloud::extract (src/point_cloud.rs:50-63): the centre
    corners[0].lerp(corners[6], 0.5) of every cell whose case is neither 0
    nor 255, in traversal order."""
    prog = oracle.Program(S.lower(scenes.csg()))
    one_over_size = F(1.0) / F(size - 1)
    half = F(0.5)
    out = []
    for z in range(size):
        for y in range(size - 1):
            for x in range(size - 1):
                keys = [(x + c[0], y + c[1], z + c[2]) for c in CORNERS]
                corners = np.array(keys, np.float32) * one_over_size
                values = prog.sample_scalar(corners)
                cube = sum(1 << i for i in range(8) if not values[i] > F(0.0))
                if cube not in (0, 255):
                    out.append(corners[0] * F(F(1.0) - half) + corners[6] * half)
    m = prog.point_cloud(size)
    assert np.array_equal(np.array(out, np.float32).reshape(-1, 3), m.vertices)


# -- LinearHashedMarchingCubes ------------------------------------------------
MASK64 = (1 << 64) - 1
DILATE_TZ, DILATE_TY, DILATE_TX = 0x4924924924924924, 0x2492492492492492, 0x9249249249249249
DILATE_T1, DILATE_T2, DILATE_T3 = 0xB6DB6DB6DB6DB6DB, 0xDB6DB6DB6DB6DB6D, 0x6DB6DB6DB6DB6DB6
LG2_3 = 0.48089834696
MAX_LEVEL = 21
SQRT_OF_3 = F(1.7320508)


def m_level(a):  # Morton::level: the reference's ln formula, floor((ln a) * LG2_3)
    import math
    return 0 if a == 0 else int(math.floor(math.log(float(a)) * LG2_3))


def m_size(a):
    return F(1.0) / F(2 << m_level(a))


def m_center(a):
    """Morton::center: de-interleave the bits below the level's top, then
    (b as f32) * size2 + size per axis."""
    lv = m_level(a)
    b = [0, 0, 0]
    for bit in range(lv):
        for axis in range(3):
            b[axis] |= ((a >> (3 * bit + axis)) & 1) << bit
    size = m_size(a)
    size2 = F(size * F(2.0))
    return np.array([F(F(b[k]) * size2) + size for k in range(3)], np.float32)


def m_add(a, b):
    return ((((a | DILATE_T1) + (b & DILATE_TZ)) & DILATE_TZ) | (((a | DILATE_T2) + (b & DILATE_TY)) & DILATE_TY)
            | (((a | DILATE_T3) + (b & DILATE_TX)) & DILATE_TX)) & MASK64


def m_sub(a, b):
    return ((((a & DILATE_TZ) - (b & DILATE_TZ)) & DILATE_TZ) | (((a & DILATE_TY) - (b & DILATE_TY)) & DILATE_TY)
            | (((a & DILATE_TX) - (b & DILATE_TX)) & DILATE_TX)) & MASK64


def m_primal_vertex(a, level, which):
    k = 1 << (3 * level)
    vk = m_add(a, which)
    dk = m_sub(vk, k)
    if vk >= (k << 1) or (dk & DILATE_TX) == 0 or (dk & DILATE_TY) == 0 or (dk & DILATE_TZ) == 0:
        return 0
    return (vk << (3 * (MAX_LEVEL - level))) & MASK64


def m_dual_vertex(a, level, which):
    return m_sub(a >> (3 * (MAX_LEVEL - level)), which)


def lhmc(prog, max_depth):
    """LinearHashedMarchingCubes::extract (src/linear_hashed_marching_cubes.rs:
    62-84) over ImplicitOctree::traverse (src/traversal/implicit_octree.rs:
    36-98) and LinearHashedOctree::build (src/linear_hashed_octree.rs:30-52).
    Returns {MortonKey pair: vertex}, the triangles as MortonKey-pair triples,
    and the number of dual-cube corners whose parent walk found no node."""
    from collections import deque
    nodes, leaves = {}, []
    queue = deque([1])
    while queue:
        key = queue.popleft()
        value = prog.sample_scalar(m_center(key))[0]
        lv = m_level(key)
        if lv < 2 or (lv < max_depth and abs(value) < F(m_size(key) * SQRT_OF_3)):
            queue.extend((key << 3) | i for i in range(8))
        else:
            leaves.append(key)
        nodes[key] = value
    primal = {}
    for key in leaves:
        lv = m_level(key)
        for i in range(8):
            v = m_primal_vertex(key, lv, i)
            if v != 0 and lv > primal.get(v, -1):
                primal[v] = lv
    verts, tris, missing = {}, [], 0
    REMAP = T["REMAP_CUBE"]
    for key, lv in sorted(primal.items()):
        keys, corners, values = [None] * 8, [None] * 8, [None] * 8
        for i in range(8):
            m = m_dual_vertex(key, lv, REMAP[i])
            while m > 1 and m not in nodes:
                m = max(m >> 3, 1)
            if m > 1:
                keys[i], corners[i], values[i] = m, m_center(m), nodes[m]
        if any(k is None for k in keys):
            missing += sum(k is None for k in keys)
            continue
        cube = sum(1 << i for i in range(8) if not values[i] > F(0.0))
        row = TRIANGLE_CONNECTION[cube]
        for k in range(0, 15, 3):
            if row[k] < 0:
                break
            tri = []
            for e in row[k:k + 3]:
                u, v = EDGE_CONNECTION[e]
                pair = tuple(sorted((keys[u], keys[v])))
                if pair not in verts:
                    delta = F(values[v] - values[u])
                    t = F(0.5) if delta == F(0.0) else F(-values[u] / delta)
                    verts[pair] = corners[u] * F(F(1.0) - t) + corners[v] * t
                tri.append(pair)
            tris.append(tuple(tri))
    return verts, tris, missing


def _canonical(tri):
    i = tri.index(min(tri))
    return tri[i:] + tri[:i]


@pytest.mark.parametrize("name,depth", [("sphere", 4), ("sphere", 5), ("torus", 5), ("csg", 5)])
def test_independent_lhmc_matches_oracle(name, depth):
    src = {"sphere": scenes.sphere(), "torus": S.Translate(S.Torus(0.25, 0.1), (0.5, 0.5, 0.5)),
           "csg": scenes.csg()}[name]
    prog = oracle.Program(S.lower(src))
    verts, tris, missing = lhmc(prog, depth)
    m = prog.lhmc(depth)
    assert missing == 0 and m.stale_corners == 0  # no corner depends on the HashMap's order
    keys = [tuple(int(x) for x in k) for k in m.keys]
    got = {_canonical(tuple(keys[j] for j in t)) for t in m.triangles}
    want = {_canonical(t) for t in tris}
    assert got == want and len(tris) == len(m.triangles) > 20
    for k, v in zip(keys, m.vertices):
        np.testing.assert_allclose(v, verts[k], rtol=0, atol=1e-6)


# -- ExtendedMarchingCubes ----------------------------------------------------
EDGE_LOOPS = T["EDGE_LOOPS"]


def emc(prog, size, rng):
    """ExtendedMarchingCubes::extract (src/extended_marching_cubes.rs:64-186)
    with MeshTopology's edge bookkeeping and rotate_edge (src/mesh.rs:64-172);
    the flips are chosen and applied in a shuffled order, as the reference's
    HashSet yields them in a random one.  Tangent planes and MinimiseQEF over
    a cell's crossings are the oracle's (emc_place)."""
    one_over_size = F(1.0) / F(size - 1)
    pts = np.array([(x, y, z) for z in range(size + 1) for y in range(size) for x in range(size)], np.float32)
    pos = pts * one_over_size
    vec = prog.sample_vector(pos)
    at = lambda x, y, z: (z * size + y) * size + x
    vertices, faces, cache, features = [], [], {}, set()
    edges, edge_to_face = set(), {}

    def add_vertex(key, v):
        if key is not None and key in cache:
            return cache[key]
        h = len(vertices)
        vertices.append(v)
        if key is not None:
            cache[key] = h
        return h

    def add_face(a, b, c):
        f = len(faces)
        faces.append([a, b, c])
        for u, v in ((a, b), (b, c), (c, a)):
            e = (min(u, v), max(u, v))
            edges.add(e)
            edge_to_face.setdefault(e, []).append(f)

    for z in range(size):
        for y in range(size - 1):
            for x in range(size - 1):
                keys = [(x + c[0], y + c[1], z + c[2]) for c in CORNERS]
                corners = [pos[at(*k)] for k in keys]
                values = [vec[at(*k)] for k in keys]
                cube = sum(1 << i for i in range(8) if not np.any(values[i] > F(0.0)))
                verts, norms, crossing = [None] * 12, [None] * 12, []
                for i in range(12):
                    if EDGE_CROSSING_MASK[cube] & (1 << i):
                        u, v = EDGE_CONNECTION[i]
                        d = np.abs(corners[u] - corners[v])
                        axis = 0 if (d[0] > d[1] and d[0] > d[2]) else (1 if d[1] > d[2] else 2)
                        delta = F(values[v][axis] - values[u][axis])
                        t = F(0.5) if delta == F(0.0) else F(-values[u][axis] / delta)
                        verts[i] = corners[u] * F(F(1.0) - t) + corners[v] * t
                        norms[i] = _normalised_or_zero(prog.sample_normal(verts[i])[0])
                        crossing.append(i)
                key = lambda e: tuple(sorted((keys[EDGE_CONNECTION[e][0]], keys[EDGE_CONNECTION[e][1]])))
                if not crossing:
                    continue
                topo, point = oracle.emc_place([verts[i] for i in crossing], [norms[i] for i in crossing])
                if topo == 0:
                    row = TRIANGLE_CONNECTION[cube]
                    for k in range(0, 15, 3):
                        if row[k] < 0:
                            break
                        a, b, c = (add_vertex(key(e), verts[e]) for e in row[k:k + 3])
                        add_face(a, b, c)
                else:
                    centre = add_vertex(None, point)
                    features.add(centre)
                    row = EDGE_LOOPS[cube]
                    at_ = 1 + row[0]
                    for l in range(row[0]):
                        n = row[1 + l]
                        for i in range(n):
                            e0, e1 = row[at_ + i], row[at_ + (i + 1) % n]
                            a = add_vertex(key(e0), verts[e0])
                            b = add_vertex(key(e1), verts[e1])
                            add_face(a, b, centre)
                        at_ += n

    def opposite(f, e):
        return next(v for v in f if v != e[0] and v != e[1])

    flips = []
    for e in rng.permutation(sorted(edges)).tolist():
        e = tuple(e)
        if e[0] in features and e[1] in features:
            continue
        adj = edge_to_face.get(e, [])
        if len(adj) == 2 and opposite(faces[adj[0]], e) in features and opposite(faces[adj[1]], e) in features:
            flips.append(e)
    for e in flips:  # rotate_edge
        adj = edge_to_face.get(e)
        if not adj or len(adj) != 2:
            continue
        fa, fb = faces[adj[0]], faces[adj[1]]
        c, d = opposite(fa, e), opposite(fb, e)
        winding = any(fa[i] == e[0] and fa[(i + 1) % 3] == e[1] for i in range(3))
        u, v = (e[1], e[0]) if winding else (e[0], e[1])
        faces[adj[0]] = [c, d, u]
        faces[adj[1]] = [c, v, d]
        ne = (min(c, d), max(c, d))
        edges.add(ne)
        edge_to_face[ne] = [adj[0], adj[1]]
        edges.discard(e)
        del edge_to_face[e]
    return np.array(vertices, np.float32).reshape(-1, 3), np.array(faces, np.uint32).reshape(-1)


@pytest.mark.parametrize("size", [3, 9, 16])
@pytest.mark.parametrize("seed", [0, 1])
def test_independent_emc_matches_oracle(size, seed):
    from emc_scenes import FIXED
    for name in ("cube", "difference", "torus"):
        prog = oracle.Program(S.lower(FIXED[name]))
        v, i = emc(prog, size, np.random.default_rng(seed))
        m = prog.extended_marching_cubes(size)
        assert np.array_equal(v, m.vertices), name
        assert np.array_equal(i, m.indices), name


def test_independent_emc_random_csg():
    from emc_scenes import random_scenes
    rng = np.random.default_rng(7)
    features = 0
    for n, src in random_scenes(31, 12):
        prog = oracle.Program(S.lower(src))
        n = min(n, 14)
        v, i = emc(prog, n, rng)
        m = prog.extended_marching_cubes(n)
        assert np.array_equal(v, m.vertices) and np.array_equal(i, m.indices)
        features += m.features
    assert features > 0
