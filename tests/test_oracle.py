"""CPU tests of the oracle (the checker) against the reference's own golden
vectors, and of the mesh invariants that pin its extraction stages (the
reference has no extractor tests of its own)."""
import json
import os
import re
import sys

import numpy as np
import pytest

import oracle
from isosurface_gb300 import scenes
from isosurface_gb300 import source as S

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _kats():
    return json.load(open(os.path.join(GOLDEN, "kats.json")))


def _normalised(n):
    n = np.asarray(n, np.float32)
    l = np.float32(np.sqrt(np.float32(np.float32(n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])))
    return n / l


@pytest.mark.parametrize("kat", _kats(), ids=lambda k: "%s:%d" % (os.path.basename(k["file"]), k["line"]))
def test_reference_kats(kat):
    """Every sample_scalar / sample_normal / sample_vector assertion of the
    reference's primitive tests (src/implicit/*.rs) holds for the oracle, bit
    for bit."""
    p = oracle.Program(S.lower(S.from_spec(kat["source"])))
    if kat["kind"] == "scalar":
        assert p.sample_scalar(kat["point"])[0] == np.float32(kat["expected"])
    elif kat["kind"] == "vector":
        assert p.has_vector
        assert np.array_equal(p.sample_vector(kat["point"])[0], np.asarray(kat["expected"], np.float32))
    else:
        got = _normalised(p.sample_normal(kat["point"])[0])
        assert np.array_equal(got, np.asarray(kat["expected"], np.float32))


def test_vector_fold():
    """vector.rs:686-690: len_sq folds left to right."""
    p = oracle.Program(S.lower(S.Sphere(0.0)))
    assert p.sample_scalar([1.0, 2.0, 3.0])[0] == np.float32(np.sqrt(np.float32(14.0)))


def _parse_header_ints(path, name):
    text = open(path).read()
    m = re.search(r"%s\[[^=]*=\s*\{(.*?)\};" % re.escape(name), text, re.S)
    return [int(t, 0) for t in re.findall(r"0x[0-9a-fA-F]+|-?\d+", m.group(1).replace("ull", ""))]


def test_tables_match_reference():
    """Both generated headers carry the reference's tables entry for entry."""
    t = json.load(open(os.path.join(GOLDEN, "mc_tables.json")))
    ref_h = os.path.join(ROOT, "oracle", "ref_tables.h")
    assert _parse_header_ints(ref_h, "EDGE_CROSSING_MASK") == t["EDGE_CROSSING_MASK"]
    assert _parse_header_ints(ref_h, "TRIANGLE_CONNECTION") == sum(t["TRIANGLE_CONNECTION"], [])
    assert _parse_header_ints(ref_h, "REMAP_CUBE") == t["REMAP_CUBE"]
    sys.path.insert(0, os.path.join(ROOT, "isosurface_gb300", "csrc"))
    try:
        import gen_mc_tables
    finally:
        sys.path.pop(0)
    counts, packed, order, nord, masks = gen_mc_tables.derive(t)
    dev_h = os.path.join(ROOT, "isosurface_gb300", "csrc", "mc_tables.h")
    assert _parse_header_ints(dev_h, "iso_tri_count") == counts
    assert _parse_header_ints(dev_h, "iso_tri_edges") == packed
    assert _parse_header_ints(dev_h, "iso_edge_order") == order
    assert _parse_header_ints(dev_h, "iso_edge_mask") == t["EDGE_CROSSING_MASK"]
    assert _parse_header_ints(dev_h, "iso_remap_cube") == t["REMAP_CUBE"]
    # the unpacked device triangle lists equal TRIANGLE_CONNECTION
    for case in range(256):
        row = t["TRIANGLE_CONNECTION"][case]
        n = counts[case]
        assert [(packed[case] >> (4 * k)) & 15 for k in range(3 * n)] == row[: 3 * n]


def edge_manifold_stats(tris):
    """(#undirected edges, #edges not shared by exactly two triangles, #directed duplicates)"""
    e = np.concatenate([tris[:, [0, 1]], tris[:, [1, 2]], tris[:, [2, 0]]])
    directed = e[:, 0].astype(np.int64) << 32 | e[:, 1].astype(np.int64)
    undirected = np.minimum(e[:, 0], e[:, 1]).astype(np.int64) << 32 | np.maximum(e[:, 0], e[:, 1]).astype(np.int64)
    u, c = np.unique(undirected, return_counts=True)
    return len(u), int(np.sum(c != 2)), len(directed) - len(np.unique(directed))


def test_mc_sphere_is_closed_genus0():
    """64^3 sphere: closed, consistently oriented, Euler characteristic 2."""
    p = oracle.Program(S.lower(scenes.sphere()))
    m = p.marching_cubes(65)
    tris = m.triangles
    ne, bad, dup = edge_manifold_stats(tris)
    assert bad == 0 and dup == 0
    assert len(m.vertices) - ne + len(tris) == 2
    # the reference's extra z layer: MarchingCubes::new(n) visits (n-1) x (n-1) x n cells
    assert m.cells == 64 * 64 * 65
    # every vertex lies on its lattice edge, between samples of opposite sign
    keys = m.keys[:, 0]
    axis = keys % 3
    pt = keys // 3
    x, y, z = pt % 65, (pt // 65) % 65, pt // (65 * 65)
    inv = np.float32(1.0) / np.float32(64)
    lo = np.stack([x, y, z], 1).astype(np.float32) * inv
    d = m.vertices - lo
    for a in range(3):
        on = axis == a
        assert np.all(d[on][:, a] >= -1e-6) and np.all(d[on][:, a] <= inv + 1e-6)
        for b in range(3):
            if b != a:
                assert np.all(np.abs(d[on][:, b]) < 1e-6)
    vals = p.sample_scalar(m.vertices)
    assert np.max(np.abs(vals)) < 0.5 * float(inv) * 2  # the field is a distance, |f| below a cell
    assert len(np.unique(keys)) == len(keys)


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_mc_random_unions_are_watertight(seed):
    """Seeded sphere unions strictly inside the sampled domain: the oracle's
    MarchingCubes mesh is closed and consistently oriented, every vertex is
    referenced, no triangle repeats a vertex, and each vertex lies within a
    cell of the surface."""
    from isosurface_gb300.scenes import random_spheres
    sp = random_spheres(seed, 12, 0.6, (0.08, 0.25))
    for size in (24, 41):
        p = oracle.Program(S.lower(S.unit_to_cube(S.SphereSet(sp))))
        m = p.marching_cubes(size)
        tris = m.triangles
        assert len(tris) > 0
        _, bad, dup = edge_manifold_stats(tris)
        assert bad == 0 and dup == 0
        assert np.array_equal(np.unique(tris), np.arange(len(m.vertices)))
        assert np.all((tris[:, 0] != tris[:, 1]) & (tris[:, 1] != tris[:, 2]) & (tris[:, 0] != tris[:, 2]))
        cell = 2.0 / (size - 1)  # the domain map stretches [0,1] over [-1,1]
        assert np.max(np.abs(p.sample_scalar(m.vertices))) < cell


def test_mc_cases_match_grid_signs():
    p = oracle.Program(S.lower(scenes.csg()))
    g = p.sample_grid(17)
    inside = ~(g > 0)
    corners = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    want = np.zeros((17, 16, 16), np.int32)
    for i, (dx, dy, dz) in enumerate(corners):
        want |= inside[dz:dz + 17, dy:dy + 16, dx:dx + 16].astype(np.int32) << i
    assert np.array_equal(p.mc_cases(17), want.astype(np.uint8))


def test_mc_boundary_and_degenerate_values():
    """A box whose faces fall exactly on lattice planes gives exact zeros
    (classified inside) and delta == 0 crossings."""
    src = S.unit_to_cube(S.RectangularPrism((0.5, 0.5, 0.5)))
    p = oracle.Program(S.lower(src))
    g = p.sample_grid(9)
    assert np.any(g == 0.0)
    m = p.marching_cubes(9)
    ne, bad, dup = edge_manifold_stats(m.triangles)
    assert dup == 0


def test_mc_empty_and_full():
    for src in (S.Sphere(-1.0), S.Sphere(10.0)):
        m = oracle.Program(S.lower(src)).marching_cubes(9)
        assert len(m.vertices) == 0 and len(m.indices) == 0


def test_morton_level_rule():
    """The GPU's integer Morton level (floor(log2 k)/3, one less at exact powers
    of 8) equals morton.rs:54-59's ln-based level for every key of depth <= 8."""
    assert oracle.lib().oracle_morton_level_rule_check(1 << 25) == 0
    assert [oracle.lib().oracle_morton_level(k) for k in (1, 7, 8, 9, 63, 64, 65, 512)] == [0, 0, 0, 1, 1, 1, 2, 2]


def test_morton_level_rule_up_to_depth_10():
    """Both level functions are monotone step functions that can only differ
    near powers of 8, so checking a window around each power up to 8^10 (keys
    of depth <= 10 are below 2^31) extends the exhaustive check above."""
    L = oracle.lib()
    for lv in range(9, 11):
        p = 1 << (3 * lv)
        for k in list(range(p - 4096, p + 4096)) + [2 * p - 1, 2 * p, 2 * p + 1]:
            msb = k.bit_length() - 1
            rule = msb // 3
            if rule > 0 and k == 1 << (3 * rule):
                rule -= 1
            assert L.oracle_morton_level(k) == rule, k


def test_morton_primal_dual_roundtrip():
    L = oracle.lib()
    key = (1 << 9) | 0b101_011_110  # a level-3 node
    lv = L.oracle_morton_level(key)
    for which in range(8):
        v = L.oracle_morton_primal_vertex(key, lv, which)
        if v:
            back = L.oracle_morton_dual_vertex(v, lv, which)
            assert back == key


def test_svd_matches_lstsq():
    rng = np.random.default_rng(3)
    for _ in range(50):
        a = rng.normal(size=(8, 3))
        b = rng.normal(size=8)
        d, x = oracle.svd_solve(a, b)
        s = np.linalg.svd(a, compute_uv=False)
        assert np.allclose(d, s, rtol=1e-4, atol=1e-9)  # chop() drops superdiagonals below 1e-5 relative
        if s.min() >= 0.1:
            assert np.allclose(x, np.linalg.lstsq(a, b, rcond=None)[0], rtol=1e-3, atol=1e-6)


def test_svd_truncates_small_singular_values():
    a = np.array([[1, 0, 0], [0, 1, 0], [0, 0, 0.05], [1, 1, 0]], np.float64)
    b = np.array([1.0, 2.0, 3.0, 3.0])
    d, x = oracle.svd_solve(a, b)
    assert d[2] < 0.1
    # svd.rs:61-69 zeroes singular values below 0.1, and solveSVD
    # (svd.rs:928-972) then skips the division for them without clearing the
    # projection, so a dropped direction enters x with weight u_i . b
    u, s, vt = np.linalg.svd(a, full_matrices=False)
    w = u.T @ b
    w = np.where(s >= 0.1, w / s, w)
    assert np.allclose(x, vt.T @ w, rtol=1e-4, atol=1e-6)


def test_dc_sphere_closed():
    p = oracle.Program(S.lower(scenes.sphere()))
    m = p.dual_contouring(33, placer=0)
    ne, bad, dup = edge_manifold_stats(m.triangles)
    assert bad == 0 and dup == 0
    assert len(m.vertices) - ne + len(m.triangles) == 2


def test_lhmc_runs_without_stale_corners():
    p = oracle.Program(S.lower(scenes.sphere()))
    m = p.lhmc(5)
    assert len(m.triangles) > 100
    assert m.stale_corners == 0
    vals = p.sample_scalar(m.vertices)
    assert np.max(np.abs(vals)) < 2.0 / 32


def test_mlp_oracle_gradient_by_finite_differences():
    """The numpy MLP oracle's analytic gradient agrees with central differences."""
    from oracle import mlp_ref
    rng = np.random.default_rng(0)
    n = mlp_ref.FF * 256 + 256 + 5 * (256 * 256 + 256) + 257
    p = rng.normal(0, 0.05, n)
    x = rng.uniform(-1, 1, (8, 3))
    t = rng.normal(0, 0.02, 8)
    loss, g = mlp_ref.loss_grad(p, x, t, 10.0)
    for idx in list(rng.choice(n, 12, replace=False)) + [n - 1, n - 2]:
        e = np.zeros(n)
        e[idx] = 1e-6
        lp, _ = mlp_ref.loss_grad(p + e, x, t, 10.0)
        lm, _ = mlp_ref.loss_grad(p - e, x, t, 10.0)
        assert abs((lp - lm) / 2e-6 - g[idx]) <= 1e-6 + 1e-4 * abs(g[idx])


def test_program_validation_rejects_garbage():
    good = S.lower(scenes.csg())
    oracle.Program(good)
    for bad in (good[:10], b"XXXX" + good[4:], good[:-4]):
        with pytest.raises(ValueError):
            oracle.Program(bad)
