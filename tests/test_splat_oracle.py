"""The point-splat oracle on a case that can be checked by hand: one point
facing the light is splatted to one pixel; the gathers grow it into the
pixels whose eye rays hit its cube, all shaded with the hemisphere's second
colour (N.L = 1)."""
import numpy as np
import pytest

from isosurface_gb300 import render
from oracle import splat_ref


def test_single_point_grows_into_a_shaded_block():
    w, h = 96, 72
    vp, vpi = render.splat_camera(w, h)
    pts = np.array([[0.5, 0.5, 0.5, 0.0, -2.0, 0.0]], np.float32)  # normal (0, -1, 0) once normalised
    owner = splat_ref.splat(pts, vp, w, h)
    assert (owner == 0).sum() == 1
    py, px = np.argwhere(owner == 0)[0]
    img = splat_ref.render(pts, vp, vpi, w, h, 0.02, render.CLEAR_RGB)
    hit = img[..., 3] == 1.0
    assert 1 < hit.sum() < (2 * 16 + 1) ** 2
    ys, xs = np.nonzero(hit)
    assert np.all(np.abs(ys - py) <= 16) and np.all(np.abs(xs - px) <= 16)
    assert hit[py, px]
    assert np.all(img[hit][:, :3] == np.float32([0.518, 0.169, 0.0]))
    assert np.all(img[~hit][:, :3] == np.float32(render.CLEAR_RGB))


def test_nothing_in_view_leaves_the_clear_colour():
    w, h = 40, 30
    vp, vpi = render.splat_camera(w, h)
    pts = np.array([[-3.0, -3.0, -3.0, 1.0, 0.0, 0.0]], np.float32)  # behind the camera
    img = splat_ref.render(pts, vp, vpi, w, h, 0.01, render.CLEAR_RGB)
    assert np.all(img[..., 3] == 0.0)
    assert np.all(img[..., :3] == np.float32(render.CLEAR_RGB))


def test_mirrored_edge_addressing():
    """edge="mirror" (the example's sampler) changes only pixels whose taps
    leave the image: an interior point renders the same, and mirrored
    addressing maps texels -1, -2 to 0, 1 and W, W + 1 to W - 1, W - 2."""
    assert list(splat_ref.mirror_index(np.array([-2, -1, 0, 9, 10, 11]), 10)) == [1, 0, 0, 9, 9, 8]
    w, h = 96, 72
    vp, vpi = render.splat_camera(w, h)
    pts = np.array([[0.5, 0.5, 0.5, 0.0, -2.0, 0.0]], np.float32)
    a = splat_ref.render(pts, vp, vpi, w, h, 0.02, render.CLEAR_RGB)
    b = splat_ref.render(pts, vp, vpi, w, h, 0.02, render.CLEAR_RGB, edge="mirror")
    assert np.array_equal(a, b)
    # the demo torus: the two passes along each axis can carry a border
    # difference 2 x 16 pixels inwards, no further
    from isosurface_gb300 import scenes
    import oracle
    from isosurface_gb300 import source as S
    prog = oracle.Program(S.lower(scenes.demo_torus()))
    m = prog.point_cloud(64)
    cloud = np.concatenate([m.vertices, prog.sample_normal(m.vertices)], 1)
    w, h = 160, 120
    vp, vpi = render.splat_camera(w, h)
    a = splat_ref.render(cloud, vp, vpi, w, h, 0.5 / 64, render.CLEAR_RGB)
    b = splat_ref.render(cloud, vp, vpi, w, h, 0.5 / 64, render.CLEAR_RGB, edge="mirror")
    margin = 2 * splat_ref.TAPS
    inner = np.zeros((h, w), bool)
    inner[margin:h - margin, margin:w - margin] = True
    assert np.array_equal(a[inner], b[inner])


def _per_pixel_render(points, vp, vpi, w, h, voxel, clear, edge):
    """The example's passes pixel by pixel and tap by tap, as its shaders run
    (examples/deferred_rasterisation.rs:95-127, 131-213), with a dict for the
    depth test: an independent check of the vectorised oracle."""
    F = np.float32
    mv = splat_ref.mat_vec
    best_key = {}
    for i, q in enumerate(points.astype(F)):
        c = mv(vp, q[0], q[1], q[2], F(1.0))
        if not c[3] > 0:
            continue
        nx, ny, nz = c[0] / c[3], c[1] / c[3], c[2] / c[3]
        if not all(F(-1.0) <= v <= F(1.0) for v in (nx, ny, nz)):
            continue
        ix = min(int(np.floor((nx + F(1.0)) * (F(w) * F(0.5)))), w - 1)
        iy = min(int(np.floor((ny + F(1.0)) * (F(h) * F(0.5)))), h - 1)
        key = (F(nz * F(0.5) + F(0.5)), i)  # depth, then the earlier point
        if (iy, ix) not in best_key or key < best_key[(iy, ix)]:
            best_key[(iy, ix)] = key
    pos = np.zeros((h, w, 3), F)
    nrm = np.zeros((h, w, 3), F)
    for (iy, ix), (_, i) in best_key.items():
        q = points[i].astype(F)
        pos[iy, ix] = q[:3]
        ln = np.sqrt(F(F(q[3] * q[3] + q[4] * q[4]) + q[5] * q[5]))
        nrm[iy, ix] = q[3:6] / ln
    e = mv(vpi, F(0.0), F(0.0), F(-1.0), F(1.0))
    eye = np.array([e[0] / e[3], e[1] / e[3], e[2] / e[3]], F)
    vox = F(voxel)

    def texel(buf, y, x):
        if edge == "mirror":
            return buf[splat_ref.mirror_index(np.int64(y), h), splat_ref.mirror_index(np.int64(x), w)]
        if 0 <= y < h and 0 <= x < w:
            return buf[y, x]
        return np.zeros(3, F)

    for pas in range(4):
        dx, dy = ((1, 0), (0, 1), (1, 0), (0, 1))[pas]
        out_p = np.zeros((h, w, 3), F)
        out_n = np.zeros((h, w, 3), F)
        img = np.zeros((h, w, 4), F)
        for y in range(h):
            for x in range(w):
                ndx = F(F(2 * x + 1) / F(w)) - F(1.0)
                ndy = F(F(2 * y + 1) / F(h)) - F(1.0)
                s = mv(vpi, ndx, ndy, F(1.0), F(1.0))
                d = np.array([s[0] / s[3], s[1] / s[3], s[2] / s[3]], F) - eye
                ln = np.sqrt(F(F(d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]))
                inv = F(1.0) / (d / ln)
                best, res, rn = splat_ref.NO_HIT, np.zeros(3, F), np.zeros(3, F)
                for t in range(-16, 17):
                    p = texel(pos, y + t * dy, x + t * dx)
                    if not F(F(abs(p[0]) + abs(p[1])) + abs(p[2])) > 0:
                        continue
                    tb = inv * ((p - vox) - eye)
                    tt = inv * ((p + vox) - eye)
                    mn, mx = np.fmin(tt, tb), np.fmax(tt, tb)
                    t0 = np.fmax(np.fmax(mn[0], mn[1]), np.fmax(mn[0], mn[2]))
                    t1 = np.fmin(np.fmin(mx[0], mx[1]), np.fmin(mx[0], mx[2]))
                    if t0 <= t1 and t0 <= best:
                        best, res, rn = t0, p, texel(nrm, y + t * dy, x + t * dx)
                out_p[y, x], out_n[y, x] = res, rn
                if best < splat_ref.NO_HIT:
                    ndl = F(F(F(rn[0] * F(0.1) + rn[1] * F(-1.0)) + rn[2] * F(0.0)) * F(0.5)) + F(0.5)
                    img[y, x, :3] = [F(c1 * F(F(1.0) - ndl) + c2 * ndl) for c1, c2 in zip(splat_ref.C1, splat_ref.C2)]
                    img[y, x, 3] = 1.0
                else:
                    img[y, x, :3] = np.asarray(clear, F)
        pos, nrm = out_p, out_n
    return img


@pytest.mark.parametrize("edge", ["empty", "mirror"])
def test_oracle_matches_a_per_pixel_restatement(edge):
    from isosurface_gb300 import scenes
    import oracle
    from isosurface_gb300 import source as S
    prog = oracle.Program(S.lower(scenes.demo_torus()))
    m = prog.point_cloud(24)
    cloud = np.concatenate([m.vertices, prog.sample_normal(m.vertices)], 1)
    w, h = 28, 20
    vp, vpi = render.splat_camera(w, h)
    want = splat_ref.render(cloud, vp, vpi, w, h, 0.5 / 24, render.CLEAR_RGB, edge=edge)
    got = _per_pixel_render(cloud, vp, vpi, w, h, 0.5 / 24, render.CLEAR_RGB, edge)
    assert (want[..., 3] == 1.0).sum() > 20
    assert np.array_equal(got, want)
