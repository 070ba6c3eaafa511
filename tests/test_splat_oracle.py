"""The point-splat oracle on a case that can be checked by hand: one point
facing the light is splatted to one pixel; the gathers grow it into the
pixels whose eye rays hit its cube, all shaded with the hemisphere's second
colour (N.L = 1)."""
import numpy as np

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
