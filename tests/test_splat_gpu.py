"""Deferred point-splat rendering (examples/deferred_rasterisation.rs) on the
GPU against the numpy restatement of its passes: the images are identical bit
for bit (both evaluate every f32 expression in the same order)."""
import numpy as np
import pytest

from isosurface_gb300 import IsoError, render, scenes
from oracle import splat_ref

pytestmark = pytest.mark.gpu
VOXEL = 0.5 / 64  # the example's voxel_size for PointCloud::new(64)


def _point_cloud(ctx):
    info = ctx.point_cloud_extract(scenes.demo_torus(), 64, normals=True)
    pts = ctx.download(info).vertices
    assert pts.shape == (info.num_vertices, 6) and len(pts) > 1000
    return pts


@pytest.mark.parametrize("width,height", [(256, 192), (333, 250)])
def test_point_splat_matches_oracle(ctx, width, height):
    pts = _point_cloud(ctx)
    img = ctx.point_splat(width, height, VOXEL)
    vp, vpi = render.splat_camera(width, height)
    want = splat_ref.render(pts, vp, vpi, width, height, VOXEL, render.CLEAR_RGB)
    assert img.shape == (height, width, 4)
    assert np.array_equal(img, want)
    hit = img[..., 3] == 1.0
    assert 0.05 < hit.mean() < 0.6
    assert np.all(img[~hit][:, :3] == np.float32(render.CLEAR_RGB))


def test_point_splat_needs_a_point_cloud_with_normals(ctx):
    ctx.mc_extract(scenes.sphere(), 17)
    with pytest.raises(IsoError):
        ctx.point_splat(64, 48, VOXEL)
    ctx.point_cloud_extract(scenes.demo_torus(), 32)  # no normals
    with pytest.raises(IsoError):
        ctx.point_splat(64, 48, VOXEL)


@pytest.mark.parametrize("width,height", [(96, 72), (256, 192)])
def test_point_splat_mirrored_edges_match_oracle(ctx, width, height):
    pts = _point_cloud(ctx)
    img = ctx.point_splat(width, height, VOXEL, edge="mirror")
    vp, vpi = render.splat_camera(width, height)
    want = splat_ref.render(pts, vp, vpi, width, height, VOXEL, render.CLEAR_RGB, edge="mirror")
    assert np.array_equal(img, want)
