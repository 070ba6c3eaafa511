"""Surrogate marching cubes (csrc/surrogate.cu): the hybrid field is the
network's trilinear interpolation outside the band and the exact field, bit
for bit, inside it; the metrics against brute-force numpy; and the ablation
that shows what the network buys (exact evaluations saved) and what the band
re-sampling buys back (accuracy)."""
import numpy as np
import pytest

from isosurface_gb300 import scenes
from isosurface_gb300.surrogate import Surrogate, case_disagreement, mesh_distance

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _device_field(size):
    pitch = size
    t = torch.full(((size + 1) * size * pitch,), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    return t, pitch


def _coarse_points(size, step):
    """World points of the coarse grid: lattice (i*step) / (size-1) through the
    [0,1] -> [-1,1] domain map, in f32 as the kernels compute them."""
    inv = np.float32(1.0) / np.float32(size - 1)
    dims = [(size - 1 + step - 1) // step + 1, (size - 1 + step - 1) // step + 1, (size + step - 1) // step + 1]
    ax = [(np.arange(d, dtype=np.float32) * np.float32(step)) * inv * np.float32(2.0) + np.float32(-1.0)
          for d in dims]
    z, y, x = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return dims, np.stack([x.ravel(), y.ravel(), z.ravel()], 1)


def _interp(coarse, dims, size, step):
    """Trilinear interpolation of the coarse grid at every fine point, in the
    kernel's f32 operation order."""
    cx, cy, cz = dims
    c = coarse.reshape(cz, cy, cx)
    f = np.float32

    def idx(n):
        i = np.arange(n)
        lo = i // step
        t = ((i - lo * step).astype(np.float32) * f(1.0 / step)).astype(np.float32)
        return lo, t

    ix, tx = idx(size)
    iy, ty = idx(size)
    iz, tz = idx(size + 1)
    jx, jy, jz = np.minimum(ix + 1, cx - 1), np.minimum(iy + 1, cy - 1), np.minimum(iz + 1, cz - 1)

    def lerp(a, b, t):
        return (a + (b - a) * t).astype(np.float32)

    Z, Y, X = np.meshgrid(np.arange(size + 1), np.arange(size), np.arange(size), indexing="ij")
    g = lambda xx, yy, zz: c[zz, yy, xx]
    v00 = lerp(g(ix[X], iy[Y], iz[Z]), g(jx[X], iy[Y], iz[Z]), tx[X])
    v10 = lerp(g(ix[X], jy[Y], iz[Z]), g(jx[X], jy[Y], iz[Z]), tx[X])
    v01 = lerp(g(ix[X], iy[Y], jz[Z]), g(jx[X], iy[Y], jz[Z]), tx[X])
    v11 = lerp(g(ix[X], jy[Y], jz[Z]), g(jx[X], jy[Y], jz[Z]), tx[X])
    return lerp(lerp(v00, v10, ty[Y]), lerp(v01, v11, ty[Y]), tz[Z])


def test_full_band_is_the_exact_mesh(ctx):
    size = 41
    src = scenes.smooth_spheres(count=64)
    net = Surrogate(ctx, seed=1)
    info, st = net.extract(src, size, coarse_step=4, band_cells=1e5)
    assert st["band_points"] == st["total_points"] == size * size * (size + 1)
    got = ctx.download(info)
    want = ctx.download(ctx.mc_extract(src, size))
    assert np.array_equal(got.vertices, want.vertices)
    assert np.array_equal(got.indices, want.indices)
    net.close()


@pytest.mark.parametrize("size,step,band", [(33, 4, 2.0), (41, 3, 1.5), (29, 1, 2.0)])
def test_field_composition(ctx, size, step, band):
    src = scenes.smooth_spheres(count=64)
    net = Surrogate(ctx, seed=2)
    # scale the output so the untrained network crosses zero inside the box
    p = net.params
    p[-257:-1] *= 4.0
    net.params = p
    field, pitch = _device_field(size)
    st = net.field(src, size, field.data_ptr(), pitch, coarse_step=step, band_cells=band)
    got = field.cpu().numpy().reshape(size + 1, size, pitch)
    exact_t, _ = _device_field(size)
    ctx.sample_grid(src, size, exact_t.data_ptr(), pitch)
    exact = exact_t.cpu().numpy().reshape(size + 1, size, pitch)

    dims, pts = _coarse_points(size, step)
    coarse = net.forward(pts, bf16=True)
    interp = _interp(coarse, dims, size, step)
    tau = np.float32(band) * (np.float32(1.0) / np.float32(size - 1)) * np.float32(2.0)
    sure_band = np.abs(interp) <= tau * 0.999 - 1e-5
    sure_out = np.abs(interp) > tau * 1.001 + 1e-5
    assert sure_band.any() and sure_out.any()
    # inside the band: the exact field, bit for bit
    assert np.array_equal(got[sure_band].view(np.uint32), exact[sure_band].view(np.uint32))
    # outside: the network's coarse values interpolated (same f32 operations)
    assert np.max(np.abs(got[sure_out] - interp[sure_out])) <= 1e-6
    n_band = int(st["band_points"])
    assert sure_band.sum() <= n_band <= size * size * (size + 1) - sure_out.sum()
    assert st["coarse_points"] == dims[0] * dims[1] * dims[2]
    net.close()


def _nn_brute(a, b):
    d = np.sqrt(((a[:, None, :].astype(np.float64) - b[None, :, :]) ** 2).sum(-1))
    return d.min(1)


@pytest.mark.parametrize("bucket", [0.01, 0.05, 0.3])
def test_mesh_distance_matches_brute_force(ctx, bucket):
    rng = np.random.default_rng(7)
    a = rng.uniform(0, 1, (1500, 3)).astype(np.float32)
    b = rng.uniform(0, 1, (2100, 3)).astype(np.float32)
    r = mesh_distance(ctx, a, b, bucket, max_rings=1024)
    dab, dba = _nn_brute(a, b), _nn_brute(b, a)
    assert r["capped"] == 0
    assert abs(r["mean_ab"] - dab.mean()) <= 1e-6 and abs(r["mean_ba"] - dba.mean()) <= 1e-6
    assert abs(r["max_ab"] - dab.max()) <= 1e-6 and abs(r["max_ba"] - dba.max()) <= 1e-6
    assert abs(r["chamfer"] - 0.5 * (dab.mean() + dba.mean())) <= 1e-6


def test_mesh_distance_identical_and_capped(ctx):
    rng = np.random.default_rng(8)
    a = rng.uniform(0, 1, (5000, 3)).astype(np.float32)
    r = mesh_distance(ctx, a, a.copy(), 0.02)
    assert r["chamfer"] == 0.0 and r["hausdorff"] == 0.0 and r["capped"] == 0
    # one far outlier: found only beyond max_rings buckets
    b = np.concatenate([a, [[5.0, 5.0, 5.0]]]).astype(np.float32)
    r = mesh_distance(ctx, b, a, 0.02, max_rings=4)
    assert r["capped"] == 1
    assert r["max_ab"] >= 4 * 0.02 * 0.999


def test_case_disagreement_matches_numpy(ctx):
    size = 37
    rng = np.random.default_rng(3)
    fa = rng.normal(0, 1, (size + 1, size, size)).astype(np.float32)
    fb = fa.copy()
    flip = rng.random(fa.shape) < 0.01
    fb[flip] = -fb[flip]
    fb[0, 0, 0] = 0.0  # !(0 > 0): inside, like a negative value
    fa[0, 0, 0] = -1.0
    sa, sb = ~(fa > 0), ~(fb > 0)
    d = sa != sb
    cells = np.zeros((size, size - 1, size - 1), bool)
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                cells |= d[dz:dz + size, dy:dy + size - 1, dx:dx + size - 1]
    ta = torch.from_numpy(fa.ravel()).cuda()
    tb = torch.from_numpy(fb.ravel()).cuda()
    torch.cuda.synchronize()
    got = case_disagreement(ctx, ta.data_ptr(), tb.data_ptr(), size, size, size + 1, size)
    assert got == int(cells.sum())


def test_ablation_band_resampling(ctx):
    """A briefly trained network on a 1024-sphere smooth union at 129^3: the
    band saves most exact evaluations, and re-sampling the band makes the
    mesh closer to the exact mesh than the network alone."""
    size = 129
    src = scenes.smooth_spheres(count=1024)
    net = Surrogate(ctx, seed=3)
    net.make_dataset(src.source, 1 << 21, -1.0, 1.0, seed=4)
    net.train(800, batch=16384, lr=2e-3)
    cell = 1.0 / (size - 1)
    exact = ctx.download(ctx.mc_extract(src, size))
    res = {}
    for band in (0.0, 2.0):
        info, st = net.extract(src, size, coarse_step=2, band_cells=band)
        m = ctx.download(info)
        assert len(m.vertices) > 0, "band %g: empty mesh" % band
        d = mesh_distance(ctx, m.vertices, exact.vertices, 2 * cell, max_rings=64)
        res[band] = (st, d)
    st0, d0 = res[0.0]
    st2, d2 = res[2.0]
    assert st0["band_points"] == 0
    assert st2["band_points"] < 0.5 * st2["total_points"]
    assert d2["chamfer"] < d0["chamfer"]
    net.close()


def test_exact_coarse_field_composition(ctx):
    """ISO_SURROGATE_EXACT_COARSE: the same pipeline with the network replaced
    by the exact source on the coarse grid -- exact inside the band, the
    interpolated exact coarse values outside it."""
    size, step, band = 33, 4, 1.5
    src = scenes.smooth_spheres(count=64)
    field, pitch = _device_field(size)
    net = Surrogate(ctx, seed=2)
    st = net.field_ex(src, size, field.data_ptr(), pitch, coarse_step=step, band_cells=band, exact_coarse=True)
    got = field.cpu().numpy().reshape(size + 1, size, pitch)
    exact_t, _ = _device_field(size)
    ctx.sample_grid(src, size, exact_t.data_ptr(), pitch)
    exact = exact_t.cpu().numpy().reshape(size + 1, size, pitch)
    dims, _ = _coarse_points(size, step)
    # coarse point (i, j, k) is lattice point (i, j, k) * step (the last ones
    # may lie beyond the grid): the exact source there, in the sample frame
    inv = np.float32(1.0) / np.float32(size - 1)
    ax = [np.arange(d, dtype=np.float32) * np.float32(step) * inv for d in dims]
    zz, yy, xx = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    coarse = ctx.sample_points(src, np.stack([xx.ravel(), yy.ravel(), zz.ravel()], 1))
    interp = _interp(coarse, dims, size, step)
    tau = np.float32(band) * (np.float32(1.0) / np.float32(size - 1)) * np.float32(2.0)
    sure_band = np.abs(interp) <= tau * 0.999 - 1e-5
    sure_out = np.abs(interp) > tau * 1.001 + 1e-5
    assert sure_band.any() and sure_out.any()
    assert np.array_equal(got[sure_band].view(np.uint32), exact[sure_band].view(np.uint32))
    assert np.max(np.abs(got[sure_out] - interp[sure_out])) <= 1e-6
    assert st["flagged"] == 0
    net.close()


def test_witness_checks_force_missed_spheres_into_the_band(ctx):
    """ISO_SURROGATE_WITNESS with a network that says "outside" everywhere
    (zero weights, output bias 1): without the checks the band is empty and
    so is the mesh; with them every sphere is flagged at its centre, its ball
    and shell are re-sampled exactly, and the mesh is the exact mesh.  A
    source that is not a sphere set is refused."""
    from isosurface_gb300 import IsoError
    size = 65
    src = scenes.smooth_spheres(count=64)
    net = Surrogate(ctx, seed=5)
    p = np.zeros(net.nparams, np.float32)
    p[-1] = 1.0
    net.params = p
    cell = 1.0 / (size - 1)
    exact = ctx.download(ctx.mc_extract(src, size))
    out = {}
    for witness in (False, True):
        field, pitch = _device_field(size)
        st = net.field_ex(src, size, field.data_ptr(), pitch, coarse_step=4, band_cells=2.0, witness=witness)
        m = ctx.download(ctx.mc_extract_field(field.data_ptr(), size, size, size + 1, pitch))
        d = mesh_distance(ctx, m.vertices, exact.vertices, 2 * cell, max_rings=64) if len(m.vertices) else None
        out[witness] = (st, m, d)
    st0, m0, d0 = out[False]
    st1, m1, d1 = out[True]
    assert st0["flagged"] == 0 and st0["band_points"] == 0 and len(m0.vertices) == 0
    assert st1["flagged"] == 64
    assert st1["band_points"] < st1["total_points"]
    # every sphere the untrained network misses is re-sampled: the exact mesh
    assert np.array_equal(m1.vertices, exact.vertices) and np.array_equal(m1.indices, exact.indices)
    with pytest.raises(IsoError):
        field, pitch = _device_field(size)
        net.field_ex(scenes.csg(), size, field.data_ptr(), pitch, witness=True)
    net.close()


def test_what_the_network_gains(ctx):
    """The comparison the surrogate exists for: network + band re-sampling
    against the same pipeline with the network replaced by exact samples of
    the coarse grid, at the same band.  With the network the exact source is
    evaluated only in the band (the coarse grid costs no exact evaluation);
    without it every coarse point is an exact evaluation too.  Both meshes
    are scored against the exact mesh."""
    size, step, band = 129, 2, 2.0
    src = scenes.smooth_spheres(count=1024)
    net = Surrogate(ctx, seed=3)
    net.make_dataset(src.source, 1 << 21, -1.0, 1.0, seed=4)
    net.train(800, batch=16384, lr=2e-3)
    cell = 1.0 / (size - 1)
    exact = ctx.download(ctx.mc_extract(src, size))
    res = {}
    for exact_coarse in (False, True):
        field, pitch = _device_field(size)
        st = net.field_ex(src, size, field.data_ptr(), pitch, coarse_step=step, band_cells=band,
                          exact_coarse=exact_coarse, witness=True)
        m = ctx.download(ctx.mc_extract_field(field.data_ptr(), size, size, size + 1, pitch))
        d = mesh_distance(ctx, m.vertices, exact.vertices, 2 * cell, max_rings=64)
        exact_evals = st["band_points"] + (st["coarse_points"] if exact_coarse else 0)
        res[exact_coarse] = (st, d, exact_evals)
    (stn, dn, en), (ste, de, ee) = res[False], res[True]
    assert en < ee                          # the network saves the coarse grid's exact evaluations
    assert stn["coarse_points"] == ste["coarse_points"]
    assert dn["chamfer"] <= 0.05 * cell     # both close to the exact mesh
    assert de["chamfer"] <= 0.05 * cell
    net.close()
