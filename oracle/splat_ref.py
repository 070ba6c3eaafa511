"""Test infrastructure: a float32 numpy restatement of the deferred point-splat
renderer of examples/deferred_rasterisation.rs (its GLSL passes), in the
operation order the CUDA kernels use, so that the two agree bit for bit.  The
library never imports this module.

Passes (examples/deferred_rasterisation.rs:95-127, 131-213, 342-421):
  1. every point of a PointCloud with interleaved normals is splatted to the
     pixel its clip position falls in, depth-tested (GL_LESS: the nearest,
     then the earliest point wins), into position (xyz, 1) and normalised
     normal buffers;
  2. three ping-pong gathers along x, y, x: each pixel casts its eye ray
     (from the near-plane centre to its far-plane point) against the cube of
     half-size `voxel` around the points stored 16 pixels either side and
     keeps the nearest hit (ties: the later tap);
  3. a last gather along y that shades a hit with the hemisphere term and
     composites over the clear colour (alpha 1 for a hit, 0 otherwise).
Row 0 of every buffer is the bottom row.  Taps past the image edge read as
empty (edge="empty", what the CUDA kernels do), or through mirrored-repeat
addressing (edge="mirror": texel -1 reads texel 0, texel W reads W - 1, ...),
the wrap of glium 0.26's default sampler through which the example reads its
buffers.
"""
import numpy as np

F = np.float32
TAPS = 16
NO_HIT = F(9999999.0)
# hemisphere colours: C1 where N.L = -1, C2 where N.L = 1
C1 = (F(0.886), F(0.757), F(0.337))
C2 = (F(0.518), F(0.169), F(0.0))
LIGHT = (F(0.1), F(-1.0), F(0.0))


def mat_vec(m, x, y, z, w):
    """Column-major m times (x, y, z, w): row r = ((m0r*x + m1r*y) + m2r*z) + m3r*w."""
    return [((m[r] * x + m[4 + r] * y) + m[8 + r] * z) + m[12 + r] * w for r in range(4)]


def splat(points, mvp, width, height):
    """Per pixel the index of the winning point (-1: none).  points: (n, 6)."""
    p = points.astype(F)
    one = F(1.0)
    cx, cy, cz, cw = mat_vec(mvp, p[:, 0], p[:, 1], p[:, 2], one)
    with np.errstate(divide="ignore", invalid="ignore"):
        nx, ny, nz = cx / cw, cy / cw, cz / cw
    keep = (cw > 0) & (nx >= -1) & (nx <= 1) & (ny >= -1) & (ny <= 1) & (nz >= -1) & (nz <= 1)
    hw, hh = F(width) * F(0.5), F(height) * F(0.5)
    xw, yw = (nx + one) * hw, (ny + one) * hh
    ix = np.minimum(np.floor(xw), F(width - 1)).astype(np.int64)
    iy = np.minimum(np.floor(yw), F(height - 1)).astype(np.int64)
    depth = nz * F(0.5) + F(0.5)
    owner = np.full(width * height, -1, np.int64)
    idx = np.nonzero(keep)[0]
    if len(idx):
        pix = iy[idx] * width + ix[idx]
        key = (depth[idx].view(np.uint32).astype(np.uint64) << np.uint64(32)) | idx.astype(np.uint64)
        order = np.lexsort((key, pix))
        pix, key = pix[order], key[order]
        first = np.ones(len(pix), bool)
        first[1:] = pix[1:] != pix[:-1]
        owner[pix[first]] = (key[first] & np.uint64(0xFFFFFFFF)).astype(np.int64)
    return owner.reshape(height, width)


def gbuffer(points, owner):
    """(position (h, w, 4), normal (h, w, 4)) buffers from the winning points."""
    h, w = owner.shape
    pos = np.zeros((h, w, 4), F)
    nrm = np.zeros((h, w, 4), F)
    hit = owner >= 0
    q = points[owner[hit]].astype(F)
    pos[hit, 0:3] = q[:, 0:3]
    pos[hit, 3] = F(1.0)
    n = q[:, 3:6]
    with np.errstate(divide="ignore", invalid="ignore"):
        ln = np.sqrt((n[:, 0] * n[:, 0] + n[:, 1] * n[:, 1]) + n[:, 2] * n[:, 2])
        nrm[hit, 0:3] = n / ln[:, None]
    return pos, nrm


def eye_rays(vpinv, width, height):
    """Per pixel the ray origin (the near-plane centre) and unit direction."""
    e = mat_vec(vpinv, F(0.0), F(0.0), F(-1.0), F(1.0))
    eye = [e[0] / e[3], e[1] / e[3], e[2] / e[3]]
    ix = np.arange(width, dtype=np.int64)[None, :]
    iy = np.arange(height, dtype=np.int64)[:, None]
    ndx = (2 * ix + 1).astype(F) / F(width) - F(1.0)
    ndy = (2 * iy + 1).astype(F) / F(height) - F(1.0)
    ndx, ndy = np.broadcast_arrays(ndx, ndy)
    s = mat_vec(vpinv, ndx, ndy, F(1.0), F(1.0))
    scr = [s[0] / s[3], s[1] / s[3], s[2] / s[3]]
    d = [scr[k] - eye[k] for k in range(3)]
    ln = np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])
    return eye, [dk / ln for dk in d]


def mirror_index(i, n):
    """Mirrored-repeat addressing of texel i in a row of n texels."""
    m = np.mod(i, 2 * n)
    return np.where(m >= n, 2 * n - 1 - m, m)


def gather(pos, nrm, eye, dirs, voxel, dx, dy, last, clear, edge="empty"):
    h, w = pos.shape[:2]
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = [F(1.0) / d for d in dirs]
    best = np.full((h, w), NO_HIT, F)
    res = np.zeros((h, w, 3), F)
    rn = np.zeros((h, w, 3), F)
    vox = F(voxel)
    for t in range(-TAPS, TAPS + 1):
        if edge == "mirror":
            ys = mirror_index(np.arange(h) + t * dy, h)
            xs = mirror_index(np.arange(w) + t * dx, w)
            p = pos[ys][:, xs, 0:3]
            n = nrm[ys][:, xs, 0:3]
        else:
            p = np.zeros((h, w, 3), F)
            n = np.zeros((h, w, 3), F)
            sy0, sy1 = max(0, t * dy), min(h, h + t * dy)
            sx0, sx1 = max(0, t * dx), min(w, w + t * dx)
            p[sy0 - t * dy:sy1 - t * dy, sx0 - t * dx:sx1 - t * dx] = pos[sy0:sy1, sx0:sx1, 0:3]
            n[sy0 - t * dy:sy1 - t * dy, sx0 - t * dx:sx1 - t * dx] = nrm[sy0:sy1, sx0:sx1, 0:3]
        full = (np.abs(p[..., 0]) + np.abs(p[..., 1])) + np.abs(p[..., 2]) > F(0.0)
        with np.errstate(invalid="ignore"):
            tmin, tmax = [], []
            for k in range(3):
                tb = inv[k] * ((p[..., k] - vox) - eye[k])
                tt = inv[k] * ((p[..., k] + vox) - eye[k])
                tmin.append(np.fmin(tt, tb))
                tmax.append(np.fmax(tt, tb))
            t0 = np.fmax(np.fmax(tmin[0], tmin[1]), np.fmax(tmin[0], tmin[2]))
            t1 = np.fmin(np.fmin(tmax[0], tmax[1]), np.fmin(tmax[0], tmax[2]))
            take = full & (t0 <= t1) & (t0 <= best)
        best = np.where(take, t0, best)
        res = np.where(take[..., None], p, res)
        rn = np.where(take[..., None], n, rn)
    if not last:
        op = np.zeros((h, w, 4), F)
        on = np.zeros((h, w, 4), F)
        op[..., 0:3] = res
        on[..., 0:3] = rn
        return op, on
    hit = best < NO_HIT
    ndl = ((rn[..., 0] * LIGHT[0] + rn[..., 1] * LIGHT[1]) + rn[..., 2] * LIGHT[2]) * F(0.5) + F(0.5)
    out = np.zeros((h, w, 4), F)
    for k in range(3):
        shade = C1[k] * (F(1.0) - ndl) + C2[k] * ndl
        out[..., k] = np.where(hit, shade, F(clear[k]))
    out[..., 3] = np.where(hit, F(1.0), F(0.0))
    return out


def render(points, mvp, vpinv, width, height, voxel, clear, edge="empty"):
    """The composited image, (height, width, 4) float32, row 0 at the bottom."""
    mvp = np.asarray(mvp, F)
    vpinv = np.asarray(vpinv, F)
    owner = splat(points, mvp, width, height)
    pos, nrm = gbuffer(points, owner)
    eye, dirs = eye_rays(vpinv, width, height)
    for i in range(3):
        pos, nrm = gather(pos, nrm, eye, dirs, voxel, (i + 1) % 2, i % 2, False, clear, edge)
    return gather(pos, nrm, eye, dirs, voxel, 0, 1, True, clear, edge)
