"""An independent float32 restatement of every source op's value and normal, written
from the program format's definitions in include/isosurface_gpu.h and the
reference's primitives (src/implicit/{sphere,rectangular_prism,cylinder,
torus,csg}.rs, src/math/vector.rs folds), checked bit for bit against the
oracle's evaluator at seeded random points (the reference's own known-answer
tests pin the primitives at a few points only; SmoothUnion, Rigid, DomainMap
and SphereSet have no reference counterpart and are checked against their
stated formulas here)."""
import numpy as np
import pytest

import oracle
from isosurface_gb300 import source as S

F = np.float32


def length(x, y, z):  # vector.rs: len_sq folds (x*x + y*y) + z*z
    return np.sqrt(F(F(x * x + y * y) + z * z))


def value(src, p):
    x, y, z = (F(c) for c in p)
    if isinstance(src, S.Sphere):
        return F(length(x, y, z) - F(src.radius))
    if isinstance(src, S.RectangularPrism):
        h = [F(v) for v in src.half_extent]
        q = [F(abs(x) - h[0]), F(abs(y) - h[1]), F(abs(z) - h[2])]
        outside = length(*(np.fmax(c, F(0.0)) for c in q))
        return F(outside + np.fmin(np.fmax(q[0], np.fmax(q[1], q[2])), F(0.0)))
    if isinstance(src, S.Cylinder):
        qx = F(abs(np.sqrt(F(x * x + y * y))) - F(src.radius))
        qz = F(abs(z) - F(src.half_length))
        return F(np.fmin(np.fmax(qx, qz), F(0.0)) + length(np.fmax(qx, F(0.0)), np.fmax(qz, F(0.0)), F(0.0)))
    if isinstance(src, S.Torus):
        qx = F(abs(np.sqrt(F(x * x + y * y))) - F(src.radius))
        return F(np.sqrt(F(qx * qx + z * z)) - F(src.tube_radius))
    if isinstance(src, S.Union):
        return np.fmin(value(src.a, p), value(src.b, p))
    if isinstance(src, S.Intersection):
        return np.fmax(value(src.a, p), value(src.b, p))
    if isinstance(src, S.Difference):  # b minus a
        return np.fmax(value(src.b, p), -value(src.a, p))
    if isinstance(src, S.SmoothUnion):
        a, b, k = value(src.a, p), value(src.b, p), F(src.k)
        h = F(np.fmax(F(k - abs(F(a - b))), F(0.0)) / k)
        return F(np.fmin(a, b) - F(F(F(h * h) * k) * F(0.25)))
    if isinstance(src, S.Translate):
        c = [F(v) for v in src.centre]
        return value(src.source, (F(x - c[0]), F(y - c[1]), F(z - c[2])))
    if isinstance(src, S.Rigid):
        t = [F(v) for v in src.t]
        m = [F(v) for v in src.m]
        d = (F(x - t[0]), F(y - t[1]), F(z - t[2]))
        q = tuple(F(F(m[3 * r] * d[0] + m[3 * r + 1] * d[1]) + m[3 * r + 2] * d[2]) for r in range(3))
        return value(src.source, q)
    if isinstance(src, S.DomainMap):
        sc, of = [F(v) for v in src.scale], [F(v) for v in src.offset]
        return value(src.source, (F(x * sc[0] + of[0]), F(y * sc[1] + of[1]), F(z * sc[2] + of[2])))
    if isinstance(src, S.CentralDifference):
        return value(src.source, p)
    if isinstance(src, S.SphereSet):
        v = None
        for cx, cy, cz, r in src.spheres:
            d = F(length(F(x - cx), F(y - cy), F(z - cz)) - r)
            if v is None:
                v = d
            elif src.smooth_k is None:
                v = np.fmin(v, d)
            else:
                v = value(S.SmoothUnion(_Const(v), _Const(d), src.smooth_k), p)
        return v
    if isinstance(src, _Const):
        return src.v
    raise TypeError(type(src))


class _Const:
    def __init__(self, v):
        self.v = v


def _scenes():
    rng = np.random.default_rng(21)
    rot = np.linalg.qr(rng.normal(size=(3, 3)))[0].astype(np.float32)
    spheres = np.concatenate([rng.uniform(-0.6, 0.6, (12, 3)), rng.uniform(0.05, 0.3, (12, 1))], 1).astype(F)
    return {
        "sphere": S.Sphere(0.7),
        "box": S.RectangularPrism((0.5, 0.3, 0.7)),
        "cylinder": S.Cylinder(0.4, 0.6),
        "torus": S.Torus(0.5, 0.15),
        "csg": S.Difference(S.Sphere(0.7), S.Union(S.RectangularPrism((0.6, 0.6, 0.6)), S.Torus(0.5, 0.15))),
        "intersection": S.Intersection(S.Sphere(0.8), S.Cylinder(0.5, 0.7)),
        "smooth": S.SmoothUnion(S.Translate(S.Sphere(0.3), (0.2, 0.0, 0.0)), S.Translate(S.Sphere(0.3), (-0.2, 0.1, 0.0)),
                                0.05),
        "rigid": S.Rigid(S.RectangularPrism((0.6, 0.2, 0.4)), (0.05, -0.03, 0.02), rot),
        "domain": S.unit_to_cube(S.Torus(0.5, 0.2)),
        "central_difference": S.CentralDifference(S.Translate(S.Torus(0.25, 0.1), (0.5, 0.5, 0.5))),
        "sphere_set_hard": S.SphereSet(spheres),
        "sphere_set_smooth": S.SphereSet(spheres, smooth_k=0.05),
    }


SCENES = _scenes()


@pytest.mark.parametrize("name", sorted(SCENES))
def test_source_values_match_oracle(name):
    src = SCENES[name]
    pts = np.random.default_rng(4).uniform(-1.1, 1.1, (400, 3)).astype(F)
    pts[:20] = 0.0  # axis planes and the origin
    pts[20:40, 1:] = 0.0
    got = np.array([value(src, p) for p in pts], F)
    want = oracle.Program(S.lower(src)).sample_scalar(pts)
    assert np.array_equal(got, want), np.nonzero(got != want)[0][:5]


def _v(x, y, z):
    return np.array([x, y, z], F)


def normal(src, p):
    """HermiteSource::sample_normal (unnormalised): the primitives as in the
    reference (sphere.rs, rectangular_prism.rs via Vec3::clamp_to_cardinal_axis,
    cylinder.rs, torus.rs), Union's component-wise min (csg.rs:47-51), and the
    header's definitions where the reference has none: Intersection,
    Difference and SmoothUnion take the deciding operand's normal, Rigid
    rotates it back by M^T, the other point ops pass it through,
    CentralDifference differentiates the value (source.rs:82-95)."""
    x, y, z = (F(c) for c in p)
    if isinstance(src, S.Sphere):
        return _v(x, y, z)
    if isinstance(src, S.RectangularPrism):  # vector.rs:612-621
        ax, ay, az = abs(x), abs(y), abs(z)
        if ax > ay and ax > az:
            return _v(x, 0.0, 0.0)
        return _v(0.0, y, 0.0) if ay > az else _v(0.0, 0.0, z)
    if isinstance(src, S.Cylinder):
        zz = F(abs(z) / F(src.half_length))
        r = F(np.sqrt(F(x * x + y * y)) / F(src.radius))
        return _v(0.0, 0.0, z) if zz > r else _v(x, y, 0.0)
    if isinstance(src, S.Torus):
        ln = length(x, y, F(0.0))
        ring = _v(1.0, 0.0, 0.0) if abs(ln) < F(1.1920929e-07) else _v(x / ln, y / ln, F(0.0) / ln)
        return _v(x, y, z) - ring * F(src.radius)
    if isinstance(src, S.Union):
        return np.fmin(normal(src.a, p), normal(src.b, p))
    if isinstance(src, S.Intersection):
        return normal(src.a, p) if value(src.a, p) >= value(src.b, p) else normal(src.b, p)
    if isinstance(src, S.Difference):
        return normal(src.b, p) if value(src.b, p) >= -value(src.a, p) else -normal(src.a, p)
    if isinstance(src, S.SmoothUnion):
        return normal(src.a, p) if value(src.a, p) <= value(src.b, p) else normal(src.b, p)
    if isinstance(src, S.Translate):
        c = [F(v) for v in src.centre]
        return normal(src.source, (F(x - c[0]), F(y - c[1]), F(z - c[2])))
    if isinstance(src, S.Rigid):
        t = [F(v) for v in src.t]
        m = [F(v) for v in src.m]
        d = (F(x - t[0]), F(y - t[1]), F(z - t[2]))
        q = tuple(F(F(m[3 * r] * d[0] + m[3 * r + 1] * d[1]) + m[3 * r + 2] * d[2]) for r in range(3))
        n = normal(src.source, q)
        return np.array([F(F(m[c] * n[0] + m[3 + c] * n[1]) + m[6 + c] * n[2]) for c in range(3)], F)
    if isinstance(src, S.DomainMap):
        sc, of = [F(v) for v in src.scale], [F(v) for v in src.offset]
        return normal(src.source, (F(x * sc[0] + of[0]), F(y * sc[1] + of[1]), F(z * sc[2] + of[2])))
    if isinstance(src, S.CentralDifference):
        e = F(src.epsilon)
        f = lambda q: value(src.source, q)
        vx = F(f((F(x + e), F(y + F(0.0)), F(z + F(0.0)))) - f((F(x - e), F(y - F(0.0)), F(z - F(0.0)))))
        vy = F(f((F(x + F(0.0)), F(y + e), F(z + F(0.0)))) - f((F(x - F(0.0)), F(y - e), F(z - F(0.0)))))
        vz = F(f((F(x + F(0.0)), F(y + F(0.0)), F(z + e))) - f((F(x - F(0.0)), F(y - F(0.0)), F(z - e))))
        e2 = F(F(2.0) * e)
        return _v(vx / e2, vy / e2, vz / e2)
    raise TypeError(type(src))


@pytest.mark.parametrize("name", sorted(n for n in SCENES if not n.startswith("sphere_set")))
def test_source_normals_match_oracle(name):
    src = SCENES[name]
    pts = np.random.default_rng(8).uniform(-1.1, 1.1, (300, 3)).astype(F)
    pts[:10] = 0.0
    got = np.array([normal(src, p) for p in pts], F)
    want = oracle.Program(S.lower(src)).sample_normal(pts)
    assert np.array_equal(got, want), np.nonzero(np.any(got != want, axis=1))[0][:5]


MAXF = F(3.40282347e38)


def vector(src, p):
    """VectorSource::sample_vector (the Directed metric of
    ExtendedMarchingCubes): sphere.rs:41-57, rectangular_prism.rs:43-70,
    cylinder.rs:50-71, torus.rs:48-100, csg.rs:41-45, 74-78, 102-106; a
    translated source samples at p - centre, CentralDifference passes through."""
    x, y, z = (F(c) for c in p)
    a = np.array([abs(x), abs(y), abs(z)], F)
    if isinstance(src, S.Sphere):
        r2 = F(F(src.radius) * F(src.radius))
        l_yz, l_xz, l_xy = (F(r2 - F(F(a[i] * a[i]) + F(a[j] * a[j]))) for i, j in ((1, 2), (0, 2), (0, 1)))
        return np.array([MAXF if l < 0 else F(a[k] - np.sqrt(l)) for k, l in enumerate((l_yz, l_xz, l_xy))], F)
    if isinstance(src, S.RectangularPrism):
        h = np.array(src.half_extent, F)
        outside = lambda i, j: F(a[i] - h[i]) > 0 or F(a[j] - h[j]) > 0
        mask = np.array([(1.0 if outside(1, 2) else -1.0), (1.0 if outside(0, 2) else -1.0),
                         (1.0 if outside(0, 1) else -1.0)], F) * MAXF
        closest = np.fmax(a, h) if (a[0] < h[0] and a[1] < h[1] and a[2] < h[2]) else np.fmin(a, h)
        return np.fmax(a - closest, mask)
    if isinstance(src, S.Cylinder):
        r, hl = F(src.radius), F(src.half_length)
        r2 = F(r * r)
        with np.errstate(invalid="ignore"):
            vx = MAXF if (a[2] > hl or a[1] > r) else F(a[0] - np.sqrt(F(r2 - F(a[1] * a[1]))))
            vy = MAXF if (a[2] > hl or a[0] > r) else F(a[1] - np.sqrt(F(r2 - F(a[0] * a[0]))))
        vz = MAXF if F(F(a[0] * a[0]) + F(a[1] * a[1])) > r2 else F(a[2] - hl)
        return np.array([vx, vy, vz], F)
    if isinstance(src, S.Torus):
        R, t = F(src.radius), F(src.tube_radius)
        with np.errstate(invalid="ignore"):
            l_xy = F(np.sqrt(F(F(a[0] * a[0]) + F(a[1] * a[1]))) - R)
            trz = np.sqrt(F(F(t * t) - F(a[2] * a[2])))
            rx, ry = F(R + trz), F(R - trz)

            def along(u, w):  # the component along axis u, w the other planar axis
                if a[2] > t or a[w] > F(R + trz):
                    return MAXF
                if a[u] == 0:
                    return F(abs(F(a[w] - R)) - t)
                return np.fmax(F(a[u] - np.sqrt(F(F(rx * rx) - F(a[w] * a[w])))),
                               F(np.sqrt(F(F(ry * ry) - F(a[w] * a[w]))) - a[u]))
            vz = MAXF if abs(l_xy) > t else F(a[2] - np.sqrt(F(F(t * t) - F(l_xy * l_xy))))
            return np.array([along(0, 1), along(1, 0), vz], F)
    if isinstance(src, S.Union):
        return np.fmin(vector(src.a, p), vector(src.b, p))
    if isinstance(src, S.Intersection):
        return np.fmax(vector(src.a, p), vector(src.b, p))
    if isinstance(src, S.Difference):
        return np.fmax(vector(src.b, p), -vector(src.a, p))
    if isinstance(src, S.Translate):
        c = [F(v) for v in src.centre]
        return vector(src.source, (F(x - c[0]), F(y - c[1]), F(z - c[2])))
    if isinstance(src, S.DomainMap):
        sc, of = [F(v) for v in src.scale], [F(v) for v in src.offset]
        return vector(src.source, (F(x * sc[0] + of[0]), F(y * sc[1] + of[1]), F(z * sc[2] + of[2])))
    if isinstance(src, S.CentralDifference):
        return vector(src.source, p)
    raise TypeError(type(src))


@pytest.mark.parametrize("name", ["sphere", "box", "cylinder", "torus", "csg", "intersection", "domain",
                                  "central_difference"])
def test_source_directed_vectors_match_oracle(name):
    src = SCENES[name]
    pts = np.random.default_rng(12).uniform(-1.1, 1.1, (400, 3)).astype(F)
    pts[:10] = 0.0
    pts[10:30, 0] = 0.0  # the torus's a.x == 0 branch
    got = np.array([vector(src, p) for p in pts], F)
    want = oracle.Program(S.lower(src)).sample_vector(pts)
    assert np.array_equal(got, want), np.nonzero(np.any(got != want, axis=1))[0][:5]
