"""Seeded synthetic scenes for the workloads the library is measured on.

No dataset exists for this path: every scene is generated from a seed with
SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number
generators", 2014), so the CPU and GPU sides see identical f32 parameters.

* ``sphere``           64^3 cells, one sphere r=0.75 at the origin of [-1,1]^3
* ``sphere_union``     512^3 cells, hard-min union of 64 spheres, centres
                       U[-0.8,0.8]^3, radii U[0.05,0.25]
* ``csg``              (box half 0.6) minus (sphere r=0.7), union torus
                       (R=0.5, r=0.15), each primitive under a seeded rigid
                       transform, for DualContouring / LinearHashedMarchingCubes
* ``chunks``           uneven chunks (50% 16^3, 35% 32^3, 15% 64^3 cells) of
                       1-16 random spheres / boxes / tori each
* ``smooth_spheres``   smooth-min (k=0.05) union of 4096 spheres, centres
                       U[-0.9,0.9]^3, radii U[0.01,0.08]
* ``bench_torus``      the reference benchmark's source, Torus(0.25, 0.1) at the
                       origin of the [0,1]^3 sample frame (benches/isosurface.rs:21-31)
* ``demo_torus``       the deferred-rasterisation example's source: the same torus
                       moved to the frame's centre, with central-difference normals
"""
import numpy as np

from .source import (CentralDifference, Difference, RectangularPrism, Rigid, Sphere, SphereSet, Torus, Translate,
                     Union, unit_to_cube)

MASK64 = (1 << 64) - 1


class SplitMix64:
    def __init__(self, seed):
        self.state = seed & MASK64

    def next_u64(self):
        self.state = (self.state + 0x9E3779B97F4A7C15) & MASK64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & MASK64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & MASK64
        return z ^ (z >> 31)

    def uniform(self, lo=0.0, hi=1.0):
        """f64 in [lo, hi) from the top 53 bits."""
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / 9007199254740992.0))

    def uniforms(self, n, lo=0.0, hi=1.0):
        return np.array([self.uniform(lo, hi) for _ in range(n)], dtype=np.float64)

    def below(self, n):
        return self.next_u64() % n


def random_spheres(seed, count, centre_range, radius_range):
    rng = SplitMix64(seed)
    out = np.empty((count, 4), np.float32)
    for i in range(count):
        out[i, 0:3] = rng.uniforms(3, -centre_range, centre_range)
        out[i, 3] = rng.uniform(*radius_range)
    return out


def random_rotation(rng):
    """Uniform rotation from a unit quaternion (Shoemake, Graphics Gems III, 1992)."""
    u1, u2, u3 = rng.uniform(), rng.uniform(), rng.uniform()
    a, b = np.sqrt(1.0 - u1), np.sqrt(u1)
    q = (a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2), b * np.sin(2 * np.pi * u3), b * np.cos(2 * np.pi * u3))
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]], dtype=np.float32)


def sphere():
    return unit_to_cube(Sphere(0.75))


def sphere_union(seed=1234, count=64):
    return unit_to_cube(SphereSet(random_spheres(seed, count, 0.8, (0.05, 0.25))))


def csg(seed=42):
    rng = SplitMix64(seed)

    def rigid(src):
        t = rng.uniforms(3, -0.1, 0.1)
        return Rigid(src, t, random_rotation(rng))

    box = rigid(RectangularPrism((0.6, 0.6, 0.6)))
    ball = rigid(Sphere(0.7))
    torus = rigid(Torus(0.5, 0.15))
    return unit_to_cube(Union(Difference(ball, box), torus))


def chunk_scene(rng):
    """One chunk's scene: 1-16 random primitives in chunk-local [-1,1]^3."""
    n = 1 + int(rng.below(16))
    prims = []
    for _ in range(n):
        kind = int(rng.below(3))
        c = rng.uniforms(3, -0.8, 0.8)
        if kind == 0:
            p = Sphere(rng.uniform(0.1, 0.5))
        elif kind == 1:
            p = RectangularPrism(tuple(rng.uniforms(3, 0.1, 0.4)))
        else:
            p = Torus(rng.uniform(0.2, 0.4), rng.uniform(0.05, 0.15))
        prims.append(Translate(p, c))
    s = prims[0]
    for p in prims[1:]:
        s = Union(s, p)
    return unit_to_cube(s)


def chunks(seed=7, count=4096):
    """(size, source) per chunk; size is MarchingCubes::new's argument (cells + 1)."""
    rng = SplitMix64(seed)
    out = []
    for _ in range(count):
        u = rng.uniform()
        cells = 16 if u < 0.50 else (32 if u < 0.85 else 64)
        out.append((cells + 1, chunk_scene(rng)))
    return out


def smooth_spheres(seed=99, count=4096, k=0.05):
    return unit_to_cube(SphereSet(random_spheres(seed, count, 0.9, (0.01, 0.08)), smooth_k=k))


def bench_torus():
    return Torus(0.25, 0.1)


def demo_torus():
    """The deferred-rasterisation example's source: CentralDifference over
    DemoSource(Torus(0.25, 0.1)), DemoSource sampling its source at p - 0.5
    (examples/deferred_rasterisation.rs:78-80, examples/common/sources.rs:38-57)."""
    return CentralDifference(Translate(Torus(0.25, 0.1), (0.5, 0.5, 0.5)))
