"""Sources with the Directed metric for the ExtendedMarchingCubes tests:
fixed scenes and seeded random CSG trees of translated primitives."""
import numpy as np

from isosurface_gb300 import source as S


def _centred(src):
    return S.Translate(src, (0.5, 0.5, 0.5))


FIXED = {
    "sphere": _centred(S.Sphere(0.3)),
    "cube": _centred(S.RectangularPrism((0.27, 0.27, 0.27))),
    "box": _centred(S.RectangularPrism((0.31, 0.23, 0.17))),
    "cylinder": _centred(S.Cylinder(0.27, 0.21)),
    "torus": _centred(S.Torus(0.25, 0.1)),
    "difference": _centred(S.Difference(S.Sphere(0.3), S.RectangularPrism((0.26, 0.26, 0.26)))),
    "intersection": _centred(S.Intersection(S.Sphere(0.35), S.RectangularPrism((0.28, 0.28, 0.28)))),
    "central_difference": S.CentralDifference(_centred(S.Torus(0.25, 0.1))),
    "domain_csg": S.unit_to_cube(S.Union(S.Difference(S.Sphere(0.7), S.RectangularPrism((0.6, 0.6, 0.6))),
                                         S.Torus(0.5, 0.15))),
}


def random_scenes(seed, count):
    """(size, source) pairs: 1-4 translated primitives joined by Union,
    Intersection and Difference, sizes 4..27."""
    rng = np.random.default_rng(seed)

    def prim():
        k = rng.integers(4)
        if k == 0:
            p = S.Sphere(float(rng.uniform(0.08, 0.35)))
        elif k == 1:
            p = S.RectangularPrism(tuple(float(x) for x in rng.uniform(0.05, 0.3, 3)))
        elif k == 2:
            p = S.Cylinder(float(rng.uniform(0.05, 0.3)), float(rng.uniform(0.05, 0.3)))
        else:
            p = S.Torus(float(rng.uniform(0.12, 0.3)), float(rng.uniform(0.03, 0.1)))
        return S.Translate(p, tuple(float(x) for x in rng.uniform(0.25, 0.75, 3)))

    out = []
    for _ in range(count):
        s = prim()
        for _ in range(int(rng.integers(0, 4))):
            op = int(rng.integers(3))
            s = S.Difference(prim(), s) if op == 2 else (S.Union, S.Intersection)[op](s, prim())
        out.append((int(rng.integers(4, 28)), s))
    return out
