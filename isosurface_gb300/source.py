"""Implicit sources, mirroring the reference's Source types, lowered to the byte
program that the GPU library evaluates.

Reference types (swiftcoder/isosurface):

* ``Sphere``            src/implicit/sphere.rs:35-63
* ``RectangularPrism``  src/implicit/rectangular_prism.rs:36-80
* ``Cylinder``          src/implicit/cylinder.rs:41-85
* ``Torus``             src/implicit/torus.rs:40-108
* ``Union`` / ``Intersection`` / ``Difference``  src/implicit/csg.rs:22-106
* ``CentralDifference`` src/source.rs:52-95
* ``Sampler``           src/sampler.rs:26-65

Sources with no reference counterpart, needed by the workloads:

* ``DomainMap``    q = p*scale + offset (the examples' DemoSource shift,
                   examples/common/sources.rs:38-57, generalised), e.g. the
                   reference's [0,1]^3 sample frame onto [-1,1]^3
* ``Translate``    q = p - centre
* ``Rigid``        q = M (p - t), normal rotated back by M^T
* ``SmoothUnion``  polynomial smooth minimum (Quilez 2013)
* ``SphereSet``    a left fold of Union (or SmoothUnion) over translated
                   spheres, evaluated as one op

A source is lowered with :func:`lower` into the program format documented in
``include/isosurface_gpu.h`` ("Source programs").  Lowering is exact: every
constant is stored as the f32 the reference would hold.
"""
import struct

import numpy as np

__all__ = [
    "Source", "Sphere", "RectangularPrism", "Cylinder", "Torus", "Union", "Intersection",
    "Difference", "SmoothUnion", "Translate", "Rigid", "DomainMap", "SphereSet",
    "CentralDifference", "Sampler", "lower", "unit_to_cube",
]

MAGIC = 0x314F5349  # "ISO1"

OP_PT_DOMAIN = 0x01
OP_PT_TRANSLATE = 0x02
OP_PT_RIGID = 0x03
OP_PT_POP = 0x04
OP_SPHERE = 0x10
OP_BOX = 0x11
OP_CYLINDER = 0x12
OP_TORUS = 0x13
OP_UNION = 0x20
OP_INTERSECTION = 0x21
OP_DIFFERENCE = 0x22
OP_SMOOTH_UNION = 0x23
OP_SPHERE_SET = 0x30
OP_CD_BEGIN = 0x40
OP_CD_END = 0x41


def _f32(v):
    return float(np.float32(v))


class _Emitter:
    def __init__(self):
        self.ops = []
        self.consts = []

    def const(self, values):
        at = len(self.consts)
        self.consts.extend(_f32(v) for v in values)
        if at >= (1 << 24):
            raise ValueError("program has too many constants")
        return at

    def op(self, code, arg=0):
        self.ops.append((arg << 8) | code)


class Source:
    """Base of every implicit source.  ``has_normal`` mirrors whether the
    reference type implements ``HermiteSource``."""

    has_normal = True

    def _emit(self, e):
        raise NotImplementedError

    def lower(self):
        return lower(self)


class Sphere(Source):
    def __init__(self, radius):
        self.radius = radius

    def _emit(self, e):
        e.op(OP_SPHERE, e.const([self.radius]))


class RectangularPrism(Source):
    def __init__(self, half_extent):
        self.half_extent = tuple(half_extent)

    def _emit(self, e):
        e.op(OP_BOX, e.const(self.half_extent))


class Cylinder(Source):
    def __init__(self, radius, half_length):
        self.radius, self.half_length = radius, half_length

    def _emit(self, e):
        e.op(OP_CYLINDER, e.const([self.radius, self.half_length]))


class Torus(Source):
    def __init__(self, radius, tube_radius):
        self.radius, self.tube_radius = radius, tube_radius

    def _emit(self, e):
        e.op(OP_TORUS, e.const([self.radius, self.tube_radius]))


class _Binary(Source):
    code = None

    def __init__(self, a, b):
        self.a, self.b = a, b

    @property
    def has_normal(self):
        return self.a.has_normal and self.b.has_normal

    def _emit(self, e):
        self.a._emit(e)
        self.b._emit(e)
        e.op(self.code)


class Union(_Binary):
    """min(a, b); normal is the component-wise min of the two normals (csg.rs:47-51)."""
    code = OP_UNION


class Intersection(_Binary):
    """max(a, b); normal of the operand attaining the max (the reference has none)."""
    code = OP_INTERSECTION


class Difference(_Binary):
    """b minus a: max(b, -a) (csg.rs:96-100); normal of b, or -normal of a."""
    code = OP_DIFFERENCE


class SmoothUnion(_Binary):
    """h = max(k - |a-b|, 0)/k ; min(a, b) - h*h*k/4."""

    def __init__(self, a, b, k):
        super().__init__(a, b)
        self.k = k

    def _emit(self, e):
        self.a._emit(e)
        self.b._emit(e)
        e.op(OP_SMOOTH_UNION, e.const([self.k]))


class _PointScope(Source):
    def __init__(self, source):
        self.source = source

    @property
    def has_normal(self):
        return self.source.has_normal

    def _emit(self, e):
        e.op(self.code, e.const(self._params()))
        self.source._emit(e)
        e.op(OP_PT_POP)


class DomainMap(_PointScope):
    code = OP_PT_DOMAIN

    def __init__(self, source, scale=(2.0, 2.0, 2.0), offset=(-1.0, -1.0, -1.0)):
        super().__init__(source)
        self.scale, self.offset = tuple(scale), tuple(offset)

    def _params(self):
        return list(self.scale) + list(self.offset)


def unit_to_cube(source, lo=-1.0, hi=1.0):
    """Map the reference's [0,1]^3 sample frame onto [lo,hi]^3: q = p*(hi-lo) + lo."""
    s = hi - lo
    return DomainMap(source, (s, s, s), (lo, lo, lo))


class Translate(_PointScope):
    code = OP_PT_TRANSLATE

    def __init__(self, source, centre):
        super().__init__(source)
        self.centre = tuple(centre)

    def _params(self):
        return list(self.centre)


class Rigid(_PointScope):
    """q = M (p - t) with M a row-major 3x3 rotation."""
    code = OP_PT_RIGID

    def __init__(self, source, translation, rotation):
        super().__init__(source)
        self.t = tuple(translation)
        self.m = [float(v) for v in np.asarray(rotation, dtype=np.float64).reshape(9)]

    def _params(self):
        return list(self.t) + self.m


class SphereSet(Source):
    """Union (hard) or SmoothUnion (smooth, k) folded left over spheres given as
    an (n, 4) array of (cx, cy, cz, r)."""

    def __init__(self, spheres, smooth_k=None):
        self.spheres = np.asarray(spheres, dtype=np.float32).reshape(-1, 4)
        if len(self.spheres) == 0:
            raise ValueError("SphereSet needs at least one sphere")
        self.smooth_k = smooth_k

    def _emit(self, e):
        n = len(self.spheres)
        if n >= (1 << 24):
            raise ValueError("too many spheres")
        head = [float(n), 0.0 if self.smooth_k is None else 1.0,
                0.0 if self.smooth_k is None else self.smooth_k]
        at = e.const(head)
        e.const(self.spheres.reshape(-1).tolist())
        e.op(OP_SPHERE_SET, at)


class CentralDifference(Source):
    """Normals by central differences of the scalar field (source.rs:52-95)."""

    def __init__(self, source, epsilon=0.000001):
        self.source, self.epsilon = source, epsilon

    def _emit(self, e):
        e.op(OP_CD_BEGIN, e.const([self.epsilon]))
        self.source._emit(e)
        e.op(OP_CD_END)


class Sampler:
    """Thin borrow wrapper over a source (sampler.rs:26-65)."""

    def __init__(self, source):
        self.source = source

    @property
    def has_normal(self):
        return self.source.has_normal

    def lower(self):
        return lower(self.source)


def lower(source):
    """Lower a source tree to program bytes."""
    if isinstance(source, Sampler):
        source = source.source
    e = _Emitter()
    source._emit(e)
    head = struct.pack("<4I", MAGIC, len(e.ops), len(e.consts), 0)
    return head + struct.pack("<%dI" % len(e.ops), *e.ops) + np.asarray(e.consts, dtype=np.float32).tobytes()


def from_spec(spec):
    """Build a source from the JSON spec used by the golden fixtures."""
    t = spec["type"]
    if t == "sphere":
        return Sphere(spec["radius"])
    if t == "box":
        return RectangularPrism(spec["half_extent"])
    if t == "cylinder":
        return Cylinder(spec["radius"], spec["half_length"])
    if t == "torus":
        return Torus(spec["radius"], spec["tube_radius"])
    if t in ("union", "intersection", "difference"):
        cls = {"union": Union, "intersection": Intersection, "difference": Difference}[t]
        return cls(from_spec(spec["a"]), from_spec(spec["b"]))
    raise ValueError("unknown source spec " + t)
