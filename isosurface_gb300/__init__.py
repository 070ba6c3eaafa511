"""GB300-native isosurface extraction, a drop-in for swiftcoder/isosurface's
extraction hot path (MarchingCubes, DualContouring, LinearHashedMarchingCubes,
ExtendedMarchingCubes and PointCloud over implicit sources), running hand-written sm_103a CUDA behind the C ABI
declared in include/isosurface_gpu.h.
"""
from .source import (CentralDifference, Cylinder, Difference, DomainMap, Intersection, RectangularPrism, Rigid,
                     Sampler, SmoothUnion, Source, Sphere, SphereSet, Torus, Translate, Union, lower, unit_to_cube)
from ._capi import IsoError
from .api import (Context, DualContouring, ExtendedMarchingCubes, IndexedInterleavedNormals, IndexedVertices,
                  LinearHashedMarchingCubes, MarchingCubes, Mesh, MinimiseQEF, OnlyInterleavedNormals, OnlyVertices,
                  ParticleBasedMinimisation, PointCloud, Program, default_context)

__all__ = [
    "CentralDifference", "Cylinder", "Difference", "DomainMap", "Intersection", "RectangularPrism", "Rigid", "Sampler",
    "SmoothUnion", "Source", "Sphere", "SphereSet", "Torus", "Translate", "Union", "lower", "unit_to_cube",
    "IsoError", "Context", "DualContouring", "ExtendedMarchingCubes", "LinearHashedMarchingCubes", "MinimiseQEF", "ParticleBasedMinimisation", "IndexedInterleavedNormals", "IndexedVertices", "MarchingCubes", "Mesh",
    "OnlyInterleavedNormals", "OnlyVertices", "PointCloud", "Program", "default_context",
]
