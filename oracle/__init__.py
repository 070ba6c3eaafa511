"""ctypes front end of the oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a CPU restatement of swiftcoder/isosurface's extraction path
(iso_oracle.cpp).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
legs use it, as the checker; the GPU library never does.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = ctypes.CDLL(path)
        vp, u8p, f32p, u32p, u64p, f64p = (ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint8),
                                           ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_uint32),
                                           ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_double))
        sig = {
            "oracle_program_create": (vp, [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t]),
            "oracle_program_destroy": (None, [vp]),
            "oracle_program_has_normal": (ctypes.c_int, [vp]),
            "oracle_program_has_vector": (ctypes.c_int, [vp]),
            "oracle_sample_vector": (None, [vp, f32p, ctypes.c_uint64, f32p]),
            "oracle_emc": (vp, [vp, ctypes.c_uint32, ctypes.c_int, u64p, ctypes.c_uint64]),
            "oracle_emc_place": (ctypes.c_int, [f32p, f32p, ctypes.c_int, f32p]),
            "oracle_sample_scalar": (None, [vp, f32p, ctypes.c_uint64, f32p]),
            "oracle_sample_normal": (None, [vp, f32p, ctypes.c_uint64, f32p]),
            "oracle_sample_grid": (None, [vp, ctypes.c_uint32, f32p]),
            "oracle_mc_cases": (None, [vp, ctypes.c_uint32, u8p]),
            "oracle_mc": (vp, [vp, ctypes.c_uint32, ctypes.c_uint32]),
            "oracle_mc_slab": (vp, [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32]),
            "oracle_point_cloud": (vp, [vp, ctypes.c_uint32]),
            "oracle_dc": (vp, [vp, ctypes.c_uint32, ctypes.c_int, f32p]),
            "oracle_lhmc": (vp, [vp, ctypes.c_uint32]),
            "oracle_lhmc_nodes": (ctypes.c_uint64, [vp, ctypes.c_uint32, u64p, ctypes.c_uint64]),
            "oracle_mesh_vertices": (ctypes.c_uint64, [vp]),
            "oracle_mesh_indices": (ctypes.c_uint64, [vp]),
            "oracle_mesh_cells": (ctypes.c_uint64, [vp]),
            "oracle_mesh_stale": (ctypes.c_uint64, [vp]),
            "oracle_mesh_copy": (None, [vp, f32p, u32p, u64p, f32p]),
            "oracle_mesh_destroy": (None, [vp]),
            "oracle_svd_solve": (None, [f64p, ctypes.c_int, f64p, f64p, f64p]),
            "oracle_place_feature": (None, [f32p, f32p, ctypes.c_int, f32p, ctypes.POINTER(ctypes.c_int)]),
            "oracle_morton_level": (ctypes.c_int, [ctypes.c_uint64]),
            "oracle_morton_center": (None, [ctypes.c_uint64, f32p]),
            "oracle_morton_primal_vertex": (ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64]),
            "oracle_morton_dual_vertex": (ctypes.c_uint64, [ctypes.c_uint64, ctypes.c_int, ctypes.c_uint64]),
            "oracle_morton_level_rule_check": (ctypes.c_uint64, [ctypes.c_uint64]),
            "oracle_mc_timed": (ctypes.c_double, [vp, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32,
                                                  ctypes.c_int, u64p, u64p]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a, ctype):
    return a.ctypes.data_as(ctypes.POINTER(ctype)) if a is not None else None


class Mesh:
    """A mesh the oracle extracted, with its per-vertex dedup keys."""

    def __init__(self, handle, with_normals=False):
        L = lib()
        nv = L.oracle_mesh_vertices(handle)
        ni = L.oracle_mesh_indices(handle)
        self.vertices = np.empty((nv, 3), np.float32)
        self.indices = np.empty(ni, np.uint32)
        self.keys = np.empty((nv, 2), np.uint64)
        self.normals = np.empty((nv, 3), np.float32) if with_normals else None
        L.oracle_mesh_copy(handle, _ptr(self.vertices, ctypes.c_float), _ptr(self.indices, ctypes.c_uint32),
                           _ptr(self.keys, ctypes.c_uint64), _ptr(self.normals, ctypes.c_float))
        self.cells = L.oracle_mesh_cells(handle)
        self.stale_corners = L.oracle_mesh_stale(handle)
        L.oracle_mesh_destroy(handle)

    @property
    def triangles(self):
        return self.indices.reshape(-1, 3)


class Program:
    """An oracle source built from program bytes."""

    def __init__(self, program_bytes):
        err = ctypes.create_string_buffer(256)
        self.h = lib().oracle_program_create(program_bytes, len(program_bytes), err, 256)
        if not self.h:
            raise ValueError("oracle rejected program: " + err.value.decode())

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_program_destroy(self.h)
            self.h = None

    @property
    def has_normal(self):
        return bool(lib().oracle_program_has_normal(self.h))

    def sample_scalar(self, pts):
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        out = np.empty(len(pts), np.float32)
        lib().oracle_sample_scalar(self.h, _ptr(pts, ctypes.c_float), len(pts), _ptr(out, ctypes.c_float))
        return out

    def sample_normal(self, pts):
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        out = np.empty((len(pts), 3), np.float32)
        lib().oracle_sample_normal(self.h, _ptr(pts, ctypes.c_float), len(pts), _ptr(out, ctypes.c_float))
        return out

    @property
    def has_vector(self):
        """Whether the source defines the Directed metric (sample_vector)."""
        return bool(lib().oracle_program_has_vector(self.h))

    def sample_vector(self, pts):
        pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
        out = np.empty((len(pts), 3), np.float32)
        lib().oracle_sample_vector(self.h, _ptr(pts, ctypes.c_float), len(pts), _ptr(out, ctypes.c_float))
        return out

    def extended_marching_cubes(self, size, normals=False, flip_order_seed=0):
        """ExtendedMarchingCubes::new(size).extract; the mesh carries
        `features` (feature vertices), `flips` (edges rotated) and
        `conflicts` (flips whose result would depend on their order).  The
        reference applies its flips in HashSet order; flip_order_seed 0 uses
        ascending order, other values a seeded random order."""
        if not self.has_vector:
            raise ValueError("ExtendedMarchingCubes needs a source with the Directed metric")
        stats = np.zeros(3, np.uint64)
        m = Mesh(lib().oracle_emc(self.h, size, 1 if normals else 0, _ptr(stats, ctypes.c_uint64),
                                  flip_order_seed), with_normals=normals)
        m.features, m.flips, m.conflicts = (int(v) for v in stats)
        return m

    def sample_grid(self, size):
        out = np.empty((size + 1, size, size), np.float32)
        lib().oracle_sample_grid(self.h, size, _ptr(out, ctypes.c_float))
        return out

    def mc_cases(self, size):
        out = np.empty((size, size - 1, size - 1), np.uint8)
        lib().oracle_mc_cases(self.h, size, _ptr(out, ctypes.c_uint8))
        return out

    def marching_cubes(self, size, normals=False):
        return Mesh(lib().oracle_mc(self.h, size, 1 if normals else 0), with_normals=normals)

    def marching_cubes_slab(self, size, z0, z1):
        return Mesh(lib().oracle_mc_slab(self.h, size, z0, z1))

    def point_cloud(self, size):
        return Mesh(lib().oracle_point_cloud(self.h, size))

    def dual_contouring(self, size, placer=0, with_duals=False):
        duals = np.empty((size, size - 1, size - 1, 4), np.float32) if with_duals else None
        m = Mesh(lib().oracle_dc(self.h, size, placer, _ptr(duals, ctypes.c_float)))
        return (m, duals) if with_duals else m

    def lhmc(self, max_depth):
        return Mesh(lib().oracle_lhmc(self.h, max_depth))

    def lhmc_nodes(self, max_depth):
        n = lib().oracle_lhmc_nodes(self.h, max_depth, None, 0)
        out = np.empty((n, 2), np.uint64)
        lib().oracle_lhmc_nodes(self.h, max_depth, _ptr(out, ctypes.c_uint64), n)
        return out

    def mc_timed(self, size, z0, z1, threads=1):
        cells = ctypes.c_uint64()
        tris = ctypes.c_uint64()
        secs = lib().oracle_mc_timed(self.h, size, z0, z1, threads, ctypes.byref(cells), ctypes.byref(tris))
        return secs, cells.value, tris.value


def svd_solve(mat, b):
    mat = np.ascontiguousarray(mat, np.float64).reshape(-1, 3)
    b = np.ascontiguousarray(b, np.float64)
    d = np.empty(3, np.float64)
    x = np.empty(3, np.float64)
    lib().oracle_svd_solve(_ptr(mat, ctypes.c_double), len(mat), _ptr(b, ctypes.c_double),
                           _ptr(d, ctypes.c_double), _ptr(x, ctypes.c_double))
    return d, x


def emc_place(vertices, normals):
    """Tangent planes over a cell's edge crossings and MinimiseQEF: (topology
    0 planar / 1 edge / 2 corner, the placed point)."""
    v = np.ascontiguousarray(vertices, np.float32).reshape(-1, 3)
    n = np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
    out = np.zeros(3, np.float32)
    topo = lib().oracle_emc_place(_ptr(v, ctypes.c_float), _ptr(n, ctypes.c_float), len(v), _ptr(out, ctypes.c_float))
    return topo, out


def place_feature(corners, normals, placer=0):
    c = np.ascontiguousarray(corners, np.float32).reshape(8, 3)
    n = np.ascontiguousarray(normals, np.float32).reshape(8, 3)
    out = np.empty(3, np.float32)
    topo = ctypes.c_int()
    lib().oracle_place_feature(_ptr(c, ctypes.c_float), _ptr(n, ctypes.c_float), placer,
                               _ptr(out, ctypes.c_float), ctypes.byref(topo))
    return out, topo.value
