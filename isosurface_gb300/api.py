"""The reference's extraction API over the GPU library.

    mc = MarchingCubes(size)
    mc.extract(Sampler(source), IndexedVertices(vertices, indices))

mirrors ``MarchingCubes::new(size).extract(&sampler, &mut extractor)``
(src/marching_cubes.rs:46-82); DualContouring, LinearHashedMarchingCubes and
PointCloud follow their reference constructors in the same way.  The mesh is
extracted on the GPU and then replayed into the extractor: bulk for the
extractors defined here, one ``extract_vertex`` / ``extract_index`` call per
element for any other object with those methods (the reference's Extractor
trait, src/extractor.rs:17-20).
"""
import ctypes

import numpy as np

from . import _capi
from ._capi import ISO_FLAG_KEYS, ISO_FLAG_NORMALS, IsoError, MeshInfo, check, lib
from .source import Sampler, Source, lower

__all__ = [
    "Context", "Program", "Mesh", "default_context", "MarchingCubes", "PointCloud",
    "OnlyVertices", "IndexedVertices", "OnlyInterleavedNormals", "IndexedInterleavedNormals",
]


class Program:
    """A source program uploaded to a context."""

    def __init__(self, ctx, source_or_bytes):
        self.ctx = ctx
        data = source_or_bytes if isinstance(source_or_bytes, (bytes, bytearray)) else lower(source_or_bytes)
        self.bytes = bytes(data)
        h = ctypes.c_void_p()
        check(lib().iso_program_create(ctx.h, self.bytes, len(self.bytes), ctypes.byref(h)), ctx.h)
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            lib().iso_program_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Mesh:
    """A mesh copied back from the device: vertices (n, 3) or (n, 6) f32,
    triangles (m, 3) u32, keys (n, 2) u64 when requested."""

    def __init__(self, vertices, indices, keys=None, cells=0):
        self.vertices = vertices
        self.indices = indices
        self.keys = keys
        self.cells = cells

    @property
    def triangles(self):
        return self.indices.reshape(-1, 3)


class Context:
    """One iso_ctx: a CUDA stream plus reusable device buffers."""

    def __init__(self, device=0):
        h = ctypes.c_void_p()
        check(lib().iso_ctx_create(device, ctypes.byref(h)))
        self.h = h
        self.device = device
        self._programs = {}
        self._vertex_floats = 3  # 6 after an extraction with per-vertex normals

    def close(self):
        if getattr(self, "h", None):
            for p in self._programs.values():
                p.close()
            self._programs.clear()
            lib().iso_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        s = ctypes.c_void_p()
        check(lib().iso_ctx_get_stream(self.h, ctypes.byref(s)), self.h)
        return s.value

    def set_stream(self, stream_handle):
        check(lib().iso_ctx_set_stream(self.h, ctypes.c_void_p(stream_handle)), self.h)

    @property
    def kernel_launches(self):
        return lib().iso_ctx_kernel_launches(self.h)

    def debug_fail_allocation(self, after):
        """Test hook: the device-buffer allocation after `after` successful
        ones fails as a failed cudaMalloc does (negative: off)."""
        check(lib().iso_debug_fail_allocation(self.h, int(after)), self.h)

    def program(self, source):
        """Upload (once per distinct program) and return a Program (a Program
        of this context is returned as it is)."""
        if isinstance(source, Program) and source.ctx is self:
            return source
        data = source if isinstance(source, (bytes, bytearray)) else lower(source)
        data = bytes(data)
        p = self._programs.get(data)
        if p is None:
            p = Program(self, data)
            self._programs[data] = p
        return p

    # -- extraction ---------------------------------------------------------
    def _flags(self, keys, normals):
        self._vertex_floats = 6 if normals else 3
        return (ISO_FLAG_KEYS if keys else 0) | (ISO_FLAG_NORMALS if normals else 0)

    def mc_extract(self, source, size, keys=False, normals=False):
        info = MeshInfo()
        flags = self._flags(keys, normals)
        check(lib().iso_mc_extract(self.h, self.program(source).h, size, flags, ctypes.byref(info)), self.h)
        return info

    def mc_extract_host(self, source, size, vertices, indices, normals=False):
        """MarchingCubes straight into host buffers: `vertices` (f32, 3 or, with
        normals, 6 per vertex) and `indices` (u32 / i32, 3 per triangle), numpy
        arrays or CPU torch tensors.  Page-locked buffers (torch
        ``pin_memory=True``) are filled by the extraction kernels themselves.
        Returns the MeshInfo; raises IsoError (capacity) when a buffer is too
        small, with the mesh left on the device for ``download``."""
        def addr(a):
            if hasattr(a, "data_ptr"):
                if a.is_cuda or not a.is_contiguous():
                    raise ValueError("host buffers must be contiguous CPU memory")
                return a.data_ptr(), a.numel()
            if not a.flags.c_contiguous:
                raise ValueError("host buffers must be contiguous")
            return a.ctypes.data, a.size
        pv, nv = addr(vertices)
        pi, ni = addr(indices)
        info = MeshInfo()
        flags = self._flags(False, normals)
        check(lib().iso_mc_extract_host(self.h, self.program(source).h, size, flags, ctypes.c_void_p(pv), nv,
                                        ctypes.c_void_p(pi), ni, ctypes.byref(info)), self.h)
        return info

    def mc_extract_field(self, field_ptr, nx, ny, nz, pitch, keys=False):
        info = MeshInfo()
        flags = self._flags(keys, False)
        check(lib().iso_mc_extract_field(self.h, ctypes.c_void_p(field_ptr), nx, ny, nz, pitch, flags,
                                         ctypes.byref(info)), self.h)
        return info

    def mc_extract_slab(self, source, size, z_begin, z_end, keys=False):
        """One slab of a z-partition of MarchingCubes::new(size): cell layers
        [z_begin, z_end) plus the halo layer below when z_begin > 0.  Returns
        (MeshInfo, halo vertices, halo triangles); see slabs.py."""
        info = MeshInfo()
        hv, ht = ctypes.c_uint64(), ctypes.c_uint64()
        flags = self._flags(keys, False)
        check(lib().iso_mc_extract_slab(self.h, self.program(source).h, size, z_begin, z_end, flags,
                                        ctypes.byref(info), ctypes.byref(hv), ctypes.byref(ht)), self.h)
        return info, int(hv.value), int(ht.value)

    def dc_extract_slab(self, source, size, z_begin, z_end, placer=0, keys=False):
        """One slab of a z-partition of DualContouring::new(size, placer):
        dual cube layers [z_begin, z_end) of size - 1, plus the halo layer
        below when z_begin > 0.  Returns (MeshInfo, halo vertices, halo
        triangles); slabs.py assembles the slabs with size - 1 as the size."""
        info = MeshInfo()
        hv, ht = ctypes.c_uint64(), ctypes.c_uint64()
        flags = self._flags(keys, False)
        check(lib().iso_dc_extract_slab(self.h, self.program(source).h, size, placer, z_begin, z_end, flags,
                                        ctypes.byref(info), ctypes.byref(hv), ctypes.byref(ht)), self.h)
        return info, int(hv.value), int(ht.value)

    def mc_cases(self, source, size):
        out = np.empty((size, size - 1, size - 1), np.uint8)
        check(lib().iso_mc_cases(self.h, self.program(source).h, size,
                                 out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))), self.h)
        return out

    def dc_extract(self, source, size, placer=0, keys=False, normals=False):
        info = MeshInfo()
        flags = self._flags(keys, normals)
        check(lib().iso_dc_extract(self.h, self.program(source).h, size, placer, flags, ctypes.byref(info)), self.h)
        return info

    def lhmc_extract(self, source, max_depth, keys=False, normals=False):
        info = MeshInfo()
        flags = self._flags(keys, normals)
        check(lib().iso_lhmc_extract(self.h, self.program(source).h, max_depth, flags, ctypes.byref(info)), self.h)
        return info

    @property
    def lhmc_stale_corners(self):
        return lib().iso_lhmc_stale_corners(self.h)

    def point_cloud_extract(self, source, size, normals=False):
        info = MeshInfo()
        flags = self._flags(False, normals)
        check(lib().iso_point_cloud_extract(self.h, self.program(source).h, size, flags, ctypes.byref(info)), self.h)
        return info

    def emc_extract(self, source, size, normals=False):
        """ExtendedMarchingCubes::new(size).extract; returns (info, flips)."""
        info = MeshInfo()
        flips = ctypes.c_uint64()
        flags = self._flags(False, normals)
        check(lib().iso_emc_extract(self.h, self.program(source).h, size, flags, ctypes.byref(info),
                                    ctypes.byref(flips)), self.h)
        return info, flips.value

    def point_splat(self, width, height, voxel_half, view_proj=None, view_proj_inverse=None, clear=None,
                    edge="empty"):
        """Deferred point-splat image of the last PointCloud extraction with
        normals (examples/deferred_rasterisation.rs), (height, width, 4)
        float32, row 0 at the bottom.  Without matrices, the example's camera
        (isosurface_gb300.render.splat_camera).  edge: gather taps past the
        image edge read as "empty", or through "mirror"ed-repeat addressing."""
        if edge not in ("empty", "mirror"):
            raise ValueError("edge must be 'empty' or 'mirror'")
        from . import render
        if view_proj is None or view_proj_inverse is None:
            view_proj, view_proj_inverse = render.splat_camera(width, height)
        vp = np.ascontiguousarray(view_proj, np.float32).reshape(16)
        vpi = np.ascontiguousarray(view_proj_inverse, np.float32).reshape(16)
        col = np.ascontiguousarray(render.CLEAR_RGB if clear is None else clear, np.float32).reshape(3)
        out = np.empty((height, width, 4), np.float32)
        f32p = ctypes.POINTER(ctypes.c_float)
        if edge == "empty":
            st = lib().iso_point_splat_render(self.h, vp.ctypes.data_as(f32p), vpi.ctypes.data_as(f32p), width,
                                              height, float(voxel_half), col.ctypes.data_as(f32p),
                                              out.ctypes.data_as(f32p))
        else:
            st = lib().iso_point_splat_render_ex(self.h, vp.ctypes.data_as(f32p), vpi.ctypes.data_as(f32p), width,
                                                 height, float(voxel_half), col.ctypes.data_as(f32p), 1,
                                                 out.ctypes.data_as(f32p))
        check(st, self.h)
        return out

    def sample_grid(self, source, size, field_ptr, pitch):
        check(lib().iso_sample_grid(self.h, self.program(source).h, size, ctypes.c_void_p(field_ptr), pitch), self.h)

    def sample_grid_near(self, source, size, field_ptr, pitch, bits_ptr):
        """Sign bits everywhere and values where marching cubes reads them
        (iso_sample_grid_near); other field entries may be left unwritten."""
        check(lib().iso_sample_grid_near(self.h, self.program(source).h, size, ctypes.c_void_p(field_ptr), pitch,
                                         ctypes.c_void_p(bits_ptr)), self.h)

    def compiled(self, source):
        """Whether the program's culled sampling runs a kernel compiled for it (iso_program_compiled)."""
        out = ctypes.c_int()
        check(lib().iso_program_compiled(self.program(source).h, ctypes.byref(out)), self.h)
        return bool(out.value)

    def lipschitz(self, source):
        """The program's Lipschitz bound used for culled sampling (0: none)."""
        out = ctypes.c_float()
        check(lib().iso_program_lipschitz(self.program(source).h, ctypes.byref(out)), self.h)
        return out.value

    def sample_points(self, source, points, normals=False):
        pts = np.ascontiguousarray(points, np.float32).reshape(-1, 3)
        vals = np.empty(len(pts), np.float32)
        nrm = np.empty((len(pts), 3), np.float32) if normals else None
        f32p = ctypes.POINTER(ctypes.c_float)
        check(lib().iso_sample_points(self.h, self.program(source).h, pts.ctypes.data_as(f32p), len(pts),
                                      vals.ctypes.data_as(f32p),
                                      nrm.ctypes.data_as(f32p) if normals else None), self.h)
        return (vals, nrm) if normals else vals

    def download(self, info, keys=False, vertex_floats=None, out=None):
        """Copy the last mesh to host numpy arrays (or into `out` = (vertices, indices)).
        Vertices are (n, 3), or (n, 6) = x y z nx ny nz after an extraction with normals."""
        if vertex_floats is None:
            vertex_floats = self._vertex_floats
        nv, nt = info.num_vertices, info.num_triangles
        if out is not None:
            v, i = out
        else:
            v = np.empty((nv, vertex_floats), np.float32)
            i = np.empty(3 * nt, np.uint32)
        k = np.empty((nv, 2), np.uint64) if keys else None
        check(lib().iso_mesh_download(
            self.h, v.ctypes.data_as(ctypes.POINTER(ctypes.c_float)), v.size,
            i.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)), i.size,
            k.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)) if keys else None, 0 if k is None else k.size), self.h)
        return Mesh(v, i, k, info.num_cells)

    def device_mesh(self):
        v, i, k = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
        info = MeshInfo()
        check(lib().iso_mesh_device(self.h, ctypes.byref(v), ctypes.byref(i), ctypes.byref(k), ctypes.byref(info)),
              self.h)
        return v.value, i.value, k.value, info


class Batch:
    """Many independent MarchingCubes chunks extracted together.

    chunks: list of (size, source); each chunk is MarchingCubes::new(size)
    over its source.  run() meshes all of them (graph=True replays one CUDA
    graph after the first, eager run); meshes() splits the result per chunk."""

    def __init__(self, ctx, chunks):
        from ._capi import ChunkDesc
        self.ctx = ctx
        progs, index, descs = [], {}, []
        for size, src in chunks:
            data = bytes(src if isinstance(src, (bytes, bytearray)) else lower(src))
            if data not in index:
                index[data] = len(progs)
                progs.append(ctx.program(data))
            descs.append(ChunkDesc(index[data], size))
        self.n = len(descs)
        self.sizes = [d.size for d in descs]
        arr = (ctypes.c_void_p * len(progs))(*[p.h.value for p in progs])
        darr = (ChunkDesc * len(descs))(*descs)
        h = ctypes.c_void_p()
        check(lib().iso_batch_create(ctx.h, arr, len(progs), darr, len(descs), ctypes.byref(h)), ctx.h)
        self.h = h
        self._programs = progs

    def close(self):
        if getattr(self, "h", None):
            lib().iso_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, graph=True):
        from ._capi import ISO_BATCH_GRAPH
        info = MeshInfo()
        self.ctx._vertex_floats = 3
        check(lib().iso_batch_run(self.h, ISO_BATCH_GRAPH if graph else 0, ctypes.byref(info)), self.ctx.h)
        return info

    def run_per_chunk(self):
        info = MeshInfo()
        self.ctx._vertex_floats = 3
        check(lib().iso_batch_run_per_chunk(self.h, ctypes.byref(info)), self.ctx.h)
        return info

    def run_per_chunk_async(self):
        """One extraction per chunk with no host synchronisation per chunk
        (the batch must have run once)."""
        info = MeshInfo()
        self.ctx._vertex_floats = 3
        check(lib().iso_batch_run_per_chunk_async(self.h, ctypes.byref(info)), self.ctx.h)
        return info

    def set_slab(self, size, depth):
        check(lib().iso_batch_set_slab(self.h, size, depth), self.ctx.h)

    def autotune(self, cache_path=None):
        out = (ctypes.c_uint32 * 64)()
        check(lib().iso_batch_autotune(self.h, cache_path.encode() if cache_path else None, out), self.ctx.h)
        chosen = {}
        for k in range(32):
            if out[2 * k]:
                chosen[int(out[2 * k])] = int(out[2 * k + 1])
        return chosen

    def extents(self):
        ext = np.empty((self.n, 4), np.uint32)
        check(lib().iso_batch_extents(self.h, ext.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))), self.ctx.h)
        return ext

    def meshes(self, info):
        whole = self.ctx.download(info)
        ext = self.extents()
        out = []
        for v0, nv, t0, nt in ext:
            out.append(Mesh(whole.vertices[v0:v0 + nv], whole.indices[3 * t0:3 * (t0 + nt)]))
        return out


_default = {}


def default_context(device=0):
    ctx = _default.get(device)
    if ctx is None:
        ctx = Context(device)
        _default[device] = ctx
    return ctx


# ---------------------------------------------------------------------------
# Extractors (src/extractor.rs)
# ---------------------------------------------------------------------------
class _Extractor:
    with_normals = False
    with_indices = True

    def take(self, vertices, indices):
        raise NotImplementedError


class OnlyVertices(_Extractor):
    """Vertices as a flat f32 list, faces discarded (extractor.rs:24-42)."""
    with_indices = False

    def __init__(self, vertices):
        self.vertices = vertices

    def take(self, vertices, indices):
        self.vertices.extend(vertices.reshape(-1).tolist())


class IndexedVertices(_Extractor):
    """Vertices as a flat f32 list plus u32 indices (extractor.rs:72-93)."""

    def __init__(self, vertices, indices):
        self.vertices, self.indices = vertices, indices

    def take(self, vertices, indices):
        self.vertices.extend(vertices.reshape(-1).tolist())
        self.indices.extend(indices.tolist())


class OnlyInterleavedNormals(OnlyVertices):
    """x y z nx ny nz per vertex, faces discarded (extractor.rs:46-69): the
    normal is source.sample_normal(vertex), computed on the device from the
    source being extracted (`source` is accepted for the reference's
    signature)."""
    with_normals = True

    def __init__(self, vertices, source=None):
        super().__init__(vertices)
        self.source = source


class IndexedInterleavedNormals(IndexedVertices):
    """x y z nx ny nz per vertex plus indices (extractor.rs:97-127)."""
    with_normals = True

    def __init__(self, vertices, indices, source=None):
        super().__init__(vertices, indices)
        self.source = source


def _replay(extractor, mesh):
    if isinstance(extractor, _Extractor):
        extractor.take(mesh.vertices, mesh.indices)
        return
    for v in mesh.vertices:
        extractor.extract_vertex(tuple(float(c) for c in v))
    for i in mesh.indices:
        extractor.extract_index(int(i))


def _source_of(sampler):
    return sampler.source if isinstance(sampler, Sampler) else sampler


class MarchingCubes:
    """MarchingCubes::<Signed>::new(size) (src/marching_cubes.rs:46-50)."""

    def __init__(self, size, context=None):
        if size < 1:
            raise ValueError("size must be at least 1")
        self.size = size
        self.context = context

    def extract(self, sampler, extractor):
        ctx = self.context or default_context()
        source = _source_of(sampler)
        info = ctx.mc_extract(source, self.size, normals=getattr(extractor, "with_normals", False))
        _replay(extractor, ctx.download(info))


class MinimiseQEF:
    """Feature placement by QEF minimisation (src/feature/qef.rs:23-68)."""
    code = 0


class ParticleBasedMinimisation:
    """Feature placement by particle descent (src/feature/particle_minimisation.rs:25-72)."""
    code = 1


class DualContouring:
    """DualContouring::new(size, placer) (src/dual_contouring.rs:51-56)."""

    def __init__(self, size, place_feature=None, context=None):
        if size < 1:
            raise ValueError("size must be at least 1")
        self.size = size
        self.placer = (place_feature or MinimiseQEF()).code
        self.context = context

    def extract(self, sampler, extractor):
        ctx = self.context or default_context()
        info = ctx.dc_extract(_source_of(sampler), self.size, self.placer,
                              normals=getattr(extractor, "with_normals", False))
        _replay(extractor, ctx.download(info))


class LinearHashedMarchingCubes:
    """LinearHashedMarchingCubes::new(max_depth) (src/linear_hashed_marching_cubes.rs:51-53)."""

    def __init__(self, max_depth, context=None):
        self.max_depth = max_depth
        self.context = context

    def extract(self, sampler, extractor):
        ctx = self.context or default_context()
        info = ctx.lhmc_extract(_source_of(sampler), self.max_depth,
                                normals=getattr(extractor, "with_normals", False))
        _replay(extractor, ctx.download(info))


class ExtendedMarchingCubes:
    """ExtendedMarchingCubes::new(size) (src/extended_marching_cubes.rs:51-55)."""

    def __init__(self, size, context=None):
        if size < 1:
            raise ValueError("size must be at least 1")
        self.size = size
        self.context = context

    def extract(self, sampler, extractor):
        ctx = self.context or default_context()
        info, _ = ctx.emc_extract(_source_of(sampler), self.size, normals=getattr(extractor, "with_normals", False))
        _replay(extractor, ctx.download(info))


class PointCloud:
    """PointCloud::<Signed>::new(size) (src/point_cloud.rs:38-48)."""

    def __init__(self, size, context=None):
        self.size = size
        self.context = context

    def extract(self, sampler, extractor):
        ctx = self.context or default_context()
        info = ctx.point_cloud_extract(_source_of(sampler), self.size,
                                       normals=getattr(extractor, "with_normals", False))
        _replay(extractor, ctx.download(info))
