"""ctypes binding of the C ABI in include/isosurface_gpu.h.

The shared library is the in-tree build (isosurface_gb300/_build/libisosurface_gpu.so,
made by isosurface_gb300/build.py).  There is no CPU fallback: if the library
is missing or no CUDA device is visible, every entry point raises.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libisosurface_gpu.so")

ISO_OK = 0
STATUS = {
    0: "ISO_OK", 1: "ISO_ERR_INVALID_ARG", 2: "ISO_ERR_CAPACITY", 3: "ISO_ERR_CUDA", 4: "ISO_ERR_TIMEOUT",
    5: "ISO_ERR_BAD_PROGRAM", 6: "ISO_ERR_NO_DEVICE", 7: "ISO_ERR_OUT_OF_MEMORY", 8: "ISO_ERR_TOO_LARGE",
    9: "ISO_ERR_UNSUPPORTED",
}
ISO_FLAG_KEYS = 1
ISO_FLAG_NORMALS = 2
ISO_FLAG_HOST_COPY = 4
ISO_SURROGATE_EXACT_COARSE = 1
ISO_SURROGATE_WITNESS = 2


class IsoError(RuntimeError):
    def __init__(self, status, message=""):
        self.status = status
        super().__init__("%s%s" % (STATUS.get(status, "ISO_ERR_%d" % status), (": " + message) if message else ""))


class MeshInfo(ctypes.Structure):
    _fields_ = [("num_vertices", ctypes.c_uint64), ("num_triangles", ctypes.c_uint64),
                ("num_cells", ctypes.c_uint64)]


class SurrogateStats(ctypes.Structure):
    _fields_ = [("coarse_points", ctypes.c_uint64), ("band_points", ctypes.c_uint64),
                ("total_points", ctypes.c_uint64)]


class MeshDistance(ctypes.Structure):
    _fields_ = [("mean_ab", ctypes.c_double), ("mean_ba", ctypes.c_double), ("max_ab", ctypes.c_double),
                ("max_ba", ctypes.c_double), ("capped", ctypes.c_uint64)]


class ChunkDesc(ctypes.Structure):
    _fields_ = [("program", ctypes.c_uint32), ("size", ctypes.c_uint32)]


ISO_BATCH_GRAPH = 1

_lib = None

vp = ctypes.c_void_p
u8p = ctypes.POINTER(ctypes.c_uint8)
f32p = ctypes.POINTER(ctypes.c_float)
u32p = ctypes.POINTER(ctypes.c_uint32)
u64p = ctypes.POINTER(ctypes.c_uint64)
i32 = ctypes.c_int
u32 = ctypes.c_uint32
u64 = ctypes.c_uint64

# name -> (restype, argtypes); every symbol include/isosurface_gpu.h declares
SIGNATURES = {
    "iso_status_str": (ctypes.c_char_p, [i32]),
    "iso_ctx_last_error": (ctypes.c_char_p, [vp]),
    "iso_ctx_create": (i32, [i32, ctypes.POINTER(vp)]),
    "iso_ctx_destroy": (i32, [vp]),
    "iso_ctx_get_stream": (i32, [vp, ctypes.POINTER(vp)]),
    "iso_ctx_set_stream": (i32, [vp, vp]),
    "iso_ctx_kernel_launches": (u64, [vp]),
    "iso_debug_fail_allocation": (i32, [vp, ctypes.c_int64]),
    "iso_debug_scan_timeout": (i32, [ctypes.c_int]),
    "iso_ctx_enable_stage_timing": (i32, [vp, i32]),
    "iso_ctx_stage_times": (i32, [vp, ctypes.POINTER(ctypes.c_double), u64p]),
    "iso_program_create": (i32, [vp, ctypes.c_char_p, ctypes.c_size_t, ctypes.POINTER(vp)]),
    "iso_program_destroy": (i32, [vp]),
    "iso_mesh_download": (i32, [vp, f32p, u64, u32p, u64, u64p, u64]),
    "iso_mesh_device": (i32, [vp, ctypes.POINTER(vp), ctypes.POINTER(vp), ctypes.POINTER(vp),
                              ctypes.POINTER(MeshInfo)]),
    "iso_sample_grid": (i32, [vp, vp, u32, vp, u64]),
    "iso_sample_grid_near": (i32, [vp, vp, u32, vp, u64, vp]),
    "iso_program_lipschitz": (i32, [vp, ctypes.POINTER(ctypes.c_float)]),
    "iso_program_compiled": (i32, [vp, ctypes.POINTER(ctypes.c_int)]),
    "iso_jit_enable": (i32, [ctypes.c_int]),
    "iso_program_source": (i32, [ctypes.c_char_p, ctypes.c_size_t, ctypes.c_char_p, ctypes.c_size_t,
                                 ctypes.POINTER(ctypes.c_size_t)]),
    "iso_mc_extract": (i32, [vp, vp, u32, u32, ctypes.POINTER(MeshInfo)]),
    "iso_mc_extract_host": (i32, [vp, vp, u32, u32, vp, u64, vp, u64, ctypes.POINTER(MeshInfo)]),
    "iso_point_splat_render": (i32, [vp, vp, vp, u32, u32, ctypes.c_float, vp, vp]),
    "iso_point_splat_render_ex": (i32, [vp, vp, vp, u32, u32, ctypes.c_float, vp, u32, vp]),
    "iso_host_register": (i32, [vp, u64]),
    "iso_host_unregister": (i32, [vp]),
    "iso_mc_extract_field": (i32, [vp, vp, u32, u32, u32, u64, u32, ctypes.POINTER(MeshInfo)]),
    "iso_mc_extract_field_noalloc": (i32, [vp, u32, u32, u32, u64, vp, u64, vp, u64, vp, ctypes.POINTER(MeshInfo)]),
    "iso_mc_extract_slab": (i32, [vp, vp, u32, u32, u32, u32, ctypes.POINTER(MeshInfo), ctypes.POINTER(u64),
                                  ctypes.POINTER(u64)]),
    "iso_mc_cases": (i32, [vp, vp, u32, u8p]),
    "iso_point_cloud_extract": (i32, [vp, vp, u32, u32, ctypes.POINTER(MeshInfo)]),
    "iso_emc_extract": (i32, [vp, vp, u32, u32, ctypes.POINTER(MeshInfo), ctypes.POINTER(ctypes.c_uint64)]),
    "iso_dc_extract": (i32, [vp, vp, u32, u32, u32, ctypes.POINTER(MeshInfo)]),
    "iso_dc_extract_slab": (i32, [vp, vp, u32, u32, u32, u32, u32, ctypes.POINTER(MeshInfo), ctypes.POINTER(u64),
                                  ctypes.POINTER(u64)]),
    "iso_lhmc_extract": (i32, [vp, vp, u32, u32, ctypes.POINTER(MeshInfo)]),
    "iso_lhmc_stale_corners": (u64, [vp]),
    "iso_batch_create": (i32, [vp, ctypes.POINTER(vp), u32, ctypes.POINTER(ChunkDesc), u32, ctypes.POINTER(vp)]),
    "iso_batch_destroy": (i32, [vp]),
    "iso_batch_run": (i32, [vp, u32, ctypes.POINTER(MeshInfo)]),
    "iso_batch_run_per_chunk": (i32, [vp, ctypes.POINTER(MeshInfo)]),
    "iso_batch_run_per_chunk_async": (i32, [vp, ctypes.POINTER(MeshInfo)]),
    "iso_batch_extents": (i32, [vp, u32p]),
    "iso_batch_set_slab": (i32, [vp, u32, u32]),
    "iso_batch_autotune": (i32, [vp, ctypes.c_char_p, u32p]),
    "iso_mlp_create": (i32, [vp, u64, ctypes.POINTER(vp)]),
    "iso_mlp_destroy": (i32, [vp]),
    "iso_mlp_num_params": (u64, []),
    "iso_mlp_get_params": (i32, [vp, f32p]),
    "iso_mlp_set_params": (i32, [vp, f32p]),
    "iso_mlp_forward": (i32, [vp, f32p, u32, f32p]),
    "iso_mlp_forward_bf16": (i32, [vp, f32p, u32, f32p]),
    "iso_mlp_loss_grad": (i32, [vp, f32p, f32p, u32, ctypes.c_float, f32p, f32p]),
    "iso_mlp_make_dataset": (i32, [vp, vp, u32, ctypes.c_float, ctypes.c_float, u64]),
    "iso_mlp_train": (i32, [vp, u32, u32, ctypes.c_float, ctypes.c_float, u64, f32p]),
    "iso_mlp_save": (i32, [vp, ctypes.c_char_p]),
    "iso_mlp_load": (i32, [vp, ctypes.c_char_p]),
    "iso_mlp_checkpoint_info": (i32, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64)]),
    "iso_surrogate_field": (i32, [vp, vp, vp, u32, u32, ctypes.c_float, vp, u64, ctypes.POINTER(SurrogateStats)]),
    "iso_surrogate_field_ex": (i32, [vp, vp, vp, u32, u32, ctypes.c_float, u32, vp, u64,
                                     ctypes.POINTER(SurrogateStats), ctypes.POINTER(u64)]),
    "iso_surrogate_extract": (i32, [vp, vp, vp, u32, u32, ctypes.c_float, u32, ctypes.POINTER(SurrogateStats),
                                    ctypes.POINTER(MeshInfo)]),
    "iso_mesh_distance": (i32, [vp, f32p, u64, f32p, u64, ctypes.c_float, u32, ctypes.POINTER(MeshDistance)]),
    "iso_field_case_disagreement": (i32, [vp, vp, vp, u32, u32, u32, u64, u64p]),
    "iso_sample_points": (i32, [vp, vp, f32p, u64, f32p, f32p]),
}


def lib():
    """Load the library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise IsoError(6, "CUDA library not built: run isosurface_gb300/build.py (%s missing)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status, ctx=None):
    if status != ISO_OK:
        msg = ""
        if ctx:
            raw = lib().iso_ctx_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise IsoError(status, msg)
