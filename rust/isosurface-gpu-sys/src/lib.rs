//! Raw FFI declarations of the GB300 isosurface extraction library, one per
//! function of `include/isosurface_gpu.h`, in the header's order.  Status
//! codes, flags and structures mirror the header; the safe wrappers that keep
//! the reference crate's `extract` signatures live in the crate's `gpu`
//! module (rust/isosurface/src/gpu).
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub type IsoStatus = c_int;

pub const ISO_OK: IsoStatus = 0;
pub const ISO_ERR_INVALID_ARG: IsoStatus = 1;
pub const ISO_ERR_CAPACITY: IsoStatus = 2;
pub const ISO_ERR_CUDA: IsoStatus = 3;
pub const ISO_ERR_TIMEOUT: IsoStatus = 4;
pub const ISO_ERR_BAD_PROGRAM: IsoStatus = 5;
pub const ISO_ERR_NO_DEVICE: IsoStatus = 6;
pub const ISO_ERR_OUT_OF_MEMORY: IsoStatus = 7;
pub const ISO_ERR_TOO_LARGE: IsoStatus = 8;
pub const ISO_ERR_UNSUPPORTED: IsoStatus = 9;

pub const ISO_STAGE_SAMPLE: usize = 0;
pub const ISO_STAGE_CLASSIFY: usize = 1;
pub const ISO_STAGE_EMIT: usize = 2;
pub const ISO_STAGE_SIGNS: usize = 3;
pub const ISO_STAGE_PLACE: usize = 4;
pub const ISO_STAGE_OCTREE: usize = 5;
pub const ISO_STAGE_MLP: usize = 6;
pub const ISO_STAGE_OTHER: usize = 7;
pub const ISO_STAGE_COUNT: usize = 8;

pub const ISO_FLAG_KEYS: u32 = 1;
pub const ISO_FLAG_NORMALS: u32 = 2;
pub const ISO_FLAG_HOST_COPY: u32 = 4;
pub const ISO_PLACER_MINIMISE_QEF: u32 = 0;
pub const ISO_PLACER_PARTICLES: u32 = 1;
pub const ISO_BATCH_GRAPH: u32 = 1;
pub const ISO_SPLAT_MIRROR_EDGES: u32 = 1;
pub const ISO_SURROGATE_EXACT_COARSE: u32 = 1;
pub const ISO_SURROGATE_WITNESS: u32 = 2;

/// Opaque library objects (only ever used behind pointers).
#[repr(C)]
pub struct IsoCtx {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct IsoProgram {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct IsoBatch {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct IsoMlp {
    _opaque: [u8; 0],
}

#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct IsoMeshInfo {
    pub num_vertices: u64,
    pub num_triangles: u64,
    pub num_cells: u64,
}

#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct IsoChunkDesc {
    pub program: u32,
    pub size: u32,
}

#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct IsoSurrogateStats {
    pub coarse_points: u64,
    pub band_points: u64,
    pub total_points: u64,
}

#[repr(C)]
#[derive(Debug, Default, Clone, Copy)]
pub struct IsoMeshDistanceResult {
    pub mean_ab: f64,
    pub mean_ba: f64,
    pub max_ab: f64,
    pub max_ba: f64,
    pub capped: u64,
}

extern "C" {
    pub fn iso_status_str(s: IsoStatus) -> *const c_char;
    pub fn iso_ctx_last_error(ctx: *const IsoCtx) -> *const c_char;
    pub fn iso_ctx_create(device: c_int, out: *mut *mut IsoCtx) -> IsoStatus;
    pub fn iso_ctx_destroy(ctx: *mut IsoCtx) -> IsoStatus;
    pub fn iso_ctx_get_stream(ctx: *mut IsoCtx, stream: *mut *mut c_void) -> IsoStatus;
    pub fn iso_ctx_set_stream(ctx: *mut IsoCtx, stream: *mut c_void) -> IsoStatus;
    pub fn iso_ctx_kernel_launches(ctx: *const IsoCtx) -> u64;
    pub fn iso_debug_fail_allocation(ctx: *mut IsoCtx, after: i64) -> IsoStatus;
    pub fn iso_debug_scan_timeout(enable: c_int) -> IsoStatus;
    pub fn iso_ctx_enable_stage_timing(ctx: *mut IsoCtx, enable: c_int) -> IsoStatus;
    pub fn iso_ctx_stage_times(ctx: *mut IsoCtx, ms: *mut f64, launches: *mut u64) -> IsoStatus;
    pub fn iso_program_create(
        ctx: *mut IsoCtx,
        bytes: *const u8,
        len: usize,
        out: *mut *mut IsoProgram,
    ) -> IsoStatus;
    pub fn iso_program_destroy(prog: *mut IsoProgram) -> IsoStatus;
    pub fn iso_mesh_download(
        ctx: *mut IsoCtx,
        vertices: *mut f32,
        vertex_floats_cap: u64,
        indices: *mut u32,
        index_cap: u64,
        keys: *mut u64,
        key_cap: u64,
    ) -> IsoStatus;
    pub fn iso_mesh_device(
        ctx: *mut IsoCtx,
        vertices: *mut *const f32,
        indices: *mut *const u32,
        keys: *mut *const u64,
        info: *mut IsoMeshInfo,
    ) -> IsoStatus;
    pub fn iso_sample_grid(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        field: *mut f32,
        pitch: u64,
    ) -> IsoStatus;
    pub fn iso_sample_grid_near(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        field: *mut f32,
        pitch: u64,
        bits: *mut u32,
    ) -> IsoStatus;
    pub fn iso_program_lipschitz(prog: *const IsoProgram, lip: *mut f32) -> IsoStatus;
    pub fn iso_program_compiled(prog: *const IsoProgram, compiled: *mut c_int) -> IsoStatus;
    pub fn iso_jit_enable(enable: c_int) -> IsoStatus;
    pub fn iso_program_source(
        bytes: *const u8,
        len: usize,
        out: *mut c_char,
        cap: usize,
        needed: *mut usize,
    ) -> IsoStatus;
    pub fn iso_mc_extract(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        flags: u32,
        info: *mut IsoMeshInfo,
    ) -> IsoStatus;
    pub fn iso_mc_extract_host(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        flags: u32,
        vertices: *mut f32,
        vertex_floats: u64,
        indices: *mut u32,
        index_count: u64,
        info: *mut IsoMeshInfo,
    ) -> IsoStatus;
    pub fn iso_host_register(p: *mut c_void, bytes: u64) -> IsoStatus;
    pub fn iso_host_unregister(p: *mut c_void) -> IsoStatus;
    pub fn iso_mc_extract_field(
        ctx: *mut IsoCtx,
        field: *const f32,
        nx: u32,
        ny: u32,
        nz: u32,
        pitch: u64,
        flags: u32,
        info: *mut IsoMeshInfo,
    ) -> IsoStatus;
    pub fn iso_mc_extract_field_noalloc(
        field: *const f32,
        nx: u32,
        ny: u32,
        nz: u32,
        pitch: u64,
        vertices: *mut f32,
        vertex_cap: u64,
        indices: *mut u32,
        triangle_cap: u64,
        stream: *mut c_void,
        info: *mut IsoMeshInfo,
    ) -> IsoStatus;
    pub fn iso_mc_extract_slab(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        z_begin: u32,
        z_end: u32,
        flags: u32,
        info: *mut IsoMeshInfo,
        halo_vertices: *mut u64,
        halo_triangles: *mut u64,
    ) -> IsoStatus;
    pub fn iso_mc_cases(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        cases_host: *mut u8,
    ) -> IsoStatus;
    pub fn iso_dc_extract(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        placer: u32,
        flags: u32,
        info: *mut IsoMeshInfo,
    ) -> IsoStatus;
    pub fn iso_dc_extract_slab(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        placer: u32,
        z_begin: u32,
        z_end: u32,
        flags: u32,
        info: *mut IsoMeshInfo,
        halo_vertices: *mut u64,
        halo_triangles: *mut u64,
    ) -> IsoStatus;
    pub fn iso_lhmc_extract(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        max_depth: u32,
        flags: u32,
        info: *mut IsoMeshInfo,
    ) -> IsoStatus;
    pub fn iso_lhmc_stale_corners(ctx: *const IsoCtx) -> u64;
    pub fn iso_batch_create(
        ctx: *mut IsoCtx,
        programs: *const *const IsoProgram,
        nprograms: u32,
        chunks: *const IsoChunkDesc,
        nchunks: u32,
        out: *mut *mut IsoBatch,
    ) -> IsoStatus;
    pub fn iso_batch_destroy(batch: *mut IsoBatch) -> IsoStatus;
    pub fn iso_batch_run(batch: *mut IsoBatch, flags: u32, info: *mut IsoMeshInfo) -> IsoStatus;
    pub fn iso_batch_run_per_chunk(batch: *mut IsoBatch, info: *mut IsoMeshInfo) -> IsoStatus;
    pub fn iso_batch_run_per_chunk_async(batch: *mut IsoBatch, info: *mut IsoMeshInfo) -> IsoStatus;
    pub fn iso_batch_extents(batch: *mut IsoBatch, extents: *mut u32) -> IsoStatus;
    pub fn iso_batch_set_slab(batch: *mut IsoBatch, size: u32, depth: u32) -> IsoStatus;
    pub fn iso_batch_autotune(batch: *mut IsoBatch, cache_path: *const c_char, chosen: *mut u32) -> IsoStatus;
    pub fn iso_mlp_create(ctx: *mut IsoCtx, seed: u64, out: *mut *mut IsoMlp) -> IsoStatus;
    pub fn iso_mlp_destroy(net: *mut IsoMlp) -> IsoStatus;
    pub fn iso_mlp_num_params() -> u64;
    pub fn iso_mlp_get_params(net: *mut IsoMlp, host: *mut f32) -> IsoStatus;
    pub fn iso_mlp_set_params(net: *mut IsoMlp, host: *const f32) -> IsoStatus;
    pub fn iso_mlp_forward(net: *mut IsoMlp, points: *const f32, n: u32, values: *mut f32) -> IsoStatus;
    pub fn iso_mlp_forward_bf16(net: *mut IsoMlp, points: *const f32, n: u32, values: *mut f32) -> IsoStatus;
    pub fn iso_mlp_loss_grad(
        net: *mut IsoMlp,
        points: *const f32,
        targets: *const f32,
        n: u32,
        clamp_d: f32,
        loss: *mut f32,
        grad: *mut f32,
    ) -> IsoStatus;
    pub fn iso_mlp_make_dataset(
        net: *mut IsoMlp,
        exact: *const IsoProgram,
        n: u32,
        lo: f32,
        hi: f32,
        seed: u64,
    ) -> IsoStatus;
    pub fn iso_mlp_train(
        net: *mut IsoMlp,
        steps: u32,
        batch: u32,
        lr: f32,
        clamp_d: f32,
        seed: u64,
        history: *mut f32,
    ) -> IsoStatus;
    pub fn iso_mlp_save(net: *mut IsoMlp, path: *const c_char) -> IsoStatus;
    pub fn iso_mlp_load(net: *mut IsoMlp, path: *const c_char) -> IsoStatus;
    pub fn iso_mlp_checkpoint_info(path: *const c_char, nparams: *mut u64, step: *mut u64) -> IsoStatus;
    pub fn iso_surrogate_field(
        ctx: *mut IsoCtx,
        net: *mut IsoMlp,
        exact: *const IsoProgram,
        size: u32,
        coarse_step: u32,
        band_cells: f32,
        field: *mut f32,
        pitch: u64,
        stats: *mut IsoSurrogateStats,
    ) -> IsoStatus;
    pub fn iso_surrogate_field_ex(
        ctx: *mut IsoCtx,
        net: *mut IsoMlp,
        exact: *const IsoProgram,
        size: u32,
        coarse_step: u32,
        band_cells: f32,
        flags: u32,
        field: *mut f32,
        pitch: u64,
        stats: *mut IsoSurrogateStats,
        flagged_primitives: *mut u64,
    ) -> IsoStatus;
    pub fn iso_surrogate_extract(
        ctx: *mut IsoCtx,
        net: *mut IsoMlp,
        exact: *const IsoProgram,
        size: u32,
        coarse_step: u32,
        band_cells: f32,
        flags: u32,
        stats: *mut IsoSurrogateStats,
        info: *mut IsoMeshInfo,
    ) -> IsoStatus;
    pub fn iso_mesh_distance(
        ctx: *mut IsoCtx,
        a: *const f32,
        na: u64,
        b: *const f32,
        nb: u64,
        bucket: f32,
        max_rings: u32,
        out: *mut IsoMeshDistanceResult,
    ) -> IsoStatus;
    pub fn iso_field_case_disagreement(
        ctx: *mut IsoCtx,
        fa: *const f32,
        fb: *const f32,
        nx: u32,
        ny: u32,
        nz: u32,
        pitch: u64,
        cells: *mut u64,
    ) -> IsoStatus;
    pub fn iso_emc_extract(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        flags: u32,
        info: *mut IsoMeshInfo,
        flips: *mut u64,
    ) -> IsoStatus;
    pub fn iso_point_cloud_extract(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        size: u32,
        flags: u32,
        info: *mut IsoMeshInfo,
    ) -> IsoStatus;
    pub fn iso_point_splat_render(
        ctx: *mut IsoCtx,
        view_proj: *const f32,
        view_proj_inverse: *const f32,
        width: u32,
        height: u32,
        voxel_half: f32,
        clear_rgb: *const f32,
        rgba: *mut f32,
    ) -> IsoStatus;
    pub fn iso_point_splat_render_ex(
        ctx: *mut IsoCtx,
        view_proj: *const f32,
        view_proj_inverse: *const f32,
        width: u32,
        height: u32,
        voxel_half: f32,
        clear_rgb: *const f32,
        flags: u32,
        rgba: *mut f32,
    ) -> IsoStatus;
    pub fn iso_sample_points(
        ctx: *mut IsoCtx,
        prog: *const IsoProgram,
        points: *const f32,
        n: u64,
        values: *mut f32,
        normals: *mut f32,
    ) -> IsoStatus;
}
