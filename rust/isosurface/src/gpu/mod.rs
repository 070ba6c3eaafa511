//! The GPU path of the crate's extractors, on the GB300 library
//! (libisosurface_gpu, bound by the isosurface-gpu-sys crate).
//!
//! Added to the crate under a `gpu` feature; each algorithm's `extract`
//! keeps its signature, gains a `LowerToDevice` bound on the source, and
//! forwards here in one line (`MarchingCubes::extract` becomes
//! `crate::gpu::marching_cubes(self.size, source, extractor)`, and likewise):
//!
//! * `MarchingCubes::extract`            (src/marching_cubes.rs:59-82)
//! * `DualContouring::extract`           (src/dual_contouring.rs:65-105)
//! * `LinearHashedMarchingCubes::extract`(src/linear_hashed_marching_cubes.rs:62-84)
//! * `PointCloud::extract`               (src/point_cloud.rs:50-63)
//! * `ExtendedMarchingCubes::extract`    (src/extended_marching_cubes.rs:64-93)
//!
//! The mesh is replayed into the caller's `Extractor` (src/extractor.rs:17-20)
//! in the library's order, which for MarchingCubes, DualContouring,
//! PointCloud and ExtendedMarchingCubes is the CPU path's order byte for
//! byte.  There is no CPU fallback: a library error panics with the
//! library's status name, as the reference panics on its own failures
//! (src/mesh.rs:196,209).
//!
//! Not compiled here (no Rust toolchain on the machines this library was
//! built on).

mod lower;

pub use self::lower::{LowerToDevice, ProgramBuilder};

use crate::{extractor::Extractor, feature::{MinimiseQEF, ParticleBasedMinimisation}, math::Vec3};
use isosurface_gpu_sys as sys;
use std::cell::RefCell;
use std::ffi::CStr;
use std::ptr;

fn check(status: sys::IsoStatus) {
    if status != sys::ISO_OK {
        let name = unsafe { CStr::from_ptr(sys::iso_status_str(status)) };
        panic!("isosurface GPU library: {}", name.to_string_lossy());
    }
}

/// One library context (CUDA stream, device buffers, last mesh) per host
/// thread, on device 0 unless ISOSURFACE_GPU_DEVICE names another.
struct Context {
    raw: *mut sys::IsoCtx,
}

impl Context {
    fn new() -> Self {
        let device = std::env::var("ISOSURFACE_GPU_DEVICE").ok().and_then(|s| s.parse().ok()).unwrap_or(0);
        let mut raw = ptr::null_mut();
        check(unsafe { sys::iso_ctx_create(device, &mut raw) });
        Context { raw }
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        unsafe { sys::iso_ctx_destroy(self.raw) };
    }
}

thread_local! {
    static CONTEXT: RefCell<Option<Context>> = RefCell::new(None);
}

fn with_context<R>(f: impl FnOnce(*mut sys::IsoCtx) -> R) -> R {
    CONTEXT.with(|c| {
        let mut c = c.borrow_mut();
        let ctx = c.get_or_insert_with(Context::new);
        f(ctx.raw)
    })
}

/// A source's program, uploaded for one extraction and freed after it.
struct Program {
    raw: *mut sys::IsoProgram,
}

impl Program {
    fn new<S: LowerToDevice + ?Sized>(ctx: *mut sys::IsoCtx, source: &S) -> Self {
        let bytes = source.program_bytes();
        let mut raw = ptr::null_mut();
        check(unsafe { sys::iso_program_create(ctx, bytes.as_ptr(), bytes.len(), &mut raw) });
        Program { raw }
    }
}

impl Drop for Program {
    fn drop(&mut self) {
        unsafe { sys::iso_program_destroy(self.raw) };
    }
}

/// Copies the context's last mesh to the host and hands it to the extractor:
/// every vertex in order, then every index (the order
/// MeshTopology::extract_indices uses, src/mesh.rs:91-100).
fn replay<E: Extractor>(ctx: *mut sys::IsoCtx, info: &sys::IsoMeshInfo, with_indices: bool, extractor: &mut E) {
    let nv = info.num_vertices as usize;
    let ni = if with_indices { 3 * info.num_triangles as usize } else { 0 };
    let mut v = vec![0f32; 3 * nv];
    let mut i = vec![0u32; ni];
    check(unsafe {
        sys::iso_mesh_download(
            ctx,
            v.as_mut_ptr(),
            v.len() as u64,
            if ni > 0 { i.as_mut_ptr() } else { ptr::null_mut() },
            i.len() as u64,
            ptr::null_mut(),
            0,
        )
    });
    for p in v.chunks_exact(3) {
        extractor.extract_vertex(Vec3::new(p[0], p[1], p[2]));
    }
    for &ix in &i {
        extractor.extract_index(ix as usize);
    }
}

/// MarchingCubes::new(size).extract(source, extractor).
pub fn marching_cubes<S: LowerToDevice, E: Extractor>(size: usize, source: &S, extractor: &mut E) {
    with_context(|ctx| {
        let prog = Program::new(ctx, source);
        let mut info = sys::IsoMeshInfo::default();
        check(unsafe { sys::iso_mc_extract(ctx, prog.raw, size as u32, 0, &mut info) });
        replay(ctx, &info, true, extractor);
    })
}

/// MarchingCubes straight into an IndexedVertices pair of vectors: the
/// library writes them itself (kernels store into them as they run when the
/// caller keeps them page-locked with `iso_host_register`).
pub fn marching_cubes_into<S: LowerToDevice>(size: usize, source: &S, vertices: &mut Vec<f32>,
                                              indices: &mut Vec<u32>) {
    with_context(|ctx| {
        let prog = Program::new(ctx, source);
        vertices.clear();
        indices.clear();
        let mut info = sys::IsoMeshInfo::default();
        let st = unsafe {
            sys::iso_mc_extract_host(ctx, prog.raw, size as u32, 0, vertices.as_mut_ptr(),
                                     vertices.capacity() as u64, indices.as_mut_ptr(),
                                     indices.capacity() as u64, &mut info)
        };
        let (nv, ni) = (3 * info.num_vertices as usize, 3 * info.num_triangles as usize);
        if st == sys::ISO_ERR_CAPACITY {
            // the mesh stays on the device: grow the vectors and copy it
            vertices.reserve(nv);
            indices.reserve(ni);
            check(unsafe {
                sys::iso_mesh_download(ctx, vertices.as_mut_ptr(), vertices.capacity() as u64,
                                       indices.as_mut_ptr(), indices.capacity() as u64, ptr::null_mut(), 0)
            });
        } else {
            check(st);
        }
        unsafe {
            vertices.set_len(nv);
            indices.set_len(ni);
        }
    })
}

/// The feature placers the device implements.
pub trait DevicePlacer {
    const PLACER: u32;
}

impl DevicePlacer for MinimiseQEF {
    const PLACER: u32 = sys::ISO_PLACER_MINIMISE_QEF;
}

impl DevicePlacer for ParticleBasedMinimisation {
    const PLACER: u32 = sys::ISO_PLACER_PARTICLES;
}

/// DualContouring::new(size, placer).extract(source, extractor).
pub fn dual_contouring<P: DevicePlacer, S: LowerToDevice, E: Extractor>(size: usize, source: &S,
                                                                          extractor: &mut E) {
    with_context(|ctx| {
        let prog = Program::new(ctx, source);
        let mut info = sys::IsoMeshInfo::default();
        check(unsafe { sys::iso_dc_extract(ctx, prog.raw, size as u32, P::PLACER, 0, &mut info) });
        replay(ctx, &info, true, extractor);
    })
}

/// LinearHashedMarchingCubes::new(max_depth).extract(source, extractor).  The
/// reference walks a HashMap, so only its triangle set is defined; the
/// library's order is deterministic.
pub fn linear_hashed_marching_cubes<S: LowerToDevice, E: Extractor>(max_depth: usize, source: &S,
                                                                      extractor: &mut E) {
    with_context(|ctx| {
        let prog = Program::new(ctx, source);
        let mut info = sys::IsoMeshInfo::default();
        check(unsafe { sys::iso_lhmc_extract(ctx, prog.raw, max_depth as u32, 0, &mut info) });
        replay(ctx, &info, true, extractor);
    })
}

/// PointCloud::new(size).extract(source, extractor): vertices only.
pub fn point_cloud<S: LowerToDevice, E: Extractor>(size: usize, source: &S, extractor: &mut E) {
    with_context(|ctx| {
        let prog = Program::new(ctx, source);
        let mut info = sys::IsoMeshInfo::default();
        check(unsafe { sys::iso_point_cloud_extract(ctx, prog.raw, size as u32, 0, &mut info) });
        replay(ctx, &info, false, extractor);
    })
}

/// ExtendedMarchingCubes::new(size).extract(source, extractor).  Sources
/// whose ops have no Directed form in the reference are refused by the
/// library (ISO_ERR_UNSUPPORTED).
pub fn extended_marching_cubes<S: LowerToDevice, E: Extractor>(size: usize, source: &S, extractor: &mut E) {
    with_context(|ctx| {
        let prog = Program::new(ctx, source);
        let mut info = sys::IsoMeshInfo::default();
        let mut flips = 0u64;
        check(unsafe { sys::iso_emc_extract(ctx, prog.raw, size as u32, 0, &mut info, &mut flips) });
        replay(ctx, &info, true, extractor);
    })
}
