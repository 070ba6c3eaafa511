/*
 * isosurface_gpu.h -- C ABI of the GB300 isosurface extraction library.
 *
 * The library replaces the extraction hot path of swiftcoder/isosurface
 * (a Rust crate).  Each extraction entry point below stands in for one
 * reference call; the reference's Rust wrapper would bind these functions
 * through `extern "C"` and replay the resulting mesh into the caller's
 * Extractor, so the reference API
 *
 *     MarchingCubes::new(n).extract(&source, &mut extractor)
 *
 * stays as it is.  Plain pointers and sizes only; no CUDA, torch or C++ types
 * cross this boundary (CUDA streams are passed as `void*`).
 *
 * Threading: one iso_ctx per host thread; calls on one context are not
 * thread-safe.  Every function returns an iso_status and never aborts.
 *
 * Output convention (IndexedVertices, src/extractor.rs:72-93): vertices are
 * f32 x,y,z triples in the reference's [0,1]^3 sample frame, indices are u32
 * triangles.  For MarchingCubes and DualContouring the library produces the
 * vertex and index buffers that the reference produces, in the same order.
 * LinearHashedMarchingCubes walks a HashMap in RandomState order in the
 * reference, so only its triangle set is defined; the library emits it in a
 * deterministic order.
 */
#ifndef ISOSURFACE_GPU_H
#define ISOSURFACE_GPU_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define ISO_API __attribute__((visibility("default")))
#else
#define ISO_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                              */
/* ------------------------------------------------------------------------ */
typedef int iso_status;
#define ISO_OK 0
#define ISO_ERR_INVALID_ARG 1   /* null pointer, size out of range, ...       */
#define ISO_ERR_CAPACITY 2      /* caller buffer too small; see *_required    */
#define ISO_ERR_CUDA 3          /* a CUDA runtime call failed                 */
#define ISO_ERR_TIMEOUT 4       /* a bounded device-side wait gave up         */
#define ISO_ERR_BAD_PROGRAM 5   /* source program failed validation           */
#define ISO_ERR_NO_DEVICE 6     /* no CUDA device / wrong device index        */
#define ISO_ERR_OUT_OF_MEMORY 7 /* device allocation failed                   */
#define ISO_ERR_TOO_LARGE 8     /* mesh does not fit u32 indices              */
#define ISO_ERR_UNSUPPORTED 9   /* source lacks what the call needs (normals) */

/* Human-readable name of a status code (static string). */
ISO_API const char* iso_status_str(iso_status s);

/* Message of the last error raised on this context ("" if none). */
ISO_API const char* iso_ctx_last_error(const struct iso_ctx* ctx);

/* ------------------------------------------------------------------------ */
/* Contexts                                                                  */
/* ------------------------------------------------------------------------ */
typedef struct iso_ctx iso_ctx;

/* Create a context on CUDA device `device`.  The context owns a CUDA stream,
 * its device work buffers (grown on demand and reused) and the device copy of
 * the last extracted mesh. */
ISO_API iso_status iso_ctx_create(int device, iso_ctx** out);
ISO_API iso_status iso_ctx_destroy(iso_ctx* ctx);

/* The cudaStream_t every kernel of this context is launched on. */
ISO_API iso_status iso_ctx_get_stream(iso_ctx* ctx, void** stream);

/* Launch on a caller-owned cudaStream_t instead (NULL restores the context's
 * own stream).  The caller keeps the stream alive while the context uses it. */
ISO_API iso_status iso_ctx_set_stream(iso_ctx* ctx, void* stream);

/* Number of kernels this context has launched since creation. */
ISO_API uint64_t iso_ctx_kernel_launches(const iso_ctx* ctx);

/* Fault injection for tests: of this context's next device-buffer
 * allocations, the one after `after` successful ones fails as a failed
 * cudaMalloc does (the buffer it was to replace is already released; the
 * call returns ISO_ERR_OUT_OF_MEMORY); the hook then switches itself off.
 * A negative `after` switches it off.  Nothing happens on the device. */
ISO_API iso_status iso_debug_fail_allocation(iso_ctx* ctx, int64_t after);

/* Test hook for the bounded device-side waits: while enabled, the
 * decoupled look-back scan of iso_mc_extract_field_noalloc runs with its
 * first block never publishing its status and the other blocks giving up
 * after 256 polls of a predecessor, so the call returns ISO_ERR_TIMEOUT
 * instead of waiting; the next call after disabling it extracts normally.
 * Process-wide (that entry point takes no context).  Nothing faults or
 * hangs: every wait is bounded either way. */
ISO_API iso_status iso_debug_scan_timeout(int enable);

/* Per-stage device timing: when enabled, every kernel the context launches is
 * bracketed by CUDA events on its stream.  iso_ctx_stage_times synchronises,
 * writes the accumulated milliseconds and launch counts of each stage
 * (ISO_STAGE_COUNT entries each) and resets them. */
#define ISO_STAGE_SAMPLE 0      /* grid sampler (field + sign bits)            */
#define ISO_STAGE_CLASSIFY 1    /* cell classification + count + scan          */
#define ISO_STAGE_EMIT 2        /* vertex / index emission                     */
#define ISO_STAGE_SIGNS 3       /* sign bits of a caller-supplied field        */
#define ISO_STAGE_PLACE 4       /* dual-contouring vertex placement            */
#define ISO_STAGE_OCTREE 5      /* octree build / dual-cube gather             */
#define ISO_STAGE_MLP 6         /* surrogate network                           */
#define ISO_STAGE_OTHER 7
#define ISO_STAGE_COUNT 8
ISO_API iso_status iso_ctx_enable_stage_timing(iso_ctx* ctx, int enable);
ISO_API iso_status iso_ctx_stage_times(iso_ctx* ctx, double* ms, uint64_t* launches);

/* ------------------------------------------------------------------------ */
/* Source programs                                                           */
/* ------------------------------------------------------------------------ */
/*
 * An implicit source (a Sampler over a Source tree: src/sampler.rs,
 * src/source.rs and the primitives under src/implicit/) is handed to the
 * library as a program:
 *
 *   u32 magic     = 0x314F5349 ("ISO1" little-endian)
 *   u32 n_ops
 *   u32 n_consts
 *   u32 flags     = 0
 *   u32 ops[n_ops]        op = word & 0xFF, a = word >> 8 (a constant index)
 *   f32 consts[n_consts]
 *
 * Ops run in postfix order over a value stack and a point stack; the point
 * stack starts with the sample point p.  Each point op opens a scope that
 * ends at its PT_POP and must leave one value.
 *
 *   0x01 PT_DOMAIN     k[a..a+6] = scale xyz, offset xyz  push q = p*scale + offset
 *   0x02 PT_TRANSLATE  k[a..a+3] = centre                 push q = p - centre
 *   0x03 PT_RIGID      k[a..a+12] = t xyz, M (row-major)  push q = M (p - t)
 *   0x04 PT_POP                                           end the innermost scope
 *   0x10 SPHERE        k[a]   = radius                    sphere.rs:35-63
 *   0x11 BOX           k[a..a+3] = half extent            rectangular_prism.rs:36-80
 *   0x12 CYLINDER      k[a..a+2] = radius, half length    cylinder.rs:41-85
 *   0x13 TORUS         k[a..a+2] = radius, tube radius    torus.rs:40-108
 *   0x20 UNION         min(a, b)                          csg.rs:35-51
 *   0x21 INTERSECTION  max(a, b)                          csg.rs:68-72
 *   0x22 DIFFERENCE    max(b, -a)  (b minus a)            csg.rs:96-100
 *   0x23 SMOOTH_UNION  k[a] = k; min(a,b) - h*h*k/4, h = max(k-|a-b|,0)/k
 *   0x30 SPHERE_SET    k[a] = n, k[a+1] = 0 hard / 1 smooth, k[a+2] = k,
 *                      then n x (cx, cy, cz, r): a left fold of UNION (or
 *                      SMOOTH_UNION) over spheres translated to their centres
 *   0x40 CD_BEGIN      k[a] = epsilon; normals of the scope up to the matching
 *   0x41 CD_END        CD_END by central differences (source.rs:52-95)
 *
 * Normals (HermiteSource::sample_normal, unnormalised): primitives as in the
 * reference; UNION takes the component-wise min of the operands' normals
 * (csg.rs:47-51); INTERSECTION, DIFFERENCE and SMOOTH_UNION (which have no
 * normal in the reference) take the normal of the operand that decides the
 * value; PT_RIGID rotates the normal back by M^T; PT_DOMAIN and PT_TRANSLATE
 * pass it through.
 */
typedef struct iso_program iso_program;

ISO_API iso_status iso_program_create(iso_ctx* ctx, const uint8_t* bytes, size_t len, iso_program** out);
ISO_API iso_status iso_program_destroy(iso_program* prog);

/* ------------------------------------------------------------------------ */
/* Mesh results                                                              */
/* ------------------------------------------------------------------------ */
typedef struct iso_mesh_info {
    uint64_t num_vertices;
    uint64_t num_triangles;
    uint64_t num_cells;       /* cells (or dual cubes / octree cubes) visited */
} iso_mesh_info;

/* Copy the context's last mesh to host buffers (pageable or pinned).
 * vertices: 3*num_vertices floats (6 with normals, x y z nx ny nz interleaved
 *           as IndexedInterleavedNormals, extractor.rs:97-127)
 * indices:  3*num_triangles u32
 * keys:     optional, 2 u64 per vertex: the vertex's dedup key (MC/DC: the
 *           lattice edge id of GridKey, index_cache.rs:48-61, in the second
 *           word 0; LHMC: the MortonKey pair, index_cache.rs:63-73)
 * Capacities are element counts; ISO_ERR_CAPACITY if any is short. */
ISO_API iso_status iso_mesh_download(iso_ctx* ctx, float* vertices, uint64_t vertex_floats_cap,
                             uint32_t* indices, uint64_t index_cap,
                             uint64_t* keys, uint64_t key_cap);

/* Device pointers of the context's last mesh (valid until the next
 * extraction on this context).  keys is NULL unless requested. */
ISO_API iso_status iso_mesh_device(iso_ctx* ctx, const float** vertices, const uint32_t** indices,
                           const uint64_t** keys, iso_mesh_info* info);

/* Extraction flags */
#define ISO_FLAG_KEYS 1u      /* also produce per-vertex dedup keys          */
#define ISO_FLAG_NORMALS 2u   /* IndexedInterleavedNormals: per-vertex source normal */
#define ISO_FLAG_HOST_COPY 4u /* iso_mc_extract_host: deliver by copy after the extraction */

/* ------------------------------------------------------------------------ */
/* Grid sampling (PrimalGrid, src/traversal/primal_grid.rs:39-89)            */
/* ------------------------------------------------------------------------ */
/* Sample the source at the points of MarchingCubes::new(size):
 * (x/(size-1), y/(size-1), z/(size-1)) in f32, x,y < size, z <= size
 * (the reference samples one layer past z = 1).  The field is written to
 * `field` (device memory, row pitch `pitch` floats >= size, x fastest, then
 * y, then z: size+1 layers of size rows). */
ISO_API iso_status iso_sample_grid(iso_ctx* ctx, const iso_program* prog, uint32_t size,
                           float* field, uint64_t pitch);
/* The same points sampled the way the extractors sample them: every sign
 * bit, but values only where marching cubes can read them.  `bits` (device
 * memory, ceil(size/32) words per row, rows as in `field`) receives bit x%32
 * of word x/32 set iff !(value > 0); `field` receives the value of at least
 * every sample within one lattice step's worth of value change of zero (the
 * ends of every edge whose signs differ), bit-identical to iso_sample_grid's;
 * other entries may be left unwritten.  Unions of spheres and programs with a
 * known Lipschitz bound (iso_program_lipschitz) skip the work far from the
 * surface. */
ISO_API iso_status iso_sample_grid_near(iso_ctx* ctx, const iso_program* prog, uint32_t size,
                                float* field, uint64_t pitch, uint32_t* bits);
/* A bound on the program value's Lipschitz constant with respect to the
 * sample point (how much the value can change per unit of distance), from
 * its primitives (exact distances) and point maps; 0 when the program has
 * none (culled sampling is then off). */
ISO_API iso_status iso_program_lipschitz(const iso_program* prog, float* lip);
/* Whether the extractors' sampling of this program runs a kernel compiled
 * for it (written out as straight-line code and compiled with NVRTC on first
 * use, cached per program contents; values bit-identical to the
 * interpreter's) rather than the interpreter: 1 or 0.  General programs
 * (no sphere set) are compiled while NVRTC is available and compilation is
 * enabled (iso_jit_enable, process-wide, default on); iso_sample_grid runs
 * every compiled program's full-field kernel, while the extractors sample a
 * flat union of translated primitives with the interpreter, which prunes
 * the primitives per sub-brick (0 here). */
ISO_API iso_status iso_program_compiled(const iso_program* prog, int* compiled);
ISO_API iso_status iso_jit_enable(int enable);
/* The CUDA C the library compiles for the program in `bytes` (host only: no
 * device or context needed), NUL-terminated into `out` (room for `cap`
 * bytes); `needed` receives its size.  `out` null: size only.
 * ISO_ERR_UNSUPPORTED for a program the library does not compile (sphere
 * sets). */
ISO_API iso_status iso_program_source(const uint8_t* bytes, size_t len, char* out, size_t cap, size_t* needed);

/* ------------------------------------------------------------------------ */
/* MarchingCubes (src/marching_cubes.rs:59-82)                               */
/* ------------------------------------------------------------------------ */
/* MarchingCubes::<Signed>::new(size).extract(&Sampler::new(&source), &mut e).
 * The mesh stays on the device in the context; `info` receives its size. */
ISO_API iso_status iso_mc_extract(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t flags,
                          iso_mesh_info* info);

/* MarchingCubes::<Signed>::new(size).extract(&Sampler::new(&source),
 * &mut IndexedVertices::new(&mut vertices, &mut indices)) into caller-owned
 * host buffers: `vertices` (room for vertex_floats floats: 3 per vertex, 6
 * with ISO_FLAG_NORMALS) and `indices` (room for index_count u32, 3 per
 * triangle).  When both are page-locked (cudaHostAlloc, cudaHostRegister)
 * and `indices` is 16-byte aligned, the extraction kernels write the mesh into
 * them as they produce it, so the transfer overlaps the extraction; any other
 * host memory receives an ordinary copy afterwards.  ISO_FLAG_HOST_COPY asks
 * for that copy (the DMA engines, no SM time) with page-locked buffers too:
 * a lone call finishes later, but calls on other contexts then overlap the
 * transfer with their own extraction in full.  The mesh also stays on
 * the device (iso_mesh_download, iso_mesh_device) and `info` receives its
 * size.  If either buffer is too small, neither is written and the call
 * returns ISO_ERR_CAPACITY (a caller can grow its buffers and call
 * iso_mesh_download).  Replaces the crate's extract into Vec<f32>/Vec<u32>
 * (src/marching_cubes.rs:59-82, src/extractor.rs:72-93). */
ISO_API iso_status iso_mc_extract_host(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t flags,
                               float* vertices, uint64_t vertex_floats, uint32_t* indices,
                               uint64_t index_count, iso_mesh_info* info);

/* Page-lock `bytes` of caller host memory at `p` (cudaHostRegister, mapped
 * and portable), so that iso_mc_extract_host can deliver into it directly;
 * for callers whose vectors come from an ordinary allocator.  The range stays
 * registered until iso_host_unregister(p).  ISO_ERR_INVALID_ARG for a null
 * or empty range or one that is already registered, ISO_ERR_CUDA otherwise. */
ISO_API iso_status iso_host_register(void* p, uint64_t bytes);
ISO_API iso_status iso_host_unregister(void* p);

/* Marching cubes over a caller-supplied device field laid out as
 * iso_sample_grid writes it (nx x ny x nz samples, row pitch `pitch` floats,
 * vertex positions (x/(nx-1)... ) as the reference computes them with
 * one_over_size = 1/(nx-1); nx == ny). */
ISO_API iso_status iso_mc_extract_field(iso_ctx* ctx, const float* field, uint32_t nx, uint32_t ny, uint32_t nz,
                                uint64_t pitch, uint32_t flags, iso_mesh_info* info);

/* Marching cubes over a caller-supplied device field that allocates nothing.
 *
 * No counterpart in the reference: it exists for callers that cannot call
 * cudaMalloc or cudaFree -- code whose GPU memory is owned by a host
 * application's own allocator or fixed budget, and per-frame loops (a
 * renderer's or game engine's remeshing step) that cannot absorb the implicit
 * device synchronisation and unbounded latency of those calls.  It needs no
 * iso_ctx (creating one allocates).
 *
 * Input and layout as iso_mc_extract_field, with nz <= 65536 (larger values
 * are ISO_ERR_INVALID_ARG).  The caller owns the outputs:
 * `vertices` (3 floats per vertex, room for vertex_cap vertices) and
 * `indices` (3 u32 per triangle, room for triangle_cap triangles), both
 * device memory; work is queued on `stream` (a cudaStream_t, NULL for the
 * default stream) and the call returns when it has finished.  The mesh equals
 * iso_mc_extract_field's.  `info` always receives the mesh size; when a
 * buffer is too small the call writes nothing and returns ISO_ERR_CAPACITY,
 * so a caller can size its buffers and call again.
 *
 * Scratch lives in a 32 MiB array of device memory inside the library, which
 * every GPU that loads the library keeps until the process exits.  A grid
 * needs about nx*ny*nz/8 + 9*ny*nz bytes of it; the largest cubic grid that
 * fits is 613 x 613 x 614 samples (MarchingCubes::new(613)), and grids whose
 * scratch would not fit are rejected with ISO_ERR_TOO_LARGE.  The first call on each device looks up that
 * array's device address.  All calls share the one array, so calls whose GPU work overlaps (other
 * streams or host threads) race and must be serialised by the caller. */
ISO_API iso_status iso_mc_extract_field_noalloc(const float* field, uint32_t nx, uint32_t ny, uint32_t nz,
                                                uint64_t pitch, float* vertices, uint64_t vertex_cap,
                                                uint32_t* indices, uint64_t triangle_cap, void* stream,
                                                iso_mesh_info* info);

/* One slab of a z-partition of MarchingCubes::new(size) across GPUs (the
 * reference is single-threaded and has no counterpart): the cell layers
 * [z_begin, z_end), 0 <= z_begin < z_end <= size.  The slab samples and
 * meshes one extra cell layer below it when z_begin > 0 (the halo layer
 * z_begin - 1, sampled by this GPU, so no field data crosses GPUs) and
 * leaves in the context the mesh of the layers [z_begin - halo, z_end) with
 * vertex positions (and, with ISO_FLAG_KEYS, keys) in the whole grid's
 * frame: its first *halo_vertices vertices and *halo_triangles triangles are
 * the halo layer's (both 0 when z_begin == 0).  The mesh of the whole grid is
 * the slabs' meshes in slab order with the halo parts dropped and the
 * indices moved by the slab's first vertex (one exchange of the slabs'
 * vertex counts): isosurface_gb300/slabs.py does that, byte-identical to
 * iso_mc_extract.  Synchronous. */
ISO_API iso_status iso_mc_extract_slab(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t z_begin,
                                       uint32_t z_end, uint32_t flags, iso_mesh_info* info, uint64_t* halo_vertices,
                                       uint64_t* halo_triangles);

/* Case index of every cell of MarchingCubes::new(size) (the bits of
 * classify_corners, marching_cubes_impl.rs:26-37) into host memory:
 * size x (size-1) x (size-1) bytes, traversal order (z, y, x). */
ISO_API iso_status iso_mc_cases(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint8_t* cases_host);

/* ------------------------------------------------------------------------ */
/* DualContouring (src/dual_contouring.rs:42-105)                             */
/* ------------------------------------------------------------------------ */
#define ISO_PLACER_MINIMISE_QEF 0u    /* MinimiseQEF, feature/qef.rs:23-68 */
#define ISO_PLACER_PARTICLES 1u       /* ParticleBasedMinimisation, feature/particle_minimisation.rs:25-72 */
/* DualContouring::new(size, placer).extract(&sampler, &mut e): one vertex per
 * primal cell (placed by `placer` in active cells, the cell centre elsewhere),
 * then marching cubes over the dual cubes (DualGrid, traversal/dual_grid.rs).
 * Needs a source with normals (HermiteSource); keys (ISO_FLAG_KEYS) are dual
 * lattice edge ids over the (size-1) x (size-1) x size dual vertices. */
ISO_API iso_status iso_dc_extract(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t placer,
                                  uint32_t flags, iso_mesh_info* info);
/* One slab of a z-partition of DualContouring::new(size, placer) across GPUs
 * (no reference counterpart): the dual cube layers [z_begin, z_end),
 * 0 <= z_begin < z_end <= size - 1, plus the halo cube layer below when
 * z_begin > 0, sampled, placed and meshed on this GPU from the primal sample
 * layers it needs (z_begin - halo .. z_end + 1), with positions and keys
 * (ISO_FLAG_KEYS) in the whole dual lattice's frame; *halo_vertices and
 * *halo_triangles count the halo layer's part, first in the mesh.  The
 * slabs assemble exactly as iso_mc_extract_slab's do, with the dual lattice's
 * size - 1 in place of the grid size (isosurface_gb300/slabs.py), into
 * iso_dc_extract's buffers byte for byte.  Synchronous. */
ISO_API iso_status iso_dc_extract_slab(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t placer,
                                       uint32_t z_begin, uint32_t z_end, uint32_t flags, iso_mesh_info* info,
                                       uint64_t* halo_vertices, uint64_t* halo_triangles);

/* ------------------------------------------------------------------------ */
/* LinearHashedMarchingCubes (src/linear_hashed_marching_cubes.rs:40-84)      */
/* ------------------------------------------------------------------------ */
/* LinearHashedMarchingCubes::new(max_depth).extract(&sampler, &mut e):
 * Morton-keyed octree (linear_hashed_octree.rs), refined where |f| is below
 * the node's half-diagonal, then marching cubes on the dual cubes of its
 * leaves (traversal/implicit_octree.rs) with MortonKey dedup.  max_depth <= 10.
 * The reference emits the mesh in HashMap order, so only the triangle set is
 * defined; keys (ISO_FLAG_KEYS) are the MortonKey pair of each vertex. */
ISO_API iso_status iso_lhmc_extract(iso_ctx* ctx, const iso_program* prog, uint32_t max_depth, uint32_t flags,
                                    iso_mesh_info* info);

/* Dual-cube corners of the last iso_lhmc_extract call on `ctx` whose parent
 * walk found no node.  The reference keeps the previous primal vertex's
 * corner data there (traversal/implicit_octree.rs:84-95), which depends on its
 * HashMap order; 0 means the extraction involved no such corner.  No input
 * reaches that case (every level-2 node exists and every primal vertex lies
 * strictly inside the domain, so each walk ends at a node of level >= 2):
 * the count is a check and reads 0. */
ISO_API uint64_t iso_lhmc_stale_corners(const iso_ctx* ctx);

/* ------------------------------------------------------------------------ */
/* Batches of independent MarchingCubes chunks                               */
/* ------------------------------------------------------------------------ */
/* No single reference call: a batch stands for a loop of
 * MarchingCubes::new(size_i).extract(&source_i, &mut e_i) over many chunks
 * (marching_cubes.rs:59-82), each chunk its own IndexedVertices mesh.
 * The context's mesh holds all chunks' vertices and triangles back to back,
 * indices local to each chunk; iso_batch_extents gives, per chunk, (first
 * vertex, vertex count, first triangle, triangle count). */
typedef struct iso_chunk_desc {
    uint32_t program;   /* index into the programs array */
    uint32_t size;      /* MarchingCubes::new(size), 2..1025 */
} iso_chunk_desc;
typedef struct iso_batch iso_batch;
#define ISO_BATCH_GRAPH 1u   /* replay the batch as one CUDA graph (sized by the previous run) */

ISO_API iso_status iso_batch_create(iso_ctx* ctx, const iso_program* const* programs, uint32_t nprograms,
                                    const iso_chunk_desc* chunks, uint32_t nchunks, iso_batch** out);
ISO_API iso_status iso_batch_destroy(iso_batch* batch);
/* Run every chunk: work-queue sampler + chunked classify/scan/emit over all
 * chunks at once.  The first run (and any run after a capacity overflow) is
 * eager; with ISO_BATCH_GRAPH later runs replay one captured CUDA graph. */
ISO_API iso_status iso_batch_run(iso_batch* batch, uint32_t flags, iso_mesh_info* info);
/* The same chunks one extraction at a time (the per-chunk-launch baseline). */
ISO_API iso_status iso_batch_run_per_chunk(iso_batch* batch, iso_mesh_info* info);
/* The same per-chunk comparison without a host synchronisation per chunk:
 * each chunk's sampler, count, scan and emit launched back to back into the
 * place and size the batch's previous run found for it (run the batch once
 * first), one synchronisation at the start and one at the end. */
ISO_API iso_status iso_batch_run_per_chunk_async(iso_batch* batch, iso_mesh_info* info);
ISO_API iso_status iso_batch_extents(iso_batch* batch, uint32_t* extents /* 4 per chunk */);
/* Sampler slab depth (z layers per work-queue tile) for chunks of `size`
 * (0: all sizes); depth 0 = whole chunk. */
ISO_API iso_status iso_batch_set_slab(iso_batch* batch, uint32_t size, uint32_t depth);
/* Times the sampler at each candidate slab depth for every chunk-size class
 * of the batch and keeps the fastest; results are cached per GPU model in
 * `cache_path` (nullable).  `chosen` (nullable) receives (size, depth) pairs. */
ISO_API iso_status iso_batch_autotune(iso_batch* batch, const char* cache_path, uint32_t* chosen);

/* ------------------------------------------------------------------------ */
/* Learned SDF surrogate (no reference counterpart)                          */
/* ------------------------------------------------------------------------ */
/* A Fourier-feature MLP (3 -> 96 features -> 6 x 256 softplus (beta 100) -> 1) that
 * stands in for an expensive many-primitive source.  It is trained on the GPU
 * by the library's own forward, backward and Adam kernels on samples labelled
 * by the exact program.  Points are in the source's own coordinates (for a
 * DomainMap(source) program, the mapped coordinates). */
typedef struct iso_mlp iso_mlp;
ISO_API iso_status iso_mlp_create(iso_ctx* ctx, uint64_t seed, iso_mlp** out);
ISO_API iso_status iso_mlp_destroy(iso_mlp* net);
ISO_API uint64_t iso_mlp_num_params(void);
/* fp32 parameters: W0[256][96], b0[256], W1..W5[256][256], b1..b5[256], w_out[256], b_out */
ISO_API iso_status iso_mlp_get_params(iso_mlp* net, float* host);
ISO_API iso_status iso_mlp_set_params(iso_mlp* net, const float* host);
/* fp32 forward of n host points (x,y,z) into n host values */
ISO_API iso_status iso_mlp_forward(iso_mlp* net, const float* points, uint32_t n, float* values);
/* the same forward on the tensor cores: bf16 weights and activations, fp32
 * accumulation (tcgen05); the bf16 copy is refreshed after every update */
ISO_API iso_status iso_mlp_forward_bf16(iso_mlp* net, const float* points, uint32_t n, float* values);
/* training loss and its gradient (NPARAMS floats, nullable): mean |e| with
 * e = y - t where |t| < d, min(y - d, 0) where t >= d, max(y + d, 0) where t <= -d */
ISO_API iso_status iso_mlp_loss_grad(iso_mlp* net, const float* points, const float* targets, uint32_t n,
                                     float clamp_d, float* loss, float* grad);
/* n training samples in [lo, hi]^3: all candidates with |f| < 0.05 and a
 * quarter of the rest, labelled by `exact` */
ISO_API iso_status iso_mlp_make_dataset(iso_mlp* net, const iso_program* exact, uint32_t n, float lo, float hi,
                                        uint64_t seed);
/* `steps` Adam steps on random batches of the dataset (cosine-decayed lr);
 * the loss of each step into history (nullable) */
ISO_API iso_status iso_mlp_train(iso_mlp* net, uint32_t steps, uint32_t batch, float lr, float clamp_d,
                                 uint64_t seed, float* history);
/* Training checkpoints: a 32-byte header ("ISOMLP01", u32 version 1, u32
 * header size 32, u64 parameter count, u64 Adam steps taken) followed by the
 * fp32 parameters and Adam's first and second moments (parameter count
 * floats each, host byte order).  Loading restores the parameters, the
 * moments and the step count (which Adam's bias correction and the batch
 * sampling use), and rebuilds the bf16 inference copy; the dataset is not
 * part of the checkpoint.  iso_mlp_checkpoint_info reads and checks a
 * checkpoint's header and size without a device (ISO_ERR_INVALID_ARG for a
 * missing, short or foreign file). */
ISO_API iso_status iso_mlp_save(iso_mlp* net, const char* path);
ISO_API iso_status iso_mlp_load(iso_mlp* net, const char* path);
ISO_API iso_status iso_mlp_checkpoint_info(const char* path, uint64_t* nparams, uint64_t* step);

/* Learned-surrogate marching cubes.  The field of MarchingCubes::new(size)
 * for `exact` is built as: the network (bf16 tensor cores) on every
 * coarse_step-th lattice point; its trilinear interpolation at every fine
 * point; fine points whose interpolated value is within band_cells fine cells
 * of zero re-sampled with `exact` (bit-identical to iso_sample_grid there).
 * The network sees the exact program's frame: a program that starts with a
 * domain map p -> p * scale + offset gives the network q = p * scale + offset,
 * and a cell is 1/(size-1) times the smallest scale. */
typedef struct iso_surrogate_stats {
    uint64_t coarse_points; /* network evaluations                         */
    uint64_t band_points;   /* fine points re-sampled with the exact source */
    uint64_t total_points;  /* fine points: size * size * (size + 1)        */
} iso_surrogate_stats;
/* the field into device memory laid out as iso_sample_grid writes it */
ISO_API iso_status iso_surrogate_field(iso_ctx* ctx, iso_mlp* net, const iso_program* exact, uint32_t size,
                                       uint32_t coarse_step, float band_cells, float* field, uint64_t pitch,
                                       iso_surrogate_stats* stats);
/* iso_surrogate_field with options (no reference counterpart):
 *   ISO_SURROGATE_EXACT_COARSE: the coarse grid from `exact` instead of the
 *     network (`net` may be NULL): the same pipeline without the network, to
 *     measure what the network gains;
 *   ISO_SURROGATE_WITNESS: spot checks against `exact` at witness points of
 *     each sphere of a sphere-set source (its centre and the six axis points
 *     of its surface); a sphere whose interpolated surrogate value says
 *     "outside" at its centre has every fine point inside it or within
 *     band_cells + 1 cells (plus half the smooth-union k) of its surface
 *     re-sampled exactly as well; a sphere whose surrogate value differs
 *     from the exact one by more than band_cells - 1 cells (at least a
 *     quarter cell) at a surface witness within two cells of the exact
 *     surface has the points within that distance of its surface
 *     re-sampled.  ISO_ERR_UNSUPPORTED for other sources.
 *     *flagged_primitives (nullable) receives the flagged count. */
#define ISO_SURROGATE_EXACT_COARSE 1u
#define ISO_SURROGATE_WITNESS 2u
ISO_API iso_status iso_surrogate_field_ex(iso_ctx* ctx, iso_mlp* net, const iso_program* exact, uint32_t size,
                                          uint32_t coarse_step, float band_cells, uint32_t flags, float* field,
                                          uint64_t pitch, iso_surrogate_stats* stats, uint64_t* flagged_primitives);
/* the field, then marching cubes on it; the mesh stays in the context as
 * after iso_mc_extract (stats nullable) */
ISO_API iso_status iso_surrogate_extract(iso_ctx* ctx, iso_mlp* net, const iso_program* exact, uint32_t size,
                                         uint32_t coarse_step, float band_cells, uint32_t flags,
                                         iso_surrogate_stats* stats, iso_mesh_info* info);

/* Nearest-vertex distances between vertex sets a and b (host, xyz f32):
 * mean and max over a of the distance to the nearest b, and the reverse.
 * Chamfer = (mean_ab + mean_ba) / 2, Hausdorff = max(max_ab, max_ba).  The
 * search uses buckets of edge `bucket` and gives up after max_rings rings
 * (such points count in `capped` and report the best distance seen, or the
 * searched radius). */
typedef struct iso_mesh_distance_result {
    double mean_ab, mean_ba, max_ab, max_ba;
    uint64_t capped;
} iso_mesh_distance_result;
ISO_API iso_status iso_mesh_distance(iso_ctx* ctx, const float* a, uint64_t na, const float* b, uint64_t nb,
                                     float bucket, uint32_t max_rings, iso_mesh_distance_result* out);
/* Cells of an nx x ny x nz lattice (x < nx-1, y < ny-1, z < nz-1) whose
 * corner signs (!(v > 0)) differ between two device fields of row pitch
 * `pitch` floats. */
ISO_API iso_status iso_field_case_disagreement(iso_ctx* ctx, const float* fa, const float* fb, uint32_t nx,
                                               uint32_t ny, uint32_t nz, uint64_t pitch, uint64_t* cells);

/* ------------------------------------------------------------------------ */
/* ExtendedMarchingCubes (src/extended_marching_cubes.rs:51-186)              */
/* ------------------------------------------------------------------------ */
/* ExtendedMarchingCubes::new(size).extract(&sampler, &mut e) over the
 * Directed metric (src/distance.rs:72-104: per axis, the distance to the
 * surface along that axis), so the program may hold only the primitives,
 * Union, Intersection, Difference, the translate and domain-map point ops
 * and CentralDifference (ISO_ERR_INVALID_ARG otherwise); size <= 513.  Cells
 * whose edge-crossing normals span more than 30 degrees get a feature vertex
 * (MinimiseQEF over their tangent planes) fanned to the case's edge loops;
 * loop segments shared by two fans are then rotated to join the fan centres
 * (flip_feature_edges).  Vertices and triangles come in the reference's
 * order.  flags: ISO_FLAG_NORMALS for IndexedInterleavedNormals.  `flips`
 * (nullable) receives the number of rotated edges. */
ISO_API iso_status iso_emc_extract(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t flags,
                                   iso_mesh_info* info, uint64_t* flips);

/* ------------------------------------------------------------------------ */
/* PointCloud (src/point_cloud.rs:50-63)                                      */
/* ------------------------------------------------------------------------ */
/* PointCloud::<Signed>::new(size).extract: the centre of every cell whose
 * case is neither 0 nor 255, in traversal order, as vertices (no indices);
 * flags: ISO_FLAG_NORMALS for the *InterleavedNormals sinks. */
ISO_API iso_status iso_point_cloud_extract(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t flags,
                                           iso_mesh_info* info);

/* Deferred point-splat rendering of the last extraction, which must be a
 * PointCloud with ISO_FLAG_NORMALS: the technique of the reference's
 * examples/deferred_rasterisation.rs (a depth-tested one-pixel splat of every
 * point into position and normal buffers, three gathers of 16 taps either
 * side along x, y, x that keep, per pixel, the nearest cube of half-size
 * `voxel_half` around a gathered point that the pixel's eye ray hits, and a
 * last gather along y that shades with the example's hemisphere term),
 * written as a headless image instead of a GL framebuffer.  `view_proj` and
 * `view_proj_inverse` are 4x4 column-major matrices (projection * view, the
 * model being the identity, and its inverse); `clear_rgb` is the background.
 * `rgba` (host memory, width * height * 4 floats, row 0 at the bottom)
 * receives the composited image: the shaded colour and alpha 1 where a point
 * was hit, the clear colour and alpha 0 elsewhere. */
ISO_API iso_status iso_point_splat_render(iso_ctx* ctx, const float* view_proj, const float* view_proj_inverse,
                                          uint32_t width, uint32_t height, float voxel_half, const float* clear_rgb,
                                          float* rgba);

/* The same with flags: ISO_SPLAT_MIRROR_EDGES reads gather taps past the
 * image edge through mirrored-repeat addressing (texel -1 is texel 0, texel
 * width is texel width - 1, ...), the wrap of the default sampler the example
 * reads its buffers with; without it they read as empty. */
#define ISO_SPLAT_MIRROR_EDGES 1u
ISO_API iso_status iso_point_splat_render_ex(iso_ctx* ctx, const float* view_proj, const float* view_proj_inverse,
                                             uint32_t width, uint32_t height, float voxel_half,
                                             const float* clear_rgb, uint32_t flags, float* rgba);

/* ------------------------------------------------------------------------ */
/* Host-side sampling helpers                                                */
/* ------------------------------------------------------------------------ */
/* Evaluate the source (scalar, and normal when normals != NULL) at n host
 * points (x,y,z triples).  Used to check the device evaluator. */
ISO_API iso_status iso_sample_points(iso_ctx* ctx, const iso_program* prog, const float* points, uint64_t n,
                             float* values, float* normals);

#ifdef __cplusplus
}
#endif
#endif /* ISOSURFACE_GPU_H */
