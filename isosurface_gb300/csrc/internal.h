// Internal declarations shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "../../include/isosurface_gpu.h"

namespace iso {

// An NVTX range over one public call, named after it, for profilers that
// record NVTX (ncu --nvtx, Nsight Systems); a pointer test when none is
// attached.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

// Device-side error bits (ctx->d_err), read back after each call.
enum : uint32_t {
    DERR_SCAN_TIMEOUT = 1u,      // decoupled look-back gave up waiting
    DERR_CAPACITY = 2u,          // a kernel found its output buffer too small
    DERR_SVD_ITER = 4u,          // QR sweeps hit their bound
    DERR_QUEUE_TIMEOUT = 8u,     // work-queue wait gave up
};

// Program kinds with a dedicated sampler.
enum ProgramKind : int {
    PK_GENERIC = 0,
    PK_SPHERE_SET_HARD = 1,  // [PT_DOMAIN] SPHERE_SET(hard) [PT_POP]
};

// Device limits of the program evaluator
constexpr int VSTACK = 16;
constexpr int PSTACK = 8;

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
};

struct ProgView {
    const uint32_t* ops;
    const float* k;
    const int32_t* jump;  // CD_BEGIN -> index of its CD_END (others 0)
    uint32_t n_ops;
    // compiled form of a hard union of translated primitives (null: run ops):
    // two float4 per primitive {centre xyz, type bits}, {parameters}
    const float4* prims = nullptr;
    uint32_t nprims = 0;
    int32_t dom_at = -1;  // constants of a leading domain map, or -1
    // a bound on the value's Lipschitz constant with respect to the sample
    // point (0: none known), and a generous bound on the f32 rounding error
    // of two values the evaluator computes at points in [0, 2]^3
    float lip = 0.0f;
    float slack = 0.0f;
};

}  // namespace iso

struct iso_ctx {
    int device = 0;
    int sms = 1;  // streaming multiprocessors of the device
    int64_t fail_alloc_after = -1;  // test hook: allocations to let through before one fails (-1: off)
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    // work buffers (grow-only, reused across calls)
    iso::DevBuf field, bits, rowtri, rowvert, scan, aux, aux2, aux3, tiles, edges;
    // last mesh
    iso::DevBuf mesh_v, mesh_i, mesh_k;
    iso_mesh_info last{};
    uint32_t last_flags = 0;
    int last_vertex_floats = 3;
    // pinned host scratch
    uint64_t* h_pinned = nullptr;
    uint32_t* d_err = nullptr;
    uint64_t launches = 0;
    uint64_t lhmc_stale = 0;  // dual-cube corners with no ancestor node in the last LHMC call
    std::string last_error;
    // per-stage event timing (iso_ctx_enable_stage_timing)
    bool timing = false;
    std::vector<cudaEvent_t> event_pool;
    struct Pending {
        int stage;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    double stage_ms[ISO_STAGE_COUNT] = {};
    uint64_t stage_launches[ISO_STAGE_COUNT] = {};
    // steady-state MarchingCubes: the whole extraction recorded as one CUDA
    // graph, replayed while the program, size, flags and buffers stay the same
    bool capturing = false;  // no allocation while a stream capture records
    // a second stream for work that overlaps the context's stream (created on
    // first use) and the events that fork it from and join it to that stream
    cudaStream_t side = nullptr;
    cudaEvent_t side_fork = nullptr, side_join = nullptr;
    // page-locked host buffers (device-side pointers) that the MarchingCubes
    // kernels fill alongside the device mesh (iso_mc_extract_host); `armed`
    // reports whether the last lattice pass could deliver there
    struct HostOut {
        float* v = nullptr;
        uint32_t* i = nullptr;
        uint64_t cap_v = 0, cap_t = 0;  // vertices, triangles
        bool armed = false;
    } host_out;
    struct McPlan {
        cudaGraphExec_t exec = nullptr;
        uint64_t prog_uid = 0;
        // the recorded program's device block and contents: a program
        // uploaded again with the same contents into the same block (the
        // block pool hands it back) replays the recording too
        const void* prog_block = nullptr;
        std::vector<uint32_t> prog_ops;
        std::vector<float> prog_consts;
        uint32_t size = 0, flags = 0;
        uint64_t jit_gen = 0;  // jit_generation() when recorded
        void* bufs[12] = {};
        float* host_v = nullptr;  // host buffers baked into the recorded kernels
        uint32_t* host_i = nullptr;
        uint64_t host_cap_v = 0, host_cap_t = 0;
        bool host_armed = false;  // the recorded kernels deliver to the host buffers
        uint64_t launches = 0;
    } mc_plan;
    uint64_t mc_last_key[3] = {};  // (program identity, size, flags) of the last eager extraction
    // device blocks of destroyed programs, reused by the next uploads
    // (capacity, block): no allocation or free, and so no device-wide
    // synchronisation, while programs come and go at a steady size
    std::vector<std::pair<size_t, void*>> free_blocks;
    // the same for LinearHashedMarchingCubes (lhmc.cu), with the counts found
    struct LhmcPlan {
        cudaGraphExec_t exec = nullptr;
        const iso_program* prog = nullptr;
        uint64_t prog_uid = 0;
        uint32_t depth = 0, flags = 0;
        void* bufs[6] = {};
        std::vector<uint32_t> nref;
        uint32_t ncubes = 0, nt = 0, nv = 0;
        uint64_t launches = 0;
    } lhmc_plan;
    uint64_t lhmc_last_key[3] = {};
};

namespace iso {
// Brackets the kernels launched in its scope with events when timing is on.
struct StageTimer {
    iso_ctx* ctx;
    int stage;
    cudaEvent_t a = nullptr;
    StageTimer(iso_ctx* c, int s);
    ~StageTimer();
};
}  // namespace iso

struct iso_program {
    iso_ctx* ctx = nullptr;
    int device = 0;  // the context's device (the program may outlive the context)
    std::vector<uint32_t> ops;
    std::vector<float> consts;
    std::vector<int32_t> jump;
    void* d_block = nullptr;  // one device allocation holding the arrays below
    uint32_t* d_ops = nullptr;
    float* d_consts = nullptr;
    int32_t* d_jump = nullptr;
    float* d_set = nullptr;  // PK_SPHERE_SET_HARD: n float4 spheres, 16-byte aligned
    int kind = iso::PK_GENERIC;
    bool has_normal = true;
    // PK_SPHERE_SET_HARD
    bool has_domain = false;
    float domain[6] = {0, 0, 0, 0, 0, 0};
    uint32_t set_at = 0, set_n = 0;
    // compiled union of translated primitives (see ProgView)
    std::vector<float> prims;  // 8 floats per primitive
    float4* d_prims = nullptr;
    int32_t prim_dom_at = -1;
    float lip = 0.0f, slack = 0.0f;  // see ProgView
    size_t block_bytes = 0;          // capacity of d_block
    uint64_t content_hash = 0;       // FNV-1a of the program bytes
    uint64_t uid = 0;  // unique per program created in this process
    iso::ProgView view() const {
        return iso::ProgView{d_ops, d_consts, d_jump, (uint32_t)ops.size(), d_prims, (uint32_t)(prims.size() / 8),
                             prim_dom_at, lip, slack};
    }
};

namespace iso {

iso_status fail(iso_ctx* ctx, iso_status s, const std::string& msg);
iso_status cuda_fail(iso_ctx* ctx, cudaError_t e, const char* what);
iso_status ensure(iso_ctx* ctx, DevBuf& b, size_t bytes);
iso_status check_launch(iso_ctx* ctx, const char* what);
iso_status read_device_errors(iso_ctx* ctx);
iso_status set_device(iso_ctx* ctx);
// Work queued on *side after fork_side starts after the work queued on the
// context's stream so far; join_side makes the context's stream wait for
// the side stream's work so far.
iso_status fork_side(iso_ctx* ctx, cudaStream_t* side);
iso_status join_side(iso_ctx* ctx);

// ctx.cu: the host side of a program from its bytes (no device work)
iso_status parse_program(const uint8_t* bytes, size_t len, iso_program* p, std::string* err);

// jit.cu: changes whenever per-program compilation is switched on or off
uint64_t jit_generation();

// sample.cu
// near_only: sign bits everywhere, values at least within reach_steps
// lattice steps' worth of value change of zero (1: the ends of crossing
// edges, which marching cubes reads); other values may be left unwritten
iso_status launch_sample_grid(iso_ctx* ctx, const iso_program* prog, uint32_t nx, uint32_t ny, uint32_t nz,
                              float inv, float* field, uint64_t pitch, uint32_t* bits, bool near_only = false,
                              uint32_t zoff = 0, float reach_steps = 1.0f);
iso_status launch_sign_bits(iso_ctx* ctx, const float* field, uint32_t nx, uint32_t ny, uint32_t nz,
                            uint64_t pitch, uint32_t* bits);
iso_status launch_sample_points(iso_ctx* ctx, const iso_program* prog, const float* d_pts, uint64_t n,
                                float* d_vals, float* d_normals);
// context-free launch of the sign-bit kernel (used by the allocation-free entry point)
cudaError_t launch_sign_bits_on(cudaStream_t stream, const float* field, uint32_t nx, uint32_t ny, uint32_t nz,
                                uint64_t pitch, uint32_t* bits);

// mc.cu -- marching cubes over a lattice of samples (sign bits + values)
struct Lattice {
    uint32_t nx, ny, nz;     // sample points along each axis
    uint64_t pitch;          // floats per row of `values`
    const float* values;     // nz x ny rows of `pitch` floats
    const uint32_t* bits;    // nz x ny rows of words_per_row words, bit set iff !(v > 0)
    uint32_t words_per_row;
    float inv;               // point position = (x*inv, y*inv, z*inv)
    const float4* positions; // DC: explicit xyz per point (w unused); null = regular grid
    uint32_t zoff = 0;       // regular grid: lattice z of layer 0 (a slab of a larger grid)
};
iso_status mc_extract_lattice(iso_ctx* ctx, const Lattice& L, uint32_t flags, iso_mesh_info* info);
iso_status mc_extract_slab(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t z_begin, uint32_t z_end,
                           uint32_t flags, iso_mesh_info* info, uint64_t* halo_vertices, uint64_t* halo_triangles);
// triangles and owned vertices of the lattice's first cell layer (synchronous)
iso_status mc_first_layer_counts(iso_ctx* ctx, const Lattice& L, uint64_t* halo_vertices, uint64_t* halo_triangles);
// iso_mc_extract without the normals sink: sampler + MarchingCubes, replaying
// the context's recorded graph when it applies
iso_status mc_extract_program(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t flags,
                              iso_mesh_info* info);
// the sampler half (signs everywhere, values near the surface) into the
// context's field and sign buffers
iso_status sample_lattice(iso_ctx* ctx, const iso_program* prog, uint32_t size, Lattice* L);
// sample layers [zlo, zlo + nz) of MarchingCubes::new(size)'s lattice (a slab, L->zoff = zlo)
iso_status sample_lattice_slab(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t zlo, uint32_t nz,
                               Lattice* L);
void mc_plan_release(iso_ctx* ctx);
void lhmc_plan_release(iso_ctx* ctx);
iso_status mc_cases_lattice(iso_ctx* ctx, const Lattice& L, uint8_t* d_cases);
// PointCloud::extract over a sampled lattice: active-cell centres into the context's mesh
iso_status point_cloud_lattice(iso_ctx* ctx, const Lattice& L, iso_mesh_info* info);

// x y z -> x y z nx ny nz for n device vertices (out must not alias v)
iso_status launch_vertex_normals(iso_ctx* ctx, const iso_program* prog, const float* v, uint64_t n, float* out);
// replace the context's last mesh vertices by interleaved vertex + normal
// (the *InterleavedNormals sinks) and mark the mesh as 6 floats per vertex
iso_status attach_normals(iso_ctx* ctx, const iso_program* prog);

// exclusive scan of n u32 into out (3 launches on ctx's stream); total
// receives the sum; sums is scratch of (n + 1023) / 1024 entries
iso_status scan_u32(iso_ctx* ctx, const uint32_t* in, uint32_t* out, uint32_t n, uint32_t* sums, uint32_t* total);

inline uint32_t words_per_row(uint32_t nx) { return (nx + 31) / 32; }
inline uint64_t default_pitch(uint32_t nx) { return ((uint64_t)nx + 7) & ~7ull; }

}  // namespace iso
