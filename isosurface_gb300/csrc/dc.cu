// DualContouring::new(size, placer).extract (src/dual_contouring.rs:65-105)
// over DualGrid::traverse (src/traversal/dual_grid.rs:52-95).
//
// The dual lattice has one vertex per primal cell: (size-1) x (size-1) x size
// vertices.  Its value is lerp(v0, v6, 0.5) of the primal corners
// (dual_grid.rs:80-81); its position is the cell centre lerp(c0, c6, 0.5)
// unless the cell is active (case not 0 or 255), where the feature placer
// puts it (dual_contouring.rs:78-87).  The dual cubes are then meshed exactly
// like MarchingCubes over the dual lattice with explicit vertex positions
// (dual_contouring.rs:88-101 is the same cell kernel with GridKey dedup), so
// the last two passes are mc_extract_lattice.
//
// Passes: (1) grid sampler (sign bits everywhere; for a program with a
// Lipschitz bound, values only near the surface, NaN elsewhere), (2) dc_dual:
// sign bits of every dual vertex, value and centre of those marching cubes
// can read, active primal cells appended to a list, (3) dc_place:
// one thread per active cell -- eight normals from the program
// (sample_normals_at_corners, marching_cubes_impl.rs:58-69), tangent planes,
// the planar cells' centre of mass or particle placement, the non-planar
// cells listed for (3b) dc_feature: their MinimiseQEF (f64 SVD) in full
// warps, (4)+(5) the lattice marching-cubes passes.
#include <cuda_runtime.h>

#include "internal.h"
#include "qef.cuh"
#include "vm.cuh"
#include "dc_core.cuh"

namespace iso {
// jit.cu: dc_place with the program's compiled normals; false (nothing
// launched) when the program has none
bool jit_dc_place(iso_ctx* ctx, const iso_program* prog, const DcCells& cells, uint64_t blocks, cudaError_t* err);

namespace {

struct DualArgs {
    const float* field;   // primal values; NaN where the sampler left them unwritten
    const uint32_t* bits; // primal sign bits (bit set iff !(v > 0)), W words per row
    uint32_t W;
    uint64_t pitch;       // primal row pitch
    uint32_t n;           // primal size: n x n x (n+1) samples
    uint32_t nzd;         // dual layers here (primal cell layers zoff .. zoff + nzd - 1)
    uint32_t zoff;        // primal cell layer of dual layer 0 (a slab of the whole lattice)
    float inv;
    float* dval;          // dual values, rows of dpitch
    uint64_t dpitch;
    float4* dpos;         // dual positions, dense (n-1) x (n-1) x nzd
    uint32_t* dbits;      // dual sign bits (bit set iff !(value > 0)), dW words per row
    uint32_t dW;
    uint32_t* list;       // active primal cells (linear dual index)
    uint32_t* count;
    uint32_t cap;
    uint32_t* err;
    bool near;            // the sampler wrote values only near the surface (NaN elsewhere)
};

// One warp per 32 dual vertices of a dual row (x = 32 w + lane): value,
// centre, sign word (by ballot) and the active primal cells.  A dual vertex
// whose primal corners 0 or 6 the near-surface sampler skipped gets its sign
// only: those corners lie more than 2.5 lattice steps' worth of value change
// from zero, so (by the Lipschitz bound) v0 and v6 share the sign of corner 0
// and the dual value lies more than 1.6 steps' worth from zero, while both
// ends of a crossing dual edge lie within one step's worth; marching cubes
// reads values and positions only at those ends.
__global__ void __launch_bounds__(256) dc_dual(DualArgs A) {
    const uint32_t m = A.n - 1, lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (gw >= (uint64_t)A.dW * m * A.nzd) return;  // warp-uniform
    const uint32_t w = (uint32_t)(gw % A.dW);
    const uint64_t row = gw / A.dW;
    const uint32_t y = (uint32_t)(row % m), z = (uint32_t)(row / m);
    const uint32_t x = 32 * w + lane;
    bool active = false, inside = false;
    if (x < m) {
        // corner signs from the sign bits, in CORNERS order (marching_cubes_tables.rs:16-25)
        auto sign_bit = [&](uint32_t xx, uint32_t yy, uint32_t zz) {
            return (__ldg(A.bits + ((size_t)zz * A.n + yy) * A.W + (xx >> 5)) >> (xx & 31)) & 1u;
        };
        const uint32_t cs = sign_bit(x, y, z) | sign_bit(x + 1, y, z) << 1 | sign_bit(x + 1, y + 1, z) << 2 |
                            sign_bit(x, y + 1, z) << 3 | sign_bit(x, y, z + 1) << 4 |
                            sign_bit(x + 1, y, z + 1) << 5 | sign_bit(x + 1, y + 1, z + 1) << 6 |
                            sign_bit(x, y + 1, z + 1) << 7;
        const float* f0 = A.field + ((size_t)z * A.n + y) * A.pitch + x;
        const float v0 = __ldg(f0), v6 = __ldg(f0 + (size_t)A.n * A.pitch + A.pitch + 1);
        const uint64_t id = ((uint64_t)z * m + y) * m + x;
        const bool sampled = v0 == v0 && v6 == v6;
        if (sampled || !A.near) {
            // Vec3::lerp / Signed::lerp with f = 0.5: (1 - f) * a + f * b (a
            // full field's own NaN gets a signed sentinel in its place)
            const float of = 1.0f - 0.5f;
            const float c0x = (float)x * A.inv, c0y = (float)y * A.inv, c0z = (float)(z + A.zoff) * A.inv;
            const float c6x = (float)(x + 1) * A.inv, c6y = (float)(y + 1) * A.inv,
                        c6z = (float)(z + 1 + A.zoff) * A.inv;
            const float dv = sampled ? of * v0 + 0.5f * v6 : ((cs & 1u) ? -3.0e38f : 3.0e38f);
            A.dpos[id] = make_float4(of * c0x + 0.5f * c6x, of * c0y + 0.5f * c6y, of * c0z + 0.5f * c6z, 0.0f);
            A.dval[((size_t)z * m + y) * A.dpitch + x] = dv;
            inside = !(dv > 0.0f);
        } else {
            inside = (cs & 1u) != 0;
        }
        active = cs != 0 && cs != 255;
    }
    const uint32_t word = __ballot_sync(0xFFFFFFFFu, inside);
    if (lane == 0) A.dbits[row * A.dW + w] = word;
    // warp-aggregated append of the active cells (their order does not matter)
    const uint32_t mask = __ballot_sync(0xFFFFFFFFu, active);
    if (mask) {
        uint32_t base = 0;
        if (lane == (uint32_t)__ffs(mask) - 1) base = atomicAdd(A.count, (uint32_t)__popc(mask));
        base = __shfl_sync(0xFFFFFFFFu, base, __ffs(mask) - 1);
        if (active) {
            const uint32_t at = base + __popc(mask & ((1u << lane) - 1u));
            if (at < A.cap) A.list[at] = (uint32_t)(((uint64_t)z * m + y) * m + x);
            else atomicOr(A.err, DERR_CAPACITY);
        }
    }
}

// The interpreter's normals (eval_hermite) as a dc_core.cuh evaluator.
struct VmHermite {
    ProgView pv;
    __device__ __forceinline__ V3 normal(V3 p) const {
        V3 nn;
        eval_hermite(pv, p, &nn);
        return nn;
    }
};

__global__ void __launch_bounds__(128) dc_place(VmHermite ev, DcCells A) { dc_place_body(ev, A); }

// MinimiseQEF of the non-planar cells dc_place listed, one per thread over
// one-warp blocks (grid-stride): each is a serial chain of f64 operations
// (the SVD, in the reference's order), and a warp's f64 instruction holds
// its sub-partition's f64 unit for many cycles however few of its lanes are
// active, so packing the chains into full warps cuts the f64 instructions
// the scattered cells of dc_place would have issued.
__global__ void __launch_bounds__(32) dc_feature(VmHermite ev, DcCells A, uint32_t* err) {
    const uint32_t n = *A.nfeatures;
    for (uint32_t i = blockIdx.x * 32 + threadIdx.x; i < n; i += gridDim.x * 32) {
        const uint32_t id = A.features[i];
        qef::F3 corners[8], normals[8];
        if (i < A.fcap) {  // the normals dc_place computed when it listed the cell
            const uint32_t m = A.n - 1;
            const uint32_t x = id % m, r = id / m, y = r % m, z = r / m;
            const uint8_t cornr[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                         {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
            for (int k = 0; k < 8; ++k) {
                corners[k] = qef::f3((float)(x + cornr[k][0]) * A.inv, (float)(y + cornr[k][1]) * A.inv,
                                     (float)(z + A.zoff + cornr[k][2]) * A.inv);
                normals[k] = A.fnormals[8 * (uint64_t)i + k];
            }
        } else {
            dc_cell_normals(ev, A, id, corners, normals);
        }
        qef::Planes t;
        qef::tangent_planes(corners, normals, &t);
        bool ok;
        const qef::F3 p = qef::minimise_qef(t, &ok);
        if (!ok) atomicOr(err, DERR_SVD_ITER);
        A.dpos[id] = DcPos{p.x, p.y, p.z, 0.0f};
    }
}

}  // namespace
}  // namespace iso

using namespace iso;

static iso_status dc_check(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t placer, uint32_t flags) {
    if (!ctx || !prog) return ISO_ERR_INVALID_ARG;
    if (prog->ctx != ctx) return fail(ctx, ISO_ERR_INVALID_ARG, "program belongs to another context");
    if (size == 0 || size > 16384) return fail(ctx, ISO_ERR_INVALID_ARG, "size out of range");
    if (placer > 1) return fail(ctx, ISO_ERR_INVALID_ARG, "placer must be 0 (MinimiseQEF) or 1 (particles)");
    if (flags & ~(uint32_t)ISO_FLAG_KEYS) return fail(ctx, ISO_ERR_INVALID_ARG, "unsupported flags");
    if ((uint64_t)(size - 1) * (size - 1) * size >= 0xFFFFFFFFull) return fail(ctx, ISO_ERR_TOO_LARGE, "grid too large");
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    ctx->last = iso_mesh_info{};
    ctx->last_flags = flags;
    ctx->last_vertex_floats = 3;
    return ISO_OK;
}

// The dual lattice's layers [zlo, zlo + nzd) of DualContouring::new(n) (dual
// layer k: one vertex per primal cell of cell layer k), from the primal
// sample layers [zlo, zlo + nzd]: values, signs and placed positions in the
// whole lattice's frame.  The whole extraction is zlo = 0, nzd = n.
static iso_status dc_lattice(iso_ctx* ctx, const iso_program* prog, uint32_t n, uint32_t placer, uint32_t zlo,
                             uint32_t nzd, Lattice* L) {
    const uint32_t m = n - 1, nzp = nzd + 1;  // primal sample layers
    const uint64_t pitch = default_pitch(n), W = words_per_row(n);
    const uint64_t ndual = (uint64_t)m * m * nzd;
    const uint64_t dpitch = default_pitch(m), dW = words_per_row(m);
    iso_status s;
    // primal field + bits | dual values | dual positions | dual bits | active list
    if ((s = ensure(ctx, ctx->field, 4ull * pitch * n * nzp)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->bits, 4ull * W * n * nzp)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->aux, 4ull * dpitch * m * nzd)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->aux2, 16ull * ndual)) != ISO_OK) return s;
    const uint64_t list_words = (ndual + 63) & ~(uint64_t)63;
    // normals kept for the first feature cells (96 bytes each, at most 96 MB)
    const uint32_t fcap = (uint32_t)std::min<uint64_t>(list_words, 1u << 20);
    if ((s = ensure(ctx, ctx->aux3, 4ull * dW * m * nzd + 8ull * list_words + 256 + 96ull * fcap)) != ISO_OK)
        return s;
    float* field = (float*)ctx->field.p;
    uint32_t* bits = (uint32_t*)ctx->bits.p;
    float* dval = (float*)ctx->aux.p;
    float4* dpos = (float4*)ctx->aux2.p;
    uint32_t* dbits = (uint32_t*)ctx->aux3.p;
    uint32_t* count = dbits + dW * m * nzd;  // active cells, then (count + 1) non-planar ones
    uint32_t* list = count + 64;
    uint32_t* features = list + list_words;
    qef::F3* fnormals = reinterpret_cast<qef::F3*>(features + list_words);
    const float inv = 1.0f / (float)(n - 1);
    // values only near the surface (programs with a Lipschitz bound): the
    // dual values read the primal ones up to 1 + sqrt(3)/2 lattice steps'
    // worth of change from zero (a dual crossing end within one step's
    // worth, and half the cell diagonal between its two corners); the
    // sampler keeps 2.5, and the others stay NaN for dc_dual to recognise
    const bool near = prog->lip > 0.0f;
    cudaError_t e = cudaSuccess;
    if (near) e = cudaMemsetAsync(field, 0xFF, 4ull * pitch * n * nzp, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "clear field");
    if ((s = launch_sample_grid(ctx, prog, n, n, nzp, inv, field, pitch, bits, near, zlo, 2.5f)) != ISO_OK) return s;
    e = cudaMemsetAsync(count, 0, 8, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "memset");
    {
        StageTimer timer(ctx, ISO_STAGE_PLACE);
        DualArgs da{field, bits, (uint32_t)W, pitch, n, nzd, zlo, inv, dval, dpitch, dpos, dbits, (uint32_t)dW,
                    list, count, (uint32_t)ndual, ctx->d_err, near};
        const uint64_t dual_warps = dW * m * nzd;
        dc_dual<<<(unsigned)((dual_warps + 7) / 8), 256, 0, ctx->stream>>>(da);
        const DcCells cells{n, zlo, inv, list, count, reinterpret_cast<DcPos*>(dpos), (int)placer, features,
                            count + 1, fnormals, fcap};
        const VmHermite ev{prog->view()};
        const uint64_t place_blocks = std::min<uint64_t>((ndual + 127) / 128, 152 * 64);
        cudaError_t je = cudaSuccess;
        if (!jit_dc_place(ctx, prog, cells, place_blocks, &je))  // the program's compiled normals (jit.cu)
            dc_place<<<(unsigned)place_blocks, 128, 0, ctx->stream>>>(ev, cells);
        else if (je != cudaSuccess)
            return cuda_fail(ctx, je, "compiled dc_place launch");
        if (placer == 0) {
            // one warp for each of the SMs' four sub-partitions
            dc_feature<<<(unsigned)(4 * std::max(ctx->sms, 1)), 32, 0, ctx->stream>>>(ev, cells, ctx->d_err);
            ctx->launches++;
        }
    }
    ctx->launches += 2;
    if ((s = check_launch(ctx, "dc passes")) != ISO_OK) return s;
    *L = Lattice{m, m, nzd, dpitch, dval, dbits, (uint32_t)dW, 0.0f, dpos, zlo};
    return ISO_OK;
}

static iso_status dc_extract_impl(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t placer,
                                     uint32_t flags, iso_mesh_info* info) {
    iso_status s = dc_check(ctx, prog, size, placer, flags);
    if (s != ISO_OK) return s;
    if (size < 3) {  // the dual lattice has no cube
        if (info) *info = ctx->last;
        return ISO_OK;
    }
    Lattice L;
    if ((s = dc_lattice(ctx, prog, size, placer, 0, size, &L)) != ISO_OK) return s;
    return mc_extract_lattice(ctx, L, flags, info);
}

// One slab of a z-partition of DualContouring::new(size): dual cube layers
// [z_begin, z_end) of the size - 1, plus the halo cube layer below when
// z_begin > 0, exactly as mc_extract_slab does for MarchingCubes.
extern "C" iso_status iso_dc_extract_slab(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t placer,
                                          uint32_t z_begin, uint32_t z_end, uint32_t flags, iso_mesh_info* info,
                                          uint64_t* halo_vertices, uint64_t* halo_triangles) {
    iso::NvtxRange nvtx_range("iso_dc_extract_slab");
    iso_status s = dc_check(ctx, prog, size, placer, flags);
    if (s != ISO_OK) return s;
    if (size < 3 || z_begin >= z_end || z_end > size - 1)
        return fail(ctx, ISO_ERR_INVALID_ARG, "need size >= 3 and 0 <= z_begin < z_end <= size - 1");
    const uint32_t halo = z_begin > 0 ? 1u : 0u, zlo = z_begin - halo;
    Lattice L;
    if ((s = dc_lattice(ctx, prog, size, placer, zlo, z_end - zlo + 1, &L)) != ISO_OK) return s;
    uint64_t hv = 0, ht = 0;
    if (halo && (s = mc_first_layer_counts(ctx, L, &hv, &ht)) != ISO_OK) return s;
    if ((s = mc_extract_lattice(ctx, L, flags, info)) != ISO_OK) return s;
    if (halo_vertices) *halo_vertices = hv;
    if (halo_triangles) *halo_triangles = ht;
    return ISO_OK;
}

// ISO_FLAG_NORMALS: the *InterleavedNormals sinks, sample_normal at every vertex
extern "C" iso_status iso_dc_extract(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t placer, uint32_t flags, iso_mesh_info* info) {
    iso::NvtxRange nvtx_range("iso_dc_extract");
    if (!ctx || !prog) return ISO_ERR_INVALID_ARG;
    if (flags & ~(uint32_t)(ISO_FLAG_KEYS | ISO_FLAG_NORMALS)) return fail(ctx, ISO_ERR_INVALID_ARG, "unsupported flags");
    iso_status s = dc_extract_impl(ctx, prog, size, placer, flags & ~(uint32_t)ISO_FLAG_NORMALS, info);
    if (s != ISO_OK || !(flags & ISO_FLAG_NORMALS)) return s;
    return attach_normals(ctx, prog);
}
