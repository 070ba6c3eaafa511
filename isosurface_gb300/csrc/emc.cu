// ExtendedMarchingCubes::new(size).extract (src/extended_marching_cubes.rs:
// 51-93) on the device.  The work of each lattice point and cell is in
// emc.cuh; here each pass is one grid-stride launch over its items, the
// counts are scanned with scan_u32, and the host reads the two totals once
// to size the mesh.
//
//   emc_sample     Directed value of every lattice point (float4 per point)
//   emc_active     case of every cell; the cells with corners on both sides
//                  go to a list, which the later passes walk instead of the grid
//   emc_count      feature decision, vertex and triangle counts per active
//                  cell; the feature cells go to a second list
//   scan_u32 x 2   first vertex and first triangle of every cell
//   emc_vertices   owned edge vertices; the edge map
//   emc_features   the feature points (MinimiseQEF), a few cells per warp
//   emc_triangles  marching-cubes triangles and fans, in traversal order
//   emc_flips      feature-edge rotations
#include <cuda_runtime.h>

#include <algorithm>

#include "internal.h"

#define ISO_TABLE static __device__ const
#include "emc_tables.h"
#include "mc_tables.h"

// The host halves of emc.cuh's functions are compiled here too, reading this
// unit's device tables; only the host build of the same functions (for the
// tests, with host tables) calls them.
#pragma nv_diag_suppress 20091
#include "emc.cuh"
#pragma nv_diag_default 20091

namespace iso {
namespace {

__global__ void __launch_bounds__(256) emc_sample(emc::Args A, uint64_t points) {
    for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < points; i += (uint64_t)gridDim.x * blockDim.x)
        emc::sample_item(A, i);
}

// Every cell's case; the cells with corners on both sides (the only ones
// with work in the later passes) are appended to `list` in any order, the
// others get their case and zero counts here.
__global__ void __launch_bounds__(256) emc_active(emc::Args A, uint64_t cells, uint32_t* list, uint32_t* count) {
    const uint32_t lane = threadIdx.x & 31;
    for (uint64_t c0 = (uint64_t)blockIdx.x * blockDim.x; c0 < cells; c0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t c = c0 + threadIdx.x;
        bool active = false;
        if (c < cells) {
            uint32_t x, y, z;
            emc::cell_xyz(A.g.n, c, &x, &y, &z);
            V3 corners[8], values[8];
            emc::load_cell(A.field, A.g, x, y, z, corners, values);
            const int cube = emc::classify_directed(values);
            active = cube != 0 && cube != 255;
            if (!active) {
                A.cell[c] = (uint16_t)cube;
                A.voff[c] = 0;
                A.toff[c] = 0;
            }
        }
        const uint32_t m = __ballot_sync(0xFFFFFFFFu, active);
        if (m) {
            const uint32_t leader = (uint32_t)__ffs(m) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(m));
            base = __shfl_sync(0xFFFFFFFFu, base, leader);
            if (active) list[base + __popc(m & ((1u << lane) - 1u))] = (uint32_t)c;
        }
    }
}

// The per-cell passes over the active cells only (one thread per cell,
// grid-stride).  The counting pass also lists the feature cells.
__global__ void __launch_bounds__(128) emc_count(emc::Args A, const uint32_t* list, const uint32_t* count,
                                                 uint32_t* features, uint32_t* nfeatures) {
    const uint32_t n = *count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t c = list[i];
        emc::count_item(A, c);
        if ((A.cell[c] >> 8) & 1) features[atomicAdd(nfeatures, 1u)] = c;
    }
}

// every vertex but the feature points
__global__ void __launch_bounds__(128) emc_vertices(emc::Args A, const uint32_t* list, const uint32_t* count) {
    const uint32_t n = *count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        emc::vertex_item(A, list[i], false);
}

// The feature points: `per` listed feature cells to a one-warp block.  Each
// is one serial chain of f64 operations (the SVD, in the reference's order),
// and a warp's f64 instruction holds its sub-partition's f64 unit for many
// cycles whatever its active lanes, so the chains go to as many warps as the
// SMs' sub-partitions can take, each warp with a few, rather than scattered
// over every warp of the vertex pass.
__global__ void __launch_bounds__(32) emc_features(emc::Args A, const uint32_t* features, const uint32_t* nfeatures,
                                                   uint32_t per) {
    const uint32_t lane = threadIdx.x;
    const uint64_t i = (uint64_t)blockIdx.x * per + lane;
    if (lane < per && i < *nfeatures) emc::feature_item(A, features[i]);
}

__global__ void __launch_bounds__(256) emc_triangles(emc::Args A, const uint32_t* list, const uint32_t* count) {
    const uint32_t n = *count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        emc::triangle_item(A, list[i]);
}

__global__ void __launch_bounds__(256) emc_flips(emc::Args A, const uint32_t* list, const uint32_t* count,
                                                 unsigned long long* flips) {
    const uint32_t n = *count;
    uint32_t mine = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        mine += emc::flip_item(A, list[i]);
    if (mine) atomicAdd(flips, (unsigned long long)mine);
}

enum : uint32_t {
    OP_PT_DOMAIN_H = 0x01, OP_PT_TRANSLATE_H = 0x02, OP_PT_POP_H = 0x04,
    OP_SPHERE_H = 0x10, OP_BOX_H = 0x11, OP_CYLINDER_H = 0x12, OP_TORUS_H = 0x13,
    OP_UNION_H = 0x20, OP_INTERSECTION_H = 0x21, OP_DIFFERENCE_H = 0x22, OP_CD_BEGIN_H = 0x40, OP_CD_END_H = 0x41,
};

// The reference defines sample_vector (the Directed metric) for its
// primitives, Union, Intersection, Difference and CentralDifference; the
// translate and domain-map point ops move the point as they do for values.
bool directed_ops_only(const iso_program* p) {
    for (uint32_t w : p->ops) {
        switch (w & 0xFF) {
        case OP_PT_DOMAIN_H: case OP_PT_TRANSLATE_H: case OP_PT_POP_H:
        case OP_SPHERE_H: case OP_BOX_H: case OP_CYLINDER_H: case OP_TORUS_H:
        case OP_UNION_H: case OP_INTERSECTION_H: case OP_DIFFERENCE_H:
        case OP_CD_BEGIN_H: case OP_CD_END_H:
            break;
        default:
            return false;
        }
    }
    return true;
}

unsigned grid_for(const iso_ctx* ctx, uint64_t items, unsigned threads, unsigned per_sm) {
    const uint64_t want = (items + threads - 1) / threads;
    return (unsigned)std::max<uint64_t>(1, std::min<uint64_t>(want, (uint64_t)ctx->sms * per_sm));
}

}  // namespace
}  // namespace iso

using namespace iso;

static iso_status emc_extract_impl(iso_ctx* ctx, const iso_program* prog, uint32_t size, iso_mesh_info* info,
                                   uint64_t* flips_out) {
    if (prog->ctx != ctx) return fail(ctx, ISO_ERR_INVALID_ARG, "program belongs to another context");
    if (size > 513) return fail(ctx, ISO_ERR_TOO_LARGE, "ExtendedMarchingCubes size above 513");
    if (!directed_ops_only(prog))
        return fail(ctx, ISO_ERR_INVALID_ARG,
                    "ExtendedMarchingCubes needs the Directed metric: primitives, Union, Intersection, Difference, "
                    "translate, domain map and CentralDifference only");
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    ctx->last = iso_mesh_info{};
    ctx->last_flags = 0;
    ctx->last_vertex_floats = 3;
    if (size < 2) {  // no cell
        if (info) *info = ctx->last;
        return ISO_OK;
    }
    const uint32_t n = size;
    const uint64_t points = emc::num_points(n), cells = emc::num_cells(n);
    const uint32_t nsums = (uint32_t)((cells + 1023) / 1024);
    // Directed field | case + feature per cell | vertex and triangle offsets,
    // scan sums, totals, flip counter | edge map
    if ((s = ensure(ctx, ctx->field, 16 * points)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->aux, 2 * cells)) != ISO_OK) return s;
    const uint64_t off_words = 2 * cells, sum_words = 2ull * nsums;
    if ((s = ensure(ctx, ctx->scan, 4 * (off_words + sum_words) + 64)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->edges, 12 * points)) != ISO_OK) return s;
    // the active cells, their count, the feature cells' count, the feature cells
    const uint64_t list_words = (cells + 63) & ~(uint64_t)63;
    if ((s = ensure(ctx, ctx->aux2, 4 * (2 * list_words + 64))) != ISO_OK) return s;
    uint32_t* active = (uint32_t*)ctx->aux2.p;
    uint32_t* nactive = active + list_words;
    uint32_t* nfeatures = nactive + 1;
    uint32_t* features = nactive + 64;
    uint32_t* scan_base = (uint32_t*)ctx->scan.p;
    uint32_t* sums = scan_base + off_words;
    uint32_t* totals = sums + sum_words;  // vertices, triangles, then the flip counter (8-byte aligned)
    unsigned long long* flips = (unsigned long long*)(totals + 2);

    emc::Args A{};
    A.prog = prog->view();
    A.g = emc::Grid{n, 1.0f / (float)(n - 1)};
    A.field = (float4*)ctx->field.p;
    A.cell = (uint16_t*)ctx->aux.p;
    A.voff = scan_base;
    A.toff = scan_base + cells;
    A.edge_map = (uint32_t*)ctx->edges.p;
    A.err = ctx->d_err;
    {
        StageTimer timer(ctx, ISO_STAGE_SAMPLE);
        emc_sample<<<grid_for(ctx, points, 256, 16), 256, 0, ctx->stream>>>(A, points);
    }
    {
        StageTimer timer(ctx, ISO_STAGE_CLASSIFY);
        cudaError_t me = cudaMemsetAsync(nactive, 0, 8, ctx->stream);  // and nfeatures
        if (me != cudaSuccess) return cuda_fail(ctx, me, "emc active count");
        emc_active<<<grid_for(ctx, cells, 256, 16), 256, 0, ctx->stream>>>(A, cells, active, nactive);
        emc_count<<<grid_for(ctx, cells, 128, 32), 128, 0, ctx->stream>>>(A, active, nactive, features, nfeatures);
        ctx->launches += 3;
        if ((s = check_launch(ctx, "emc count")) != ISO_OK) return s;
        if ((s = scan_u32(ctx, A.voff, A.voff, (uint32_t)cells, sums, totals)) != ISO_OK) return s;
        if ((s = scan_u32(ctx, A.toff, A.toff, (uint32_t)cells, sums + nsums, totals + 1)) != ISO_OK) return s;
    }
    cudaError_t e = cudaMemsetAsync(flips, 0, 8, ctx->stream);
    uint32_t tot[2] = {0, 0}, nfeat = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(tot, totals, 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&nfeat, nfeatures, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "emc counts");
    const uint64_t nv = tot[0], nt = tot[1];
    if ((s = ensure(ctx, ctx->mesh_v, 12 * nv + 16)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->mesh_i, 12 * nt + 16)) != ISO_OK) return s;
    A.vertices = (float*)ctx->mesh_v.p;
    A.indices = (uint32_t*)ctx->mesh_i.p;
    A.cap_v = nv;
    A.cap_t = nt;
    {
        StageTimer timer(ctx, ISO_STAGE_EMIT);
        if (nfeat) {
            // the feature points on a side stream, beside the other passes
            // (none reads them): a few feature cells per warp, one warp for
            // each of the SMs' four sub-partitions while there are enough
            cudaStream_t side;
            if ((s = fork_side(ctx, &side)) != ISO_OK) return s;
            const uint64_t slots = 4ull * (uint64_t)std::max(ctx->sms, 1);
            const uint32_t per = (uint32_t)std::min<uint64_t>(32, (nfeat + slots - 1) / slots);
            emc_features<<<(unsigned)((nfeat + per - 1) / per), 32, 0, side>>>(A, features, nfeatures, per);
            ctx->launches++;
        }
        emc_vertices<<<grid_for(ctx, cells, 128, 32), 128, 0, ctx->stream>>>(A, active, nactive);
        emc_triangles<<<grid_for(ctx, cells, 256, 16), 256, 0, ctx->stream>>>(A, active, nactive);
        emc_flips<<<grid_for(ctx, cells, 256, 16), 256, 0, ctx->stream>>>(A, active, nactive, flips);
        if (nfeat && (s = join_side(ctx)) != ISO_OK) return s;
    }
    ctx->launches += 3;
    if ((s = check_launch(ctx, "emc emit")) != ISO_OK) return s;
    unsigned long long nflips = 0;
    e = cudaMemcpyAsync(&nflips, flips, 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "emc emit");
    if ((s = read_device_errors(ctx)) != ISO_OK) return s;
    ctx->last.num_vertices = nv;
    ctx->last.num_triangles = nt;
    ctx->last.num_cells = cells;
    if (flips_out) *flips_out = nflips;
    if (info) *info = ctx->last;
    return ISO_OK;
}

// ISO_FLAG_NORMALS: IndexedInterleavedNormals, sample_normal at every vertex
extern "C" iso_status iso_emc_extract(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t flags,
                                      iso_mesh_info* info, uint64_t* flips) {
    iso::NvtxRange nvtx_range("iso_emc_extract");
    if (!ctx || !prog) return ISO_ERR_INVALID_ARG;
    if (flags & ~(uint32_t)ISO_FLAG_NORMALS) return fail(ctx, ISO_ERR_INVALID_ARG, "unsupported flags");
    iso_status s = emc_extract_impl(ctx, prog, size, info, flips);
    if (s != ISO_OK || !(flags & ISO_FLAG_NORMALS)) return s;
    if ((s = attach_normals(ctx, prog)) != ISO_OK) return s;
    if (info) *info = ctx->last;
    return ISO_OK;
}
