// Batched MarchingCubes: thousands of independent chunks, each a
// MarchingCubes::new(size_i).extract over its own source, in one pass.
//
// * Sampling: one persistent kernel drains a work queue of (chunk, z-slab,
//   y-range) tiles (largest cost first); each block samples its tile with the
//   culled sampler of bricks.cuh (sign bits everywhere, values where marching
//   cubes can read them, primitives pruned per sub-brick).  The slab depth
//   per chunk-size class comes from iso_batch_autotune.
// * Classification, scan and emission: the chunked marching-cubes passes of
//   mc.cu over a table of grids whose 32-cell chunks are laid out
//   range-aligned in one global index space (mc_chunk.cuh).
// * iso_batch_run with ISO_BATCH_GRAPH captures all of it in one CUDA graph
//   and replays it; output capacities come from the previous run (the first
//   run is eager and sizes them), and an overflow is detected on the device
//   and answered with an eager re-run.
// * iso_batch_run_per_chunk runs the same chunks one extraction at a time
//   (sample, count, scan, emit, with the host syncs of iso_mc_extract) and
//   concatenates the meshes: the comparison point for the batch.
//
// Output: the context's mesh holds all chunks' vertices and triangles
// back to back; indices are local to each chunk (each chunk is its own
// IndexedVertices mesh); iso_batch_extents gives each chunk's
// (first vertex, vertices, first triangle, triangles).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "bricks.cuh"
#include "internal.h"
#include "vm.cuh"

namespace iso {
// defined in mc.cu
iso_status mc_extract_grids(iso_ctx* ctx, const void* d_grids, uint32_t ngrids, const uint32_t* d_range_grid,
                            uint32_t chunks, uint32_t max_cw, void* scratch, uint64_t cap_v, uint64_t cap_t,
                            float* out_v, uint32_t* out_i, uint32_t* extents, uint64_t* totals, bool sync_sizes);
size_t mc_grid_bytes();
void mc_fill_grid(void* dst, const Lattice& L, uint32_t chunk0, uint32_t* nchunks, uint32_t* cw);
size_t mc_grids_scratch_bytes(uint32_t chunks, uint32_t ngrids);
}  // namespace iso

using namespace iso;

namespace {

struct SampleGrid {
    ProgView pv;
    uint32_t n;  // MarchingCubes::new(n): n x n x (n+1) samples
    float inv;
    float* field;
    uint64_t pitch;
    uint32_t* bits;
    uint32_t W;
};

struct Tile {
    uint32_t grid, z0, z1, y0, y1;  // layers [z0, z1), rows [y0, y1), all x
};

// A persistent grid: each block takes tiles from the work queue (largest
// first) and samples them whole with the culled sampler (bricks.cuh).
__global__ void __launch_bounds__(256) batch_sample(const Tile* tiles, const SampleGrid* grids, uint32_t ntiles,
                                                    uint32_t* next) {
    __shared__ uint32_t s_tile, s_n;
    __shared__ uint8_t s_cls[BRICK_MAX];
    __shared__ uint64_t s_keep[BRICK_MAX];
    __shared__ uint32_t s_list[BRICK_MAX];
    while (true) {
        __syncthreads();  // the previous tile is done with the shared arrays
        if (threadIdx.x == 0) s_tile = atomicAdd(next, 1u);
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= ntiles) return;
        const Tile tl = tiles[t];
        const SampleGrid sg = grids[tl.grid];
        const BrickTile T{BrickLattice{sg.pv.lip, sg.pv.slack, sg.n, sg.n, sg.n + 1, sg.inv, sg.field, sg.pitch,
                                       sg.bits, sg.W, 0, 1.0f},
                          tl.y0, tl.y1, tl.z0, tl.z1};
        brick_tile(VmEval{sg.pv}, T, s_cls, s_keep, s_list, &s_n);
    }
}

// The tiles of one chunk of `n` (n x n x (n + 1) samples) for slab depth
// `depth` (0: the whole chunk), rounded up to whole sub-bricks (4 layers)
// and cut in y so that a tile holds at most BRICK_MAX sub-bricks.
template <class F>
void chunk_tiles(uint32_t grid, uint32_t n, uint32_t depth, F&& add) {
    const uint32_t nz = n + 1, SX = 4 * words_per_row(n);
    uint32_t zg = ((depth ? depth : nz) + 3) / 4;
    zg = std::max(1u, std::min(zg, BRICK_MAX / SX));
    const uint32_t ty = std::max(1u, std::min((n + 3) / 4, BRICK_MAX / (SX * zg)));
    for (uint32_t z0 = 0; z0 < nz; z0 += 4 * zg)
        for (uint32_t y0 = 0; y0 < n; y0 += 4 * ty)
            add(Tile{grid, z0, std::min(nz, z0 + 4 * zg), y0, std::min(n, y0 + 4 * ty)});
}

struct Chunk {
    uint32_t prog, size;
};

}  // namespace

struct iso_batch {
    iso_ctx* ctx = nullptr;
    std::vector<const iso_program*> programs;
    std::vector<Chunk> chunks;
    std::vector<uint32_t> slab;      // slab depth per chunk (0 = whole grid)
    // device layout
    void* arena = nullptr;
    size_t arena_bytes = 0;
    SampleGrid* d_sgrids = nullptr;
    void* d_grids = nullptr;
    uint32_t* d_range_grid = nullptr;
    Tile* d_tiles = nullptr;
    uint32_t ntiles = 0;
    uint32_t* d_next = nullptr;  // the sampler's work-queue counter
    uint32_t* d_extents = nullptr;   // 4 per chunk
    uint64_t* d_totals = nullptr;    // [0] triangles [1] vertices
    void* d_scratch = nullptr;       // chunk-pass scratch
    uint32_t total_chunks = 0, max_cw = 0;
    std::vector<SampleGrid> sgrids;
    std::vector<uint32_t> grid_chunk0;
    // outputs and graph
    uint64_t cap_v = 0, cap_t = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    // the context's mesh buffers the graph was captured with: another
    // extraction on the context may regrow (free and reallocate) them
    void* graph_v = nullptr;
    void* graph_i = nullptr;
    bool sized = false;
    // iso_batch_run_per_chunk_async: each chunk as a grid of its own
    void* d_solo_grids = nullptr;
    std::vector<uint32_t> solo_chunks, solo_cw;
};

namespace {

// Device copy of `tiles`.
cudaError_t upload_tiles(const std::vector<Tile>& tiles, Tile** d_tiles) {
    cudaError_t e = cudaMalloc((void**)d_tiles, sizeof(Tile) * std::max<size_t>(tiles.size(), 1));
    if (e == cudaSuccess && !tiles.empty())
        e = cudaMemcpy(*d_tiles, tiles.data(), sizeof(Tile) * tiles.size(), cudaMemcpyHostToDevice);
    return e;
}

iso_status build_tiles(iso_batch* b) {
    std::vector<std::pair<double, Tile>> t;
    for (uint32_t i = 0; i < b->chunks.size(); ++i) {
        const uint32_t n = b->chunks[i].size;
        const double cost_per_point = (double)b->programs[b->chunks[i].prog]->ops.size();
        chunk_tiles(i, n, b->slab[i], [&](const Tile& tl) {
            t.push_back({cost_per_point * ((n + 31) / 32 * 32) * (tl.y1 - tl.y0) * (tl.z1 - tl.z0), tl});
        });
    }
    std::stable_sort(t.begin(), t.end(), [](const auto& a, const auto& c) { return a.first > c.first; });
    std::vector<Tile> tiles(t.size());
    for (size_t i = 0; i < t.size(); ++i) tiles[i] = t[i].second;
    if (b->d_tiles) cudaFree(b->d_tiles);
    b->d_tiles = nullptr;
    b->ntiles = (uint32_t)tiles.size();
    cudaError_t e = upload_tiles(tiles, &b->d_tiles);
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (b->graph) {
        cudaGraphDestroy(b->graph);
        b->graph = nullptr;
    }
    return e == cudaSuccess ? ISO_OK : cuda_fail(b->ctx, e, "tiles");
}

// blocks of batch_sample that fill every SM (looked up once per process)
unsigned sample_blocks(int sms) {
    static std::atomic<int> per_sm{0};
    return persistent_blocks((const void*)batch_sample, per_sm, sms);
}

// the culled sampler over `ntiles` tiles (the queue counter zeroed first)
cudaError_t launch_sampler(iso_ctx* ctx, const Tile* d_tiles, uint32_t ntiles, const SampleGrid* d_sgrids,
                           uint32_t* next) {
    cudaError_t e = cudaMemsetAsync(next, 0, 4, ctx->stream);
    if (e != cudaSuccess) return e;
    batch_sample<<<sample_blocks(ctx->sms), 256, 0, ctx->stream>>>(d_tiles, d_sgrids, ntiles, next);
    return cudaGetLastError();
}

// enqueue the whole batch on the context's stream (no host sync)
iso_status enqueue(iso_batch* b, bool sync_sizes) {
    iso_ctx* ctx = b->ctx;
    {
        StageTimer timer(ctx, ISO_STAGE_SAMPLE);
        cudaError_t e = launch_sampler(ctx, b->d_tiles, b->ntiles, b->d_sgrids, b->d_next);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "batch sampler");
    }
    ctx->launches++;
    return mc_extract_grids(ctx, b->d_grids, (uint32_t)b->chunks.size(), b->d_range_grid, b->total_chunks, b->max_cw,
                            b->d_scratch, b->cap_v, b->cap_t, (float*)ctx->mesh_v.p, (uint32_t*)ctx->mesh_i.p,
                            b->d_extents, b->d_totals, sync_sizes);
}

iso_status finish(iso_batch* b, iso_mesh_info* info) {
    iso_ctx* ctx = b->ctx;
    cudaError_t e = cudaMemcpyAsync(ctx->h_pinned, b->d_totals, 16, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctx->h_pinned + 2, ctx->d_err, 4, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "batch totals");
    const uint64_t nt = ctx->h_pinned[0], nv = ctx->h_pinned[1];
    uint64_t cells = 0;
    for (auto& c : b->chunks) cells += (uint64_t)(c.size - 1) * (c.size - 1) * c.size;
    ctx->last.num_vertices = nv;
    ctx->last.num_triangles = nt;
    ctx->last.num_cells = cells;
    ctx->last_flags = 0;
    ctx->last_vertex_floats = 3;
    if (info) *info = ctx->last;
    if ((uint32_t)ctx->h_pinned[2]) return read_device_errors(ctx);
    return ISO_OK;
}

}  // namespace

extern "C" {

iso_status iso_batch_create(iso_ctx* ctx, const iso_program* const* programs, uint32_t nprograms,
                            const iso_chunk_desc* chunks, uint32_t nchunks, iso_batch** out) {
    if (!ctx || !out || (!programs && nprograms) || (!chunks && nchunks) || nchunks == 0) return ISO_ERR_INVALID_ARG;
    *out = nullptr;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    iso_batch* b = new iso_batch();
    b->ctx = ctx;
    b->programs.assign(programs, programs + nprograms);
    for (uint32_t i = 0; i < nprograms; ++i)
        if (!programs[i] || programs[i]->ctx != ctx) {
            delete b;
            return fail(ctx, ISO_ERR_INVALID_ARG, "null program or program of another context");
        }
    for (uint32_t i = 0; i < nchunks; ++i) {
        if (chunks[i].program >= nprograms || chunks[i].size < 2 || chunks[i].size > 1025) {
            delete b;
            return fail(ctx, ISO_ERR_INVALID_ARG, "chunk program index out of range or size not in [2, 1025]");
        }
        b->chunks.push_back(Chunk{chunks[i].program, chunks[i].size});
    }
    b->slab.assign(nchunks, 4);
    // layout: per chunk field + bits; grid tables; chunk-pass scratch
    size_t off = 0;
    auto take = [&](size_t bytes) {
        off = (off + 255) & ~(size_t)255;
        const size_t at = off;
        off += bytes;
        return at;
    };
    std::vector<size_t> field_off(nchunks), bits_off(nchunks);
    uint32_t chunk0 = 0;
    b->grid_chunk0.resize(nchunks);
    for (uint32_t i = 0; i < nchunks; ++i) {
        const uint32_t n = b->chunks[i].size;
        field_off[i] = take(4ull * default_pitch(n) * n * (n + 1));
        bits_off[i] = take(4ull * words_per_row(n) * n * (n + 1));
        const uint32_t cw = (n - 1 + 31) / 32;
        const uint32_t nch = cw * (n - 1) * n;
        b->grid_chunk0[i] = chunk0;
        chunk0 += (nch + 255) / 256 * 256;
        b->max_cw = std::max(b->max_cw, cw);
    }
    b->total_chunks = chunk0;
    const uint32_t nranges = chunk0 / 256;
    const size_t sg_off = take(sizeof(SampleGrid) * nchunks);
    const size_t g_off = take(mc_grid_bytes() * nchunks);
    const size_t rg_off = take(4ull * nranges);
    const size_t next_off = take(256);
    const size_t ext_off = take(16ull * nchunks);
    const size_t tot_off = take(64);
    const size_t scr_off = take(mc_grids_scratch_bytes(b->total_chunks, nchunks));
    b->arena_bytes = off;
    cudaError_t e = cudaMalloc(&b->arena, b->arena_bytes);
    if (e != cudaSuccess) {
        delete b;
        return cuda_fail(ctx, e, "batch arena");
    }
    char* base = (char*)b->arena;
    b->d_sgrids = (SampleGrid*)(base + sg_off);
    b->d_grids = base + g_off;
    b->d_range_grid = (uint32_t*)(base + rg_off);
    b->d_next = (uint32_t*)(base + next_off);
    b->d_extents = (uint32_t*)(base + ext_off);
    b->d_totals = (uint64_t*)(base + tot_off);
    b->d_scratch = base + scr_off;
    std::vector<char> grids(mc_grid_bytes() * nchunks);
    std::vector<uint32_t> range_grid(nranges);
    b->sgrids.resize(nchunks);
    for (uint32_t i = 0; i < nchunks; ++i) {
        const uint32_t n = b->chunks[i].size;
        const iso_program* p = b->programs[b->chunks[i].prog];
        SampleGrid sg{p->view(), n, 1.0f / (float)(n - 1), (float*)(base + field_off[i]), default_pitch(n),
                      (uint32_t*)(base + bits_off[i]), words_per_row(n)};
        b->sgrids[i] = sg;
        Lattice L{n, n, n + 1, default_pitch(n), sg.field, sg.bits, sg.W, sg.inv, nullptr};
        uint32_t nch = 0, cw = 0;
        mc_fill_grid(grids.data() + mc_grid_bytes() * i, L, b->grid_chunk0[i], &nch, &cw);
        for (uint32_t r = b->grid_chunk0[i] / 256; r < (b->grid_chunk0[i] + nch + 255) / 256; ++r) range_grid[r] = i;
    }
    e = cudaMemcpy(b->d_sgrids, b->sgrids.data(), sizeof(SampleGrid) * nchunks, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(b->d_grids, grids.data(), grids.size(), cudaMemcpyHostToDevice);
    if (e == cudaSuccess && nranges)
        e = cudaMemcpy(b->d_range_grid, range_grid.data(), 4ull * nranges, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        iso_batch_destroy(b);
        return cuda_fail(ctx, e, "batch tables");
    }
    if ((s = build_tiles(b)) != ISO_OK) {
        iso_batch_destroy(b);
        return s;
    }
    *out = b;
    return ISO_OK;
}

iso_status iso_batch_destroy(iso_batch* b) {
    if (!b) return ISO_ERR_INVALID_ARG;
    cudaSetDevice(b->ctx->device);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    if (b->d_tiles) cudaFree(b->d_tiles);
    if (b->arena) cudaFree(b->arena);
    if (b->d_solo_grids) cudaFree(b->d_solo_grids);
    delete b;
    return ISO_OK;
}

iso_status iso_batch_set_slab(iso_batch* b, uint32_t size, uint32_t depth) {
    if (!b) return ISO_ERR_INVALID_ARG;
    for (size_t i = 0; i < b->chunks.size(); ++i)
        if (size == 0 || b->chunks[i].size == size) b->slab[i] = depth;
    return build_tiles(b);
}

iso_status iso_batch_run(iso_batch* b, uint32_t flags, iso_mesh_info* info) {
    iso::NvtxRange nvtx_range("iso_batch_run");
    if (!b) return ISO_ERR_INVALID_ARG;
    iso_ctx* ctx = b->ctx;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    const bool graph = (flags & ISO_BATCH_GRAPH) != 0;
    if (!graph || !b->sized) {
        // eager: sizes are read back between the count and the emit passes
        s = enqueue(b, true);
        if (s != ISO_OK) return s;
        if ((s = finish(b, info)) != ISO_OK) return s;
        if (!b->sized || ctx->last.num_vertices > b->cap_v || ctx->last.num_triangles > b->cap_t) {
            b->cap_v = ctx->last.num_vertices + ctx->last.num_vertices / 4 + 1024;
            b->cap_t = ctx->last.num_triangles + ctx->last.num_triangles / 4 + 1024;
            b->sized = true;
            if (b->exec) {
                cudaGraphExecDestroy(b->exec);
                b->exec = nullptr;
            }
            if (b->graph) {
                cudaGraphDestroy(b->graph);
                b->graph = nullptr;
            }
        }
        return ISO_OK;
    }
    if ((s = ensure(ctx, ctx->mesh_v, 12 * b->cap_v)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->mesh_i, 12 * b->cap_t)) != ISO_OK) return s;
    if (b->exec && (b->graph_v != ctx->mesh_v.p || b->graph_i != ctx->mesh_i.p)) {
        cudaGraphExecDestroy(b->exec);
        cudaGraphDestroy(b->graph);
        b->exec = nullptr;
        b->graph = nullptr;
    }
    if (!b->exec) {
        cudaError_t e = cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "begin capture");
        const bool timing = ctx->timing;
        ctx->timing = false;  // no events inside the graph
        s = enqueue(b, false);
        ctx->timing = timing;
        cudaGraph_t g = nullptr;
        e = cudaStreamEndCapture(ctx->stream, &g);
        if (s != ISO_OK) {
            if (g) cudaGraphDestroy(g);
            return s;
        }
        if (e != cudaSuccess) return cuda_fail(ctx, e, "end capture");
        b->graph = g;
        e = cudaGraphInstantiate(&b->exec, g, 0);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "instantiate graph");
        b->graph_v = ctx->mesh_v.p;
        b->graph_i = ctx->mesh_i.p;
    }
    {
        StageTimer timer(ctx, ISO_STAGE_OTHER);
        cudaError_t e = cudaGraphLaunch(b->exec, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "graph launch");
    }
    ctx->launches += 6;
    s = finish(b, info);
    if (s == ISO_ERR_CAPACITY || ctx->last.num_vertices > b->cap_v || ctx->last.num_triangles > b->cap_t) {
        b->sized = false;  // grow and run eagerly
        return iso_batch_run(b, 0, info);
    }
    return s;
}

iso_status iso_batch_run_per_chunk(iso_batch* b, iso_mesh_info* info) {
    iso::NvtxRange nvtx_range("iso_batch_run_per_chunk");
    if (!b) return ISO_ERR_INVALID_ARG;
    iso_ctx* ctx = b->ctx;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    // each chunk through the single-grid path, then appended to the batch output
    std::vector<uint32_t> ext(4 * b->chunks.size());
    uint64_t nv = 0, nt = 0;
    std::vector<float> hv;
    std::vector<uint32_t> hi;
    if ((s = ensure(ctx, ctx->aux3, 12 * std::max<uint64_t>(b->cap_v, 1 << 20) + 12 * std::max<uint64_t>(b->cap_t, 1 << 20))) != ISO_OK)
        return s;
    uint64_t cap_v = ctx->aux3.bytes / 24, cap_t = ctx->aux3.bytes / 24;
    float* out_v = (float*)ctx->aux3.p;
    uint32_t* out_i = (uint32_t*)((char*)ctx->aux3.p + 12 * cap_v);
    for (size_t i = 0; i < b->chunks.size(); ++i) {
        const SampleGrid& g = b->sgrids[i];
        const uint32_t n = g.n;
        if ((s = launch_sample_grid(ctx, b->programs[b->chunks[i].prog], n, n, n + 1, g.inv, g.field, g.pitch,
                                    g.bits, true)) != ISO_OK)
            return s;
        Lattice L{n, n, n + 1, g.pitch, g.field, g.bits, g.W, g.inv, nullptr};
        iso_mesh_info mi;
        if ((s = mc_extract_lattice(ctx, L, 0, &mi)) != ISO_OK) return s;
        if (nv + mi.num_vertices > cap_v || nt + mi.num_triangles > cap_t)
            return fail(ctx, ISO_ERR_CAPACITY, "per-chunk output arena too small");
        cudaMemcpyAsync(out_v + 3 * nv, ctx->mesh_v.p, 12 * mi.num_vertices, cudaMemcpyDeviceToDevice, ctx->stream);
        cudaMemcpyAsync(out_i + 3 * nt, ctx->mesh_i.p, 12 * mi.num_triangles, cudaMemcpyDeviceToDevice, ctx->stream);
        ext[4 * i + 0] = (uint32_t)nv;
        ext[4 * i + 1] = (uint32_t)mi.num_vertices;
        ext[4 * i + 2] = (uint32_t)nt;
        ext[4 * i + 3] = (uint32_t)mi.num_triangles;
        nv += mi.num_vertices;
        nt += mi.num_triangles;
    }
    // hand the concatenated mesh over as the context's mesh
    if ((s = ensure(ctx, ctx->mesh_v, 12 * std::max<uint64_t>(nv, 1))) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->mesh_i, 12 * std::max<uint64_t>(nt, 1))) != ISO_OK) return s;
    cudaMemcpyAsync(ctx->mesh_v.p, out_v, 12 * nv, cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(ctx->mesh_i.p, out_i, 12 * nt, cudaMemcpyDeviceToDevice, ctx->stream);
    cudaMemcpyAsync(b->d_extents, ext.data(), 4 * ext.size(), cudaMemcpyHostToDevice, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "per-chunk run");
    uint64_t cells = 0;
    for (auto& c : b->chunks) cells += (uint64_t)(c.size - 1) * (c.size - 1) * c.size;
    ctx->last = iso_mesh_info{nv, nt, cells};
    ctx->last_flags = 0;
    ctx->last_vertex_floats = 3;
    if (info) *info = ctx->last;
    return ISO_OK;
}

iso_status iso_batch_run_per_chunk_async(iso_batch* b, iso_mesh_info* info) {
    iso::NvtxRange nvtx_range("iso_batch_run_per_chunk_async");
    if (!b) return ISO_ERR_INVALID_ARG;
    iso_ctx* ctx = b->ctx;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    if (!b->sized) return fail(ctx, ISO_ERR_INVALID_ARG, "run the batch once first (it sizes every chunk's output)");
    const uint32_t n_ch = (uint32_t)b->chunks.size();
    if (!b->d_solo_grids) {
        // every chunk as a grid of its own, chunk ids from 0
        std::vector<char> grids(mc_grid_bytes() * n_ch);
        b->solo_chunks.resize(n_ch);
        b->solo_cw.resize(n_ch);
        for (uint32_t i = 0; i < n_ch; ++i) {
            const SampleGrid& g = b->sgrids[i];
            Lattice L{g.n, g.n, g.n + 1, g.pitch, g.field, g.bits, g.W, g.inv, nullptr};
            mc_fill_grid(grids.data() + mc_grid_bytes() * i, L, 0, &b->solo_chunks[i], &b->solo_cw[i]);
        }
        cudaError_t e = cudaMalloc(&b->d_solo_grids, grids.size());
        if (e == cudaSuccess) e = cudaMemcpy(b->d_solo_grids, grids.data(), grids.size(), cudaMemcpyHostToDevice);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "per-chunk grids");
    }
    // each chunk's output place and size, from the last run of the batch
    std::vector<uint32_t> ext(4ull * n_ch);
    cudaError_t e = cudaMemcpyAsync(ext.data(), b->d_extents, 16ull * n_ch, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "chunk extents");
    const uint64_t nv = (uint64_t)ext[4ull * (n_ch - 1)] + ext[4ull * (n_ch - 1) + 1];
    const uint64_t nt = (uint64_t)ext[4ull * (n_ch - 1) + 2] + ext[4ull * (n_ch - 1) + 3];
    if ((s = ensure(ctx, ctx->mesh_v, 12 * std::max<uint64_t>(nv, 1))) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->mesh_i, 12 * std::max<uint64_t>(nt, 1))) != ISO_OK) return s;
    float* out_v = (float*)ctx->mesh_v.p;
    uint32_t* out_i = (uint32_t*)ctx->mesh_i.p;
    uint32_t* dummy_extents = (uint32_t*)(b->d_totals + 4);  // [0, 16) of the totals block's unused half
    uint64_t* totals = b->d_totals;
    // per chunk: its sampler, count, scan and emit, queued back to back
    for (uint32_t i = 0; i < n_ch; ++i) {
        const SampleGrid& g = b->sgrids[i];
        if ((s = launch_sample_grid(ctx, b->programs[b->chunks[i].prog], g.n, g.n, g.n + 1, g.inv, g.field, g.pitch,
                                    g.bits, true)) != ISO_OK)
            return s;
        if ((s = mc_extract_grids(ctx, (const char*)b->d_solo_grids + mc_grid_bytes() * i, 1, nullptr,
                                  b->solo_chunks[i], b->solo_cw[i], b->d_scratch, ext[4ull * i + 1],
                                  ext[4ull * i + 3], out_v + 3ull * ext[4ull * i], out_i + 3ull * ext[4ull * i + 2],
                                  dummy_extents, totals, false)) != ISO_OK)
            return s;
    }
    e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "per-chunk run");
    if ((s = read_device_errors(ctx)) != ISO_OK) return s;
    uint64_t cells = 0;
    for (auto& c : b->chunks) cells += (uint64_t)(c.size - 1) * (c.size - 1) * c.size;
    ctx->last = iso_mesh_info{nv, nt, cells};
    ctx->last_flags = 0;
    ctx->last_vertex_floats = 3;
    if (info) *info = ctx->last;
    return ISO_OK;
}

iso_status iso_batch_extents(iso_batch* b, uint32_t* extents) {
    if (!b || !extents) return ISO_ERR_INVALID_ARG;
    iso_ctx* ctx = b->ctx;
    cudaError_t e = cudaMemcpyAsync(extents, b->d_extents, 16ull * b->chunks.size(), cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, "extents");
}

iso_status iso_batch_autotune(iso_batch* b, const char* cache_path, uint32_t* chosen) {
    if (!b) return ISO_ERR_INVALID_ARG;
    iso_ctx* ctx = b->ctx;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    cudaDeviceProp prop;
    cudaGetDeviceProperties(&prop, ctx->device);
    // cached depths are for this sampler design on this GPU model
    const std::string gpu = std::string(prop.name) + " bricks";
    std::map<uint32_t, uint32_t> classes;  // size -> chunk count
    for (auto& c : b->chunks) classes[c.size]++;
    std::map<uint32_t, uint32_t> best;
    // cache lines: "<gpu>|<size>|<depth>"
    if (cache_path) {
        if (FILE* f = std::fopen(cache_path, "r")) {
            char line[512];
            while (std::fgets(line, sizeof(line), f)) {
                std::string l(line);
                size_t a = l.find('|'), c = l.rfind('|');
                if (a == std::string::npos || c == a) continue;
                if (l.substr(0, a) != gpu) continue;
                best[(uint32_t)std::stoul(l.substr(a + 1, c - a - 1))] = (uint32_t)std::stoul(l.substr(c + 1));
            }
            std::fclose(f);
        }
    }
    const uint32_t candidates[] = {4, 8, 16, 0};
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    std::vector<uint32_t> saved = b->slab;
    bool wrote = false;
    for (auto& cl : classes) {
        if (best.count(cl.first)) continue;
        float best_ms = 1e30f;
        uint32_t best_depth = 4;
        for (uint32_t d : candidates) {
            // time the sampler on this class's chunks only, slab depth d
            std::vector<std::pair<double, Tile>> t;
            for (uint32_t i = 0; i < b->chunks.size(); ++i) {
                if (b->chunks[i].size != cl.first) continue;
                chunk_tiles(i, cl.first, d, [&](const Tile& tl) { t.push_back({0.0, tl}); });
            }
            std::vector<Tile> tiles(t.size());
            for (size_t i = 0; i < t.size(); ++i) tiles[i] = t[i].second;
            Tile* d_t = nullptr;
            if (upload_tiles(tiles, &d_t) != cudaSuccess) {
                if (d_t) cudaFree(d_t);
                cudaGetLastError();
                return fail(ctx, ISO_ERR_OUT_OF_MEMORY, "autotune tiles");
            }
            float ms = 1e30f;
            for (int rep = 0; rep < 4; ++rep) {
                cudaEventRecord(e0, ctx->stream);
                launch_sampler(ctx, d_t, (uint32_t)tiles.size(), b->d_sgrids, b->d_next);
                cudaEventRecord(e1, ctx->stream);
                cudaEventSynchronize(e1);
                float t_ms = 0.0f;
                cudaEventElapsedTime(&t_ms, e0, e1);
                if (rep > 0) ms = std::min(ms, t_ms);
            }
            cudaFree(d_t);
            if (ms < best_ms) {
                best_ms = ms;
                best_depth = d;
            }
        }
        best[cl.first] = best_depth;
        wrote = true;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "autotune");
    if (cache_path && wrote) {
        if (FILE* f = std::fopen(cache_path, "a")) {
            for (auto& kv : best) std::fprintf(f, "%s|%u|%u\n", gpu.c_str(), kv.first, kv.second);
            std::fclose(f);
        }
    }
    for (size_t i = 0; i < b->chunks.size(); ++i) b->slab[i] = best[b->chunks[i].size];
    if (chosen) {
        size_t k = 0;
        for (auto& kv : best) {
            chosen[2 * k] = kv.first;
            chosen[2 * k + 1] = kv.second;
            ++k;
        }
    }
    (void)saved;
    return build_tiles(b);
}

}  // extern "C"
