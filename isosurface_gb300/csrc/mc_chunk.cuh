// Chunked marching-cubes passes (included by mc.cu inside iso::{anonymous}).
//
// A chunk is 32 consecutive cells of a row (x = 32c .. 32c+31); inside a
// grid, chunk id = row * CW + c with CW = ceil((nx-1)/32), which is the
// reference's (z, y, x) visit order.  A chunk's eight corner bit-vectors (bit
// i: corner k of cell 32c+i is inside) come from four sign-bit rows with
// funnel shifts, so activity and owned-vertex counts cost a few dozen bit
// operations per 32 cells.
//
// Offsets come in two forms.  Chunk mode (the block emit): pass 1 gives every
// chunk its exclusive prefix inside its range of 256 chunks plus each range's
// total; a one-block scan turns range totals into range offsets; chunk base =
// range offset + in-range prefix.  Several grids can be processed by one
// launch in this mode: each grid's chunks occupy a run of whole ranges of a
// global chunk index space, range_grid maps a range to its grid (a null map
// means one grid), and vertex indices are written relative to the grid's
// first vertex, so each grid gets its own mesh.  Segment mode (the cell emit,
// one grid): pass 1 writes one record per 32-chunk segment (prefix inside
// its range, own counts), each range's prefix inside its block of 8 ranges
// and each block's totals; the one-block scan runs over the block totals;
// segment base = block offset + in-block range prefix + in-range prefix.
// Corners, load_corners, case_at, chunk_valid, active_cells and owned_count
// are defined in mc.cu above the include.

constexpr uint32_t RANGE = 256;  // chunks per counting warp / per emit block
constexpr int RANGE_ROUNDS = RANGE / 32;

// q = n / d for n < 2^32, d < 2^31, with m = floor(2^64 / d) + 1 (d > 1)
struct FastDiv {
    uint32_t d;
    uint64_t m;
};
inline FastDiv make_fastdiv(uint32_t d) { return FastDiv{d, d > 1 ? (~0ull / d + 1) : 0ull}; }
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv& f) {
    return f.d == 1 ? n : (uint32_t)__umul64hi((uint64_t)n, f.m);
}

// One lattice: nx x ny x nz samples (sign bits + values, optional explicit
// positions) and where its chunks sit in the global chunk index space.
struct Grid {
    const uint32_t* bits;
    const float* values;
    const float4* positions;  // null: regular grid, point = (x, y, z) * inv
    uint64_t pitch;
    uint32_t W, CW, nx, ny, nz;
    FastDiv div_cw, div_ncy;
    float inv;
    uint32_t zoff;     // lattice z of layer 0 (a slab of a larger grid): positions and keys use z + zoff
    uint32_t chunk0;   // first global chunk id (a multiple of RANGE)
    uint32_t nchunks;  // CW * (ny-1) * (nz-1)
};

inline Grid make_grid(const Lattice& L, uint32_t chunk0) {
    Grid g;
    g.bits = L.bits;
    g.values = L.values;
    g.positions = L.positions;
    g.pitch = L.pitch;
    g.W = L.words_per_row;
    g.nx = L.nx;
    g.ny = L.ny;
    g.nz = L.nz;
    g.CW = (L.nx - 1 + 31) / 32;
    g.div_cw = make_fastdiv(g.CW);
    g.div_ncy = make_fastdiv(L.ny - 1);
    g.inv = L.inv;
    g.zoff = L.zoff;
    g.chunk0 = chunk0;
    g.nchunks = g.CW * (L.ny - 1) * (L.nz - 1);
    return g;
}

__device__ __forceinline__ uint32_t grid_of_range(const uint32_t* range_grid, uint32_t range) {
    return range_grid ? __ldg(range_grid + range) : 0u;
}

struct ChunkCountArgs {
    const Grid* grids;
    const uint32_t* range_grid;
    uint32_t chunks;   // global (padded) chunk count
    uint2* local;      // chunk mode: chunks + 1 (vertex, triangle) exclusive prefixes inside the range
    uint2* rangeagg;   // per range: (vertices, triangles)
    uint4* segs;       // segment mode: per 32 chunks (first vertex, first triangle) inside the range,
                       // (vertices, triangles); rangeagg then holds each range's prefix inside
                       // its block of 8 ranges and blockagg each block's totals
    uint2* blockagg;
};

// Segments of 32 chunks per warp in mc_cell_emit: a segment (two cell rows at
// 513^3) holds a dozen or two active cells, so a warp takes several and hands
// out their active cells together.
constexpr int EMIT_SEGS = 2;
constexpr int EMIT_CH = 32 * EMIT_SEGS;  // chunks per warp

// N chunks of a warp in shared memory: corner words (padded to 9 words, so
// that lanes reading different chunks hit different banks), active-cell masks
// and the exclusive prefix of their counts in chunk order.
template <int N>
struct ChunkStage {
    uint32_t q[N][9];
    uint32_t act[N];
    uint32_t excl[N];
    // the chunk holding active cell number kk (kk < the chunks' total): the
    // last one whose prefix is <= kk
    __device__ __forceinline__ uint32_t find(uint32_t kk) const {
        uint32_t j = 0;
#pragma unroll
        for (uint32_t step = N / 2; step > 0; step >>= 1)
            if (excl[j + step] <= kk) j += step;
        return j;
    }
};
using EmitChunks = ChunkStage<EMIT_CH>;

// Pass 1: per-chunk (SEG = false) or per-segment (32 chunks, SEG = true)
// counts and in-range prefixes.  One warp per range of 256 chunks, 32 per
// round (no barrier); the next round's corner words are loaded while this
// round is counted, so the loads' latency overlaps the counting.
#ifndef ISO_COUNT_BLOCKS
#define ISO_COUNT_BLOCKS 4  // resident blocks per SM the register budget is sized for (64 registers)
#endif
template <bool SEG>
__global__ void __launch_bounds__(256, ISO_COUNT_BLOCKS) mc_chunk_count(ChunkCountArgs A) {
    __shared__ uint8_t s_ntri[256];
    __shared__ uint16_t s_owned[8];
    __shared__ uint32_t s_tri[8][32];  // chunk mode, per warp: triangles of each of the round's chunks
    __shared__ ChunkStage<SEG ? 64 : 2> s_pair[8];  // segment mode, per warp: two rounds of chunks
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    pdl_wait();     // the grid record and the sign bits
    pdl_trigger();
    s_ntri[threadIdx.x] = iso_tri_count[threadIdx.x];
    if (threadIdx.x < 8) s_owned[threadIdx.x] = iso_owned_mask[threadIdx.x];
    __syncthreads();
    const uint32_t range = blockIdx.x * 8 + (threadIdx.x >> 5);
    const bool live = range * RANGE <= A.chunks;  // warp-uniform
    if (!SEG && !live) return;
    uint32_t agg_t = 0, agg_v = 0;
    if (live) {
        const Grid g = A.grids[grid_of_range(A.range_grid, min(range, A.chunks / RANGE - (A.chunks % RANGE == 0)))];
        const uint32_t ncx = g.nx - 1;
        // corner words of chunk ch (zeros outside the grid)
        auto fetch = [&](uint32_t ch, uint32_t& y, uint32_t& z, uint32_t& c, bool& in) {
            const uint32_t lc = ch - g.chunk0;
            in = ch < A.chunks && lc < g.nchunks;
            Corners q;
            if (in) {
                const uint32_t row = fdiv(lc, g.div_cw);
                c = lc - row * g.CW;
                z = fdiv(row, g.div_ncy);
                y = row - z * (g.ny - 1);
                q = load_corners(g.bits, g.W, g.ny, y, z, c);
            } else {
    #pragma unroll
                for (int k = 0; k < 8; ++k) q.k[k] = 0;
                y = z = c = 0;
            }
            return q;
        };
        uint32_t ny_, nz_, nc_;
        bool nin;
        uint32_t pair_total = 0, vr_first = 0;  // segment mode
        Corners qn = fetch(range * RANGE + lane, ny_, nz_, nc_, nin);
        for (int r = 0; r < RANGE_ROUNDS; ++r) {
            const uint32_t ch = range * RANGE + r * 32 + lane;
            const Corners q = qn;
            const uint32_t y = ny_, z = nz_, c = nc_;
            const bool in = nin;
            if (r + 1 < RANGE_ROUNDS) qn = fetch(ch + 32, ny_, nz_, nc_, nin);
            uint32_t v = 0;
            const uint32_t act = in ? active_cells(q, chunk_valid(c, ncx)) : 0u;
            if (act) {
                if (y > 0 && z > 0) {
                    // interior row: cells own edges 5 (k5^k6), 6 (k6^k7), 10 (k2^k6);
                    // the row's x == 0 cell also owns 7 (k7^k4) and 11 (k3^k7)
                    v = __popc((q.k[5] ^ q.k[6]) & act) + __popc((q.k[6] ^ q.k[7]) & act) + __popc((q.k[2] ^ q.k[6]) & act);
                    if (c == 0 && (act & 1u)) v += ((q.k[7] ^ q.k[4]) & 1u) + ((q.k[3] ^ q.k[7]) & 1u);
                } else {
                    const int cls = (y == 0 ? 2 : 0) | (z == 0 ? 4 : 0);
                    v = owned_count(q, act, s_owned[cls], s_owned[cls | 1], c == 0 ? 1u : 0u);
                }
            }
            if constexpr (SEG) {
                // two rounds (two segments) at a time: the chunks go to shared
                // memory, and the pair's active cells are handed out one per
                // lane in chunk order, their triangles summed per segment
                const uint32_t h = r & 1;
                ChunkStage<64>& P = s_pair[warp];
                uint32_t vr = 0;
                if (__any_sync(FULL, act != 0)) {
#pragma unroll
                    for (int k = 0; k < 8; ++k) P.q[32 * h + lane][k] = q.k[k];
                    P.act[32 * h + lane] = act;
                    const uint32_t n = __popc(act);
                    const uint32_t incl = warp_incl_scan(n, lane);
                    P.excl[32 * h + lane] = pair_total + incl - n;
                    pair_total += __shfl_sync(FULL, incl, 31);
                    vr = __reduce_add_sync(FULL, v);
                } else {
                    // no active cell in the round (most rounds): no corners to
                    // stage, no counts to scan (v is 0 without active cells);
                    // the chunk lookup never lands on a chunk without any
                    P.act[32 * h + lane] = 0;
                    P.excl[32 * h + lane] = pair_total;
                }
                if (h == 0) {
                    vr_first = vr;
                    continue;
                }
                __syncwarp();
                uint32_t t0 = 0, t1 = 0;
                for (uint32_t b0 = 0; b0 < pair_total; b0 += 32) {
                    const uint32_t kk = b0 + lane;
                    if (kk < pair_total) {
                        const uint32_t j = P.find(kk);
                        Corners cq;
#pragma unroll
                        for (int k = 0; k < 8; ++k) cq.k[k] = P.q[j][k];
                        const uint32_t t = s_ntri[case_at(cq, __fns(P.act[j], 0, (int)(kk - P.excl[j]) + 1))];
                        if (j < 32)
                            t0 += t;
                        else
                            t1 += t;
                    }
                }
                const uint32_t tr0 = __reduce_add_sync(FULL, t0), tr1 = __reduce_add_sync(FULL, t1);
                const uint32_t first = ch - lane - 32;  // the pair's first chunk
                if (lane == 0 && first < A.chunks) A.segs[first / 32] = make_uint4(agg_v, agg_t, vr_first, tr0);
                agg_v += vr_first;
                agg_t += tr0;
                if (lane == 0 && first + 32 < A.chunks) A.segs[first / 32 + 1] = make_uint4(agg_v, agg_t, vr, tr1);
                agg_v += vr;
                agg_t += tr1;
                pair_total = 0;
                __syncwarp();  // the pair's chunks are read before the next pair overwrites them
                continue;
            }
            // triangles: the round's active cells one per lane (in chunk order),
            // their counts summed back per chunk in shared memory
            s_tri[warp][lane] = 0;
            const uint32_t n = __popc(act);
            const uint32_t incl = warp_incl_scan(n, lane), excl = incl - n;
            const uint32_t total = __shfl_sync(FULL, incl, 31);
            __syncwarp();
            for (uint32_t b0 = 0; b0 < total; b0 += 32) {
                const uint32_t kk = b0 + lane;
                uint32_t src = 0;
    #pragma unroll
                for (uint32_t step = 16; step > 0; step >>= 1) {
                    const uint32_t cand = src + step;
                    const uint32_t e = __shfl_sync(FULL, excl, cand & 31);
                    if (cand < 32 && e <= kk) src = cand;
                }
                const uint32_t sact = __shfl_sync(FULL, act, src), sexcl = __shfl_sync(FULL, excl, src);
                Corners cq;
    #pragma unroll
                for (int k = 0; k < 8; ++k) cq.k[k] = __shfl_sync(FULL, q.k[k], src);
                if (kk < total) {
                    const uint32_t i = __fns(sact, 0, (int)(kk - sexcl) + 1);
                    atomicAdd(&s_tri[warp][src], (uint32_t)s_ntri[case_at(cq, i)]);
                }
            }
            __syncwarp();
            const uint32_t t = s_tri[warp][lane];
            __syncwarp();
            const uint32_t ti = warp_incl_scan(t, lane), vi = warp_incl_scan(v, lane);
            if (ch <= A.chunks) A.local[ch] = make_uint2(agg_v + vi - v, agg_t + ti - t);
            agg_t += __shfl_sync(FULL, ti, 31);
            agg_v += __shfl_sync(FULL, vi, 31);
        }
    }
    if (!SEG) {
        if (lane == 0 && range * RANGE < A.chunks) A.rangeagg[range] = make_uint2(agg_v, agg_t);
        return;
    }
    // segment mode: each range's exclusive prefix inside the block's eight
    // ranges, and the block's totals (scanned across blocks by mc_range_scan)
    __shared__ uint2 s_agg[8];
    if (lane == 0) s_agg[warp] = range * RANGE < A.chunks ? make_uint2(agg_v, agg_t) : make_uint2(0, 0);
    __syncthreads();
    if (threadIdx.x < 8) {  // thread w: range blockIdx.x * 8 + w
        const uint32_t r = blockIdx.x * 8 + threadIdx.x;
        uint2 pre = make_uint2(0, 0);
        for (uint32_t w = 0; w < threadIdx.x; ++w) {
            pre.x += s_agg[w].x;
            pre.y += s_agg[w].y;
        }
        if (r * RANGE < A.chunks) A.rangeagg[r] = pre;
        if (threadIdx.x == 7) A.blockagg[blockIdx.x] = make_uint2(pre.x + s_agg[7].x, pre.y + s_agg[7].y);
    }
}

// Exclusive scan of the range totals (one block).  Each thread holds
// SCAN_ITEMS consecutive ranges per pass (all loaded before any is used), so
// 8K ranges take one pass of one block scan.  rangepre[nr] and totals
// receive the grand totals; local[chunks] (chunk mode) is cleared when
// `chunks` starts a range that no warp counted.
constexpr int SCAN_ITEMS = 8;

__global__ void __launch_bounds__(1024) mc_range_scan(const uint2* rangeagg, uint32_t nr, uint2* rangepre,
                                                      uint64_t* totals, uint2* local, uint32_t chunks, uint32_t* err) {
    __shared__ uint64_t s_wv[32], s_wt[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    pdl_wait();     // the counting pass's totals
    pdl_trigger();
    uint64_t carry_t = 0, carry_v = 0;
    for (uint32_t base = 0; base < nr; base += 1024 * SCAN_ITEMS) {
        const uint32_t i0 = base + threadIdx.x * SCAN_ITEMS;
        uint2 a[SCAN_ITEMS];
        uint32_t sv = 0, st = 0;  // a range holds at most 256 * 32 * 5 triangles
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            a[k] = i0 + k < nr ? rangeagg[i0 + k] : make_uint2(0, 0);
            sv += a[k].x;
            st += a[k].y;
        }
        uint64_t vi = sv, ti = st;
        for (int o = 1; o < 32; o <<= 1) {
            const uint64_t tv = __shfl_up_sync(FULL, vi, o), tt = __shfl_up_sync(FULL, ti, o);
            if (lane >= o) {
                vi += tv;
                ti += tt;
            }
        }
        if (lane == 31) {
            s_wv[warp] = vi;
            s_wt[warp] = ti;
        }
        __syncthreads();
        if (warp == 0) {  // inclusive scan of the 32 warp totals
            uint64_t wv = s_wv[lane], wt = s_wt[lane];
            for (int o = 1; o < 32; o <<= 1) {
                const uint64_t tv = __shfl_up_sync(FULL, wv, o), tt = __shfl_up_sync(FULL, wt, o);
                if (lane >= o) {
                    wv += tv;
                    wt += tt;
                }
            }
            s_wv[lane] = wv;
            s_wt[lane] = wt;
        }
        __syncthreads();
        uint64_t ev = carry_v + (warp ? s_wv[warp - 1] : 0) + vi - sv;
        uint64_t et = carry_t + (warp ? s_wt[warp - 1] : 0) + ti - st;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; ++k) {
            if (i0 + k < nr) {
                if (ev > 0xFFFFFFFFull || et > 0xFFFFFFFFull) atomicOr(err, DERR_CAPACITY);
                rangepre[i0 + k] = make_uint2((uint32_t)ev, (uint32_t)et);
            }
            ev += a[k].x;
            et += a[k].y;
        }
        carry_v += s_wv[31];
        carry_t += s_wt[31];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        totals[0] = carry_t;
        totals[1] = carry_v;
        rangepre[nr] = make_uint2((uint32_t)carry_v, (uint32_t)carry_t);
        if (local && chunks % RANGE == 0) local[chunks] = make_uint2(0, 0);
    }
}

struct ChunkEmitArgs {
    const Grid* grids;
    const uint32_t* range_grid;
    uint32_t chunks;
    const uint2* local;
    const uint2* rangepre;
    float* out_v;
    uint32_t* out_i;
    uint64_t* out_k;
    uint64_t cap_v, cap_t;
    uint32_t* err;
    uint32_t* edge_id;  // mc_cell_emit: vertex id per lattice edge, keyed by (upper end point * 3 + axis)
    // mc_cell_emit / mc_resolve_ids: page-locked host buffers (device-side
    // pointers, null: none) that also receive the mesh when all of it fits
    // both them and the device buffers (`totals` = triangles, vertices)
    float* host_v;
    uint32_t* host_i;
    uint64_t host_cap_v, host_cap_t;
    const uint64_t* totals;
    // mc_cell_emit: rangepre holds each range's prefix inside its block of 8
    // ranges, blockpre each block's exclusive prefix
    const uint2* blockpre;
};

// whether this launch copies the mesh to the host buffers
__device__ __forceinline__ bool mesh_to_host(const float* host, const uint64_t* totals, uint64_t host_cap_v,
                                             uint64_t host_cap_t, uint64_t cap_v, uint64_t cap_t) {
    if (!host) return false;
    const uint64_t nt = totals[0], nv = totals[1];
    return nv <= host_cap_v && nt <= host_cap_t && nv <= cap_v && nt <= cap_t;
}

__device__ __forceinline__ uint2 chunk_base(const ChunkEmitArgs& A, uint32_t ch) {
    const uint2 l = __ldg(&A.local[ch]);
    const uint2 b = __ldg(&A.rangepre[ch / RANGE]);
    return make_uint2(l.x + b.x, l.y + b.y);
}

// Pass 2.  Block b emits the chunks of range b (one grid).  Every non-owned
// edge of a cell in those chunks is owned by a cell in chunk ch-1, ch-CW or
// ch-CW-1 (same layer) or ch-S, ch-S-1, ch-S-CW, ch-S-CW-1 (layer below,
// S = CW*(ny-1)), so the block caches the corner vectors and vertex bases of
// the bands R1 = [c0-CW-1, c0+256) and R2 = R1 - S (grid-local chunk ids) in
// shared memory.  Active cells are compacted in chunk order and processed one
// per thread in rounds of 256, with block scans giving each cell's output
// offsets; each distinct edge of a cell is resolved to its vertex id once.
constexpr int EMIT_LIST_CAP = 256 * 32;

struct EmitTables {
    uint8_t tri_count[256];
    uint8_t edge_count[256];
    uint16_t edge_mask[256];
    uint64_t tri_edges[256];
    uint64_t edge_order[256];
    uint64_t tri_slot[256];
    uint64_t rank[2][256];  // classes 0 (interior) and 1 (x == 0)
    uint16_t owned[8];
};

size_t block_emit_smem(uint32_t CW) {
    const size_t span = RANGE + CW + 1;
    return ((sizeof(EmitTables) + 15) & ~(size_t)15) + 2 * span * 8 * 4 + 2 * span * 4 + EMIT_LIST_CAP * 2;
}

__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* s_w, uint32_t* total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t inc = warp_incl_scan(v, lane);
    if (lane == 31) s_w[warp] = inc;
    __syncthreads();
    uint32_t before = 0, all = 0;
#pragma unroll
    for (int w = 0; w < 8; ++w) {
        const uint32_t t = s_w[w];
        if (w < warp) before += t;
        all += t;
    }
    __syncthreads();
    *total = all;
    return before + inc - v;
}

__device__ __forceinline__ uint32_t rank_of(const EmitTables& tb, int cls, uint32_t cs, uint32_t e) {
    const uint64_t w = cls < 2 ? tb.rank[cls][cs] : iso_owned_rank[cls][cs];
    return (uint32_t)(w >> (4 * e)) & 15u;
}

__global__ void __launch_bounds__(256) mc_block_emit(ChunkEmitArgs A, uint32_t max_cw) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_w[8], s_w2[8];
    EmitTables& tb = *reinterpret_cast<EmitTables*>(smem);
    const Grid g = A.grids[grid_of_range(A.range_grid, blockIdx.x)];
    const uint32_t CW = g.CW, ncx = g.nx - 1, ncy = g.ny - 1;
    const int span = RANGE + (int)CW + 1;
    const int span_max = RANGE + (int)max_cw + 1;
    uint32_t* q1 = reinterpret_cast<uint32_t*>(smem + ((sizeof(EmitTables) + 15) & ~(size_t)15));
    uint32_t* q2 = q1 + span_max * 8;
    uint32_t* vb1 = q2 + span_max * 8;
    uint32_t* vb2 = vb1 + span_max;
    uint16_t* list = reinterpret_cast<uint16_t*>(vb2 + span_max);
    const uint32_t gc0 = blockIdx.x * RANGE;           // global chunk id of the block's first chunk
    const uint32_t c0 = gc0 - g.chunk0;                 // grid-local
    if (c0 >= g.nchunks) return;                        // padding range
    const int64_t S = (int64_t)CW * ncy;
    const int64_t r1 = (int64_t)c0 - CW - 1, r2 = r1 - S;
    const uint2 bb = chunk_base(A, gc0);
    const uint32_t c_end = min(c0 + RANGE, g.nchunks);
    if (chunk_base(A, g.chunk0 + c_end).y == bb.y) return;  // no triangle in the block
    const uint32_t grid_v0 = chunk_base(A, g.chunk0).x;     // first vertex of this grid's mesh
    for (int i = threadIdx.x; i < 256; i += blockDim.x) {
        tb.tri_count[i] = iso_tri_count[i];
        tb.edge_count[i] = iso_edge_count[i];
        tb.edge_mask[i] = iso_edge_mask[i];
        tb.tri_edges[i] = iso_tri_edges[i];
        tb.edge_order[i] = iso_edge_order[i];
        tb.tri_slot[i] = iso_tri_slot[i];
        tb.rank[0][i] = iso_owned_rank[0][i];
        tb.rank[1][i] = iso_owned_rank[1][i];
    }
    if (threadIdx.x < 8) tb.owned[threadIdx.x] = iso_owned_mask[threadIdx.x];
    for (int i = threadIdx.x; i < 2 * span; i += 256) {
        const bool first = i < span;
        const int64_t ch = first ? r1 + i : r2 + (i - span);
        if (ch < 0 || ch >= (int64_t)g.nchunks) continue;
        const uint32_t chu = (uint32_t)ch;
        const uint32_t row = fdiv(chu, g.div_cw);
        const uint32_t c = chu - row * CW;
        const uint32_t z = fdiv(row, g.div_ncy);
        const Corners q = load_corners(g.bits, g.W, g.ny, row - z * ncy, z, c);
        uint32_t* dst = first ? q1 + i * 8 : q2 + (i - span) * 8;
#pragma unroll
        for (int k = 0; k < 8; ++k) dst[k] = q.k[k];
        (first ? vb1 : vb2)[first ? i : i - span] = chunk_base(A, g.chunk0 + chu).x - grid_v0;
    }
    __syncthreads();

    // compact the block's active cells, in chunk order
    const uint32_t mych = c0 + threadIdx.x;
    uint32_t act = 0;
    if (mych < g.nchunks) {
        Corners q;
#pragma unroll
        for (int k = 0; k < 8; ++k) q.k[k] = q1[(CW + 1 + threadIdx.x) * 8 + k];
        act = active_cells(q, chunk_valid(mych - fdiv(mych, g.div_cw) * CW, ncx));
    }
    uint32_t nlist;
    uint32_t pos = block_excl_scan(__popc(act), s_w, &nlist);
    while (act) {
        const uint32_t i = __ffs(act) - 1;
        act &= act - 1;
        list[pos++] = (uint16_t)((threadIdx.x << 5) | i);
    }
    __syncthreads();

    const bool explicit_pos = g.positions != nullptr;
    uint32_t vcarry = bb.x, tcarry = bb.y;  // global offsets
    for (uint32_t r0 = 0; r0 < nlist; r0 += 256) {
        const uint32_t j = r0 + threadIdx.x;
        const bool have = j < nlist;
        uint32_t x = 0, y = 0, z = 0, cs = 0, nown = 0, nt = 0;
        int cls = 0;
        if (have) {
            const uint32_t ent = list[j];
            const uint32_t t = ent >> 5, i = ent & 31;
            const uint32_t ch = c0 + t;
            const uint32_t row = fdiv(ch, g.div_cw);
            z = fdiv(row, g.div_ncy);
            y = row - z * ncy;
            x = 32 * (ch - row * CW) + i;
            uint32_t cs_ = 0;
#pragma unroll
            for (int k = 0; k < 8; ++k) cs_ |= ((q1[(CW + 1 + t) * 8 + k] >> i) & 1u) << k;
            cs = cs_;
            cls = (x == 0 ? 1 : 0) | (y == 0 ? 2 : 0) | (z == 0 ? 4 : 0);
            nown = __popc((uint32_t)tb.edge_mask[cs] & tb.owned[cls]);
            nt = tb.tri_count[cs];
        }
        uint32_t vtot, ttot;
        const uint32_t vpre = block_excl_scan(nown, s_w, &vtot);
        const uint32_t tpre = block_excl_scan(nt, s_w2, &ttot);
        if (have) {
            const uint32_t own = tb.owned[cls];
            const uint32_t vstart = vcarry + vpre;  // global vertex slot
            const uint64_t ord = tb.edge_order[cs];
            const uint32_t ne = tb.edge_count[cs];
            uint32_t ids[12];  // grid-local vertex ids by first-use rank
            uint32_t r = 0;
            for (uint32_t k = 0; k < ne; ++k) {
                const uint32_t e = (uint32_t)(ord >> (4 * k)) & 15u;
                if ((own >> e) & 1u) {
                    // owned: this cell writes the vertex (first use in visit order)
                    const uint32_t u = iso_edge_connection[e][0], v = iso_edge_connection[e][1];
                    const uint32_t ux = x + iso_corners[u][0], uy = y + iso_corners[u][1], uz = z + iso_corners[u][2];
                    const uint32_t vx = x + iso_corners[v][0], vy = y + iso_corners[v][1], vz = z + iso_corners[v][2];
                    const float fa = __ldg(g.values + ((size_t)uz * g.ny + uy) * g.pitch + ux);
                    const float fb = __ldg(g.values + ((size_t)vz * g.ny + vy) * g.pitch + vx);
                    float pax, pay, paz, pbx, pby, pbz;
                    if (explicit_pos) {
                        const float4 qa = __ldg(g.positions + ((size_t)uz * g.ny + uy) * g.nx + ux);
                        const float4 qb = __ldg(g.positions + ((size_t)vz * g.ny + vy) * g.nx + vx);
                        pax = qa.x; pay = qa.y; paz = qa.z; pbx = qb.x; pby = qb.y; pbz = qb.z;
                    } else {
                        pax = (float)ux * g.inv; pay = (float)uy * g.inv; paz = (float)(uz + g.zoff) * g.inv;
                        pbx = (float)vx * g.inv; pby = (float)vy * g.inv; pbz = (float)(vz + g.zoff) * g.inv;
                    }
                    // Signed::find_crossing_point (distance.rs:64-69)
                    const float delta = fb - fa;
                    const float tt = (delta == 0.0f) ? 0.5f : -fa / delta;
                    const float omt = 1.0f - tt;
                    const uint32_t vid = vstart + r;
                    if (vid < A.cap_v) {
                        A.out_v[3 * (size_t)vid + 0] = pax * omt + pbx * tt;
                        A.out_v[3 * (size_t)vid + 1] = pay * omt + pby * tt;
                        A.out_v[3 * (size_t)vid + 2] = paz * omt + pbz * tt;
                        if (A.out_k) {
                            const uint32_t lx = x + c_edge_lo[e][0], ly = y + c_edge_lo[e][1], lz = z + c_edge_lo[e][2];
                            A.out_k[2 * (size_t)vid] = (((uint64_t)(lz + g.zoff) * g.ny + ly) * g.nx + lx) * 3 + c_edge_axis[e];
                            A.out_k[2 * (size_t)vid + 1] = 0;
                        }
                    } else {
                        atomicOr(A.err, DERR_CAPACITY);
                    }
                    ids[k] = vid - grid_v0;
                    ++r;
                    continue;
                }
                // not owned: the lowest (z, y, x) cell adjacent to the lattice edge owns it
                const uint32_t ax = c_edge_axis[e];
                const uint32_t lx = x + c_edge_lo[e][0], ly = y + c_edge_lo[e][1], lz = z + c_edge_lo[e][2];
                uint32_t ox = lx, oy = ly, oz = lz, d1, d2;
                if (ax != 0) ox = lx > 0 ? lx - 1 : 0;
                if (ax != 1) oy = ly > 0 ? ly - 1 : 0;
                if (ax != 2) oz = lz > 0 ? lz - 1 : 0;
                if (ax == 0) { d1 = ly - oy; d2 = lz - oz; }
                else if (ax == 1) { d1 = lx - ox; d2 = lz - oz; }
                else { d1 = lx - ox; d2 = ly - oy; }
                const uint32_t oe = c_local_edge[ax][d1 + 2 * d2];
                const uint32_t oc = ox >> 5, oi = ox & 31;
                const int64_t och = ((int64_t)oz * ncy + oy) * CW + oc;
                const uint32_t* oq;
                uint32_t obase;
                if (och >= r1 && och < r1 + span) {
                    oq = q1 + (och - r1) * 8;
                    obase = vb1[och - r1];
                } else if (och >= r2 && och < r2 + span) {
                    oq = q2 + (och - r2) * 8;
                    obase = vb2[och - r2];
                } else {
                    atomicOr(A.err, DERR_CAPACITY);
                    oq = q1;
                    obase = 0;
                }
                Corners q;
#pragma unroll
                for (int kk = 0; kk < 8; ++kk) q.k[kk] = oq[kk];
                const uint32_t sel = (1u << oi) - 1u;
                const int ocls = (ox == 0 ? 1 : 0) | (oy == 0 ? 2 : 0) | (oz == 0 ? 4 : 0);
                uint32_t prior;
                if (oy > 0 && oz > 0) {
                    // interior row: cells own edges 5 (k5^k6), 6 (k6^k7), 10 (k2^k6);
                    // the row's x == 0 cell also owns 7 (k7^k4) and 11 (k3^k7)
                    prior = __popc((q.k[5] ^ q.k[6]) & sel) + __popc((q.k[6] ^ q.k[7]) & sel) +
                            __popc((q.k[2] ^ q.k[6]) & sel);
                    if (oc == 0 && oi > 0) prior += ((q.k[7] ^ q.k[4]) & 1u) + ((q.k[3] ^ q.k[7]) & 1u);
                } else {
                    const int rcls = (oy == 0 ? 2 : 0) | (oz == 0 ? 4 : 0);
                    prior = owned_count(q, sel, tb.owned[rcls], tb.owned[rcls | 1], oc == 0 ? 1u : 0u);
                }
                ids[k] = obase + prior + rank_of(tb, ocls, case_at(q, oi), oe);
            }
            // triangles (march_cube, marching_cubes_impl.rs:102-117)
            const uint64_t slot = tb.tri_slot[cs];
            const size_t tstart = (size_t)tcarry + tpre;
            if (tstart + nt <= A.cap_t) {
                for (uint32_t k = 0; k < 3 * nt; ++k) A.out_i[3 * tstart + k] = ids[(slot >> (4 * k)) & 15u];
            } else {
                atomicOr(A.err, DERR_CAPACITY);
            }
        }
        vcarry += vtot;
        tcarry += ttot;
    }
}

// One vertex on lattice edge (pa, pb) with values (fa, fb): the crossing
// point (Signed::find_crossing_point, distance.rs:64-69), its optional lattice
// edge key (lower end point * 3 + axis), and its grid-local id in the edge map
// under ``key``.
__device__ __forceinline__ void put_vertex(const ChunkEmitArgs& A, const Grid& g, float fa, float fb, float pax,
                                           float pay, float paz, float pbx, float pby, float pbz, uint32_t vid,
                                           uint32_t key, uint32_t grid_v0, uint32_t lx, uint32_t ly, uint32_t lz,
                                           uint32_t ax) {
    const float delta = fb - fa;
    const float tt = (delta == 0.0f) ? 0.5f : -fa / delta;
    const float omt = 1.0f - tt;
    if (vid < A.cap_v) {
        A.out_v[3 * (size_t)vid + 0] = pax * omt + pbx * tt;
        A.out_v[3 * (size_t)vid + 1] = pay * omt + pby * tt;
        A.out_v[3 * (size_t)vid + 2] = paz * omt + pbz * tt;
        if (A.out_k) {
            A.out_k[2 * (size_t)vid] = (((uint64_t)(lz + g.zoff) * g.ny + ly) * g.nx + lx) * 3 + ax;
            A.out_k[2 * (size_t)vid + 1] = 0;
        }
    } else {
        atomicOr(A.err, DERR_CAPACITY);
    }
    A.edge_id[key] = vid - grid_v0;
}

// Active cell number kk (in chunk order) of the warp's chunks starting at
// grid chunk rc; every lane calls it, have = kk < total.
struct SegCell {
    uint32_t x, y, z, cs, nown, nt;
    int cls;
    bool have;
    uint4 pk;  // interior cells: the case's packed entry (iso_case_pack)
};

__device__ __forceinline__ SegCell seg_cell(const Grid& g, uint32_t rc, uint32_t kk, uint32_t total,
                                            const EmitChunks& S) {
    SegCell c{0, 0, 0, 0, 0, 0, 0, kk < total, make_uint4(0, 0, 0, 0)};
    if (!c.have) return c;
    const uint32_t j = S.find(kk);
    Corners cq;
#pragma unroll
    for (int k = 0; k < 8; ++k) cq.k[k] = S.q[j][k];
    const uint32_t i = __fns(S.act[j], 0, (int)(kk - S.excl[j]) + 1);
    const uint32_t cch = rc + j;
    const uint32_t row = fdiv(cch, g.div_cw);
    c.z = fdiv(row, g.div_ncy);
    c.y = row - c.z * (g.ny - 1);
    c.x = 32 * (cch - row * g.CW) + i;
    c.cs = case_at(cq, i);
    c.cls = (c.x == 0 ? 1 : 0) | (c.y == 0 ? 2 : 0) | (c.z == 0 ? 4 : 0);
    if (c.cls == 0) {
        c.pk = __ldg(reinterpret_cast<const uint4*>(&iso_case_pack[c.cs]));
        c.nown = __popc(c.pk.z & 0x460u);  // owned edges 5, 6, 10
        c.nt = (c.pk.z >> 12) & 7u;
    } else {
        c.nown = __popc((uint32_t)__ldg(&iso_edge_mask[c.cs]) & __ldg(&iso_owned_mask[c.cls]));
        c.nt = __ldg(&iso_tri_count[c.cs]);
    }
    return c;
}

// The vertices and triangles of one round of cells (every lane calls it).
// koff (lane e < 12): the edge-map key of cell edge e relative to 3 * (corner
// 0's lattice point).
__device__ __forceinline__ void emit_cells(const ChunkEmitArgs& A, const Grid& g, const SegCell& c, uint32_t vstart,
                                           uint32_t tstart, uint32_t koff, uint32_t grid_v0) {
    uint32_t own = 0, cell = 0;
    uint64_t tedges = 0;
    if (c.have) {
        cell = (c.z * g.ny + c.y) * g.nx + c.x;  // lattice point of corner 0
        if (c.cls == 0) {
            own = c.pk.z & 0x460u;
            tedges = ((uint64_t)c.pk.y << 32) | c.pk.x;
        } else {
            own = (uint32_t)__ldg(&iso_edge_mask[c.cs]) & __ldg(&iso_owned_mask[c.cls]);
            tedges = __ldg(&iso_tri_edges[c.cs]);
        }
    }
    if (own) {
        // owned edges: this cell creates their vertices, numbered by
        // first use in the cell's visit order (rank table)
        if (c.cls == 0) {
            // interior cell: its owned edges are among 5, 6 and 10, the
            // three edges ending at corner 6 = (x+1, y+1, z+1); all their
            // values are loaded before any vertex is formed
            const float* v6 = g.values + ((size_t)(c.z + 1) * g.ny + (c.y + 1)) * g.pitch + (c.x + 1);
            const bool e5 = (own >> 5) & 1u, e6 = (own >> 6) & 1u, e10 = (own >> 10) & 1u;
            const float f6 = __ldg(v6);
            const float f5 = e5 ? __ldg(v6 - g.pitch) : 0.0f;                    // corner 5
            const float f7 = e6 ? __ldg(v6 - 1) : 0.0f;                          // corner 7
            const float f2 = e10 ? __ldg(v6 - (size_t)g.ny * g.pitch) : 0.0f;    // corner 2
            const float X0 = (float)c.x * g.inv, X1 = (float)(c.x + 1) * g.inv;
            const float Y0 = (float)c.y * g.inv, Y1 = (float)(c.y + 1) * g.inv;
            const float Z0 = (float)(c.z + g.zoff) * g.inv, Z1 = (float)(c.z + 1 + g.zoff) * g.inv;
            const uint32_t k6 = 3 * (cell + g.nx * (g.ny + 1) + 1);  // corner 6's key base
            if (e5)  // corners 5 -> 6, y axis
                put_vertex(A, g, f5, f6, X1, Y0, Z1, X1, Y1, Z1, vstart + (c.pk.z >> 16 & 15u), k6 + 1, grid_v0,
                           c.x + 1, c.y, c.z + 1, 1);
            if (e6)  // corners 6 -> 7, x axis
                put_vertex(A, g, f6, f7, X1, Y1, Z1, X0, Y1, Z1, vstart + (c.pk.z >> 20 & 15u), k6 + 0, grid_v0,
                           c.x, c.y + 1, c.z + 1, 0);
            if (e10)  // corners 2 -> 6, z axis
                put_vertex(A, g, f2, f6, X1, Y1, Z0, X1, Y1, Z1, vstart + (c.pk.z >> 24 & 15u), k6 + 2, grid_v0,
                           c.x + 1, c.y + 1, c.z, 2);
        } else {
            const uint64_t rk = __ldg(&iso_owned_rank[c.cls][c.cs]);
            for (uint32_t m = own; m; m &= m - 1) {
                const uint32_t e = __ffs(m) - 1;
                const uint32_t ax = __ldg(&g_edge_axis[e]);
                const uint32_t lx = c.x + __ldg(&g_edge_lo[e][0]), ly = c.y + __ldg(&g_edge_lo[e][1]),
                               lz = c.z + __ldg(&g_edge_lo[e][2]);
                const uint32_t hx = lx + (ax == 0), hy = ly + (ax == 1), hz = lz + (ax == 2);
                const uint32_t u = __ldg(&iso_edge_connection[e][0]), v = __ldg(&iso_edge_connection[e][1]);
                const uint32_t ux = c.x + __ldg(&iso_corners[u][0]), uy = c.y + __ldg(&iso_corners[u][1]),
                               uz = c.z + __ldg(&iso_corners[u][2]);
                const uint32_t vx = c.x + __ldg(&iso_corners[v][0]), vy = c.y + __ldg(&iso_corners[v][1]),
                               vz = c.z + __ldg(&iso_corners[v][2]);
                const float fa = __ldg(g.values + ((size_t)uz * g.ny + uy) * g.pitch + ux);
                const float fb = __ldg(g.values + ((size_t)vz * g.ny + vy) * g.pitch + vx);
                put_vertex(A, g, fa, fb, (float)ux * g.inv, (float)uy * g.inv, (float)(uz + g.zoff) * g.inv,
                           (float)vx * g.inv, (float)vy * g.inv, (float)(vz + g.zoff) * g.inv,
                           vstart + (uint32_t)(rk >> (4 * e) & 15u), ((hz * g.ny + hy) * g.nx + hx) * 3 + ax,
                           grid_v0, lx, ly, lz, ax);
            }
        }
    }
    // triangles (march_cube, marching_cubes_impl.rs:102-117) as edge-map
    // keys, resolved to vertex ids once every owner has written its ids
    const bool tfit = (uint64_t)tstart + c.nt <= A.cap_t;
    if (c.have && !tfit) atomicOr(A.err, DERR_CAPACITY);
    const uint32_t kmax = __reduce_max_sync(FULL, 3 * c.nt);
    for (uint32_t k = 0; k < kmax; ++k) {
        const uint32_t ko = __shfl_sync(FULL, koff, (uint32_t)(tedges >> (4 * k)) & 15u);
        if (k < 3 * c.nt && tfit) A.out_i[3 * (size_t)tstart + k] = 3 * cell + ko;
    }
}

// Pass 2, cell-parallel, for one lattice given by values alone (no explicit
// sample positions) whose edge count fits 32 bits.  Warp = EMIT_SEGS
// consecutive segments of 32 chunks, whose first vertex and triangle come
// from pass 1's segment records.  Lane = chunk, once per segment: corner
// words and active cells, staged in shared memory with their count prefix.
// The chunks' active cells are then handed out 32 at a time in chunk order
// (lane = cell: the owning chunk by a binary search over the prefix, the bit
// by __fns), so lanes stay busy however the active cells are spread.  A
// cell's own offsets are the warp's base plus a running warp scan of
// owned-vertex and triangle counts in cell order (the reference's emission
// order).  Every owned vertex records its id in a dense per-lattice-edge map,
// and triangles are written as map keys; mc_resolve_ids then replaces each
// key by the id its owner recorded (the map needs no initialisation: every
// crossing edge has an owner, and only crossing edges are referenced).  Keys
// are 3 * (upper end point) + axis, so the (at most three) edges an interior
// cell owns, which all end at its corner 6, share one 12-byte slot.
__global__ void __launch_bounds__(256, 5) mc_cell_emit(ChunkEmitArgs A, const uint4* segs, uint32_t nsegs) {
    __shared__ EmitChunks s_ch[8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    pdl_trigger();
    const uint32_t seg0 = (blockIdx.x * 8 + warp) * EMIT_SEGS;  // the warp's first segment
    if (seg0 >= nsegs) return;
    // the staging below reads only the sign bits and the grid record, which
    // the counting pass's predecessors wrote: it overlaps the counting pass
    const Grid g = A.grids[0];
    const uint32_t rc = seg0 * 32, c_end = min(rc + (uint32_t)EMIT_CH, g.nchunks);
    EmitChunks& S = s_ch[warp];
    // lane = chunk, EMIT_SEGS times: corner bit-vectors, active cells, prefix
    uint32_t total = 0;
#pragma unroll
    for (int h = 0; h < EMIT_SEGS; ++h) {
        const uint32_t ch = rc + 32 * h + lane;
        Corners q;
        uint32_t act = 0;
        if (ch < c_end) {
            const uint32_t row = fdiv(ch, g.div_cw);
            const uint32_t cc = ch - row * g.CW;
            const uint32_t z = fdiv(row, g.div_ncy);
            q = load_corners(g.bits, g.W, g.ny, row - z * (g.ny - 1), z, cc);
            act = active_cells(q, chunk_valid(cc, g.nx - 1));
        } else {
#pragma unroll
            for (int k = 0; k < 8; ++k) q.k[k] = 0;
        }
        if (__any_sync(FULL, act != 0)) {
#pragma unroll
            for (int k = 0; k < 8; ++k) S.q[32 * h + lane][k] = q.k[k];
            S.act[32 * h + lane] = act;
            const uint32_t n = __popc(act);
            const uint32_t incl = warp_incl_scan(n, lane);
            S.excl[32 * h + lane] = total + incl - n;
            total += __shfl_sync(FULL, incl, 31);
        } else {
            // no active cell in the segment: nothing to stage (the chunk
            // lookup never lands on a chunk without active cells)
            S.act[32 * h + lane] = 0;
            S.excl[32 * h + lane] = total;
        }
    }
    if (total == 0) return;  // no active cell: no vertex, no triangle
    pdl_wait();              // the counts and their scan
    // records: (first vertex, first triangle) in the range, (vertices, triangles)
    const uint4 sr = __ldg(&segs[seg0]);
    uint32_t nv_w = sr.z;
#pragma unroll
    for (int h = 1; h < EMIT_SEGS; ++h)
        if (seg0 + h < nsegs) nv_w += __ldg(&segs[seg0 + h]).z;
    const uint32_t range = seg0 / (RANGE / 32);  // EMIT_SEGS divides the 8 segments of a range
    const uint2 rin = __ldg(&A.rangepre[range]), rb = __ldg(&A.blockpre[range / 8]);
    const uint32_t vbase = rb.x + rin.x + sr.x, tbase = rb.y + rin.y + sr.y;
    __syncwarp();
    uint32_t koff = 0;
    if (lane < 12) {
        const uint32_t ax = __ldg(&g_edge_axis[lane]);
        const uint32_t hx = __ldg(&g_edge_lo[lane][0]) + (ax == 0), hy = __ldg(&g_edge_lo[lane][1]) + (ax == 1),
                       hz = __ldg(&g_edge_lo[lane][2]) + (ax == 2);
        koff = 3 * (hx + g.nx * (hy + g.ny * hz)) + ax;
    }
    uint32_t vcarry = vbase, tcarry = tbase;  // global offsets of the next cell's outputs
    for (uint32_t b0 = 0; b0 < total; b0 += 32) {
        const SegCell c = seg_cell(g, rc, b0 + lane, total, S);
        const uint32_t vi = warp_incl_scan(c.nown, lane), ti = warp_incl_scan(c.nt, lane);
        const uint32_t vstart = vcarry + vi - c.nown, tstart = tcarry + ti - c.nt;
        vcarry += __shfl_sync(FULL, vi, 31);
        tcarry += __shfl_sync(FULL, ti, 31);
        emit_cells(A, g, c, vstart, tstart, koff, 0u);
    }
    if (mesh_to_host(A.host_v, A.totals, A.host_cap_v, A.host_cap_t, A.cap_v, A.cap_t)) {
        // the segments' vertices, just written by this warp, in whole lines
        // to the host (the warp's own stores are ordered before its reads)
        __syncwarp();
        const size_t f0 = 3 * (size_t)vbase, f1 = f0 + 3 * (size_t)nv_w;
        for (size_t f = f0 + lane; f < f1; f += 32) A.host_v[f] = __ldcg(A.out_v + f);
    }
}

// Triangle corners: edge-map key -> vertex id recorded by the owner, for the
// 3 * min(triangles, capacity) corners written (the count is read on the
// device, so no host round trip is needed).  Four corners per thread and
// step, so four independent gathers are in flight; the resolved corners also
// go to the page-locked host buffer when the mesh is delivered there.  Keys
// outside the map (corners of triangles an emit without room skipped) are
// left alone.
__global__ void __launch_bounds__(256) mc_resolve_ids(uint32_t* __restrict__ idx, const uint64_t* totals,
                                                      uint64_t cap_t, const uint32_t* __restrict__ edge_id,
                                                      uint32_t nedges, uint32_t* host_i, uint64_t host_cap_v,
                                                      uint64_t host_cap_t, uint64_t cap_v) {
    pdl_wait();  // the emitted keys and the edge map
    const uint64_t n = 3 * min(totals[0], cap_t);
    const bool to_host = mesh_to_host(reinterpret_cast<const float*>(host_i), totals, host_cap_v, host_cap_t, cap_v,
                                      cap_t);
    const uint64_t n4 = n / 4, stride = (uint64_t)gridDim.x * blockDim.x;
    const uint64_t t0 = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    uint4* __restrict__ p = reinterpret_cast<uint4*>(idx);
    for (uint64_t i = t0; i < n4; i += stride) {
        uint4 v = p[i];
        const uint32_t a = v.x < nedges ? __ldg(edge_id + v.x) : v.x;
        const uint32_t b = v.y < nedges ? __ldg(edge_id + v.y) : v.y;
        const uint32_t c = v.z < nedges ? __ldg(edge_id + v.z) : v.z;
        const uint32_t d = v.w < nedges ? __ldg(edge_id + v.w) : v.w;
        v = make_uint4(a, b, c, d);
        p[i] = v;
        if (to_host) reinterpret_cast<uint4*>(host_i)[i] = v;
    }
    const uint64_t k = 4 * n4 + t0;  // the last n % 4 corners
    if (k < n) {
        uint32_t v = idx[k];
        if (v < nedges) idx[k] = v = __ldg(edge_id + v);
        if (to_host) host_i[k] = v;
    }
}

// grid of mc_resolve_ids for at most 3 * cap_t corners
inline unsigned resolve_blocks(uint64_t cap_t) {
    return (unsigned)std::min<uint64_t>(std::max<uint64_t>((3 * cap_t / 4 + 255) / 256, 1), 16384);
}

// Per-grid mesh extents: (first vertex, vertex count, first triangle, triangle count).
__global__ void mc_grid_extents(const Grid* grids, uint32_t ngrids, const uint2* local, const uint2* rangepre,
                                uint4* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ngrids) return;
    const Grid g = grids[i];
    const uint32_t a = g.chunk0, b = g.chunk0 + g.nchunks;
    const uint2 la = local[a], ra = rangepre[a / RANGE], lb = local[b], rb = rangepre[b / RANGE];
    const uint32_t v0 = la.x + ra.x, t0 = la.y + ra.y, v1 = lb.x + rb.x, t1 = lb.y + rb.y;
    out[i] = make_uint4(v0, v1 - v0, t0, t1 - t0);
}
