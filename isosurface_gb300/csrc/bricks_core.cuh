// Culled sampling of a general program for marching cubes (and, at the end,
// the plain sampler of every point): the device code, written so that it
// also compiles on its own under NVRTC (no includes: the
// library includes it after its own headers, the run-time compiler after a
// prelude of fixed-width integer types and vm_math.cuh).
//
// Marching cubes reads a sample's value only at the ends of crossing edges
// (sign change between lattice neighbours one step `inv` apart), and both
// ends of such an edge lie within lip * inv of zero when the program's value
// is lip-Lipschitz in the sample point.  A sub-brick of 8 (x) x 4 (y) x 4 (z)
// points whose centre value v satisfies |v| > lip * h + lip * inv (h: the
// distance from the centre to its farthest point; plus rounding slack) holds
// no such end: all its samples have v's sign and no value of it is ever
// read.  Such a sub-brick gets sign bits only; every sample of the others is
// evaluated with the program's evaluator, so every value written is
// bit-identical to the full sampler's, and so is every sign bit.
//
// For a hard union of translated primitives (at most 64) each sub-brick also
// keeps only the primitives that can attain the minimum in it: primitive i's
// values over the sub-brick lie within lip * h of d_i(centre), so i is
// dropped when d_i - lip * h exceeds min_j (d_j + lip * h); the minimum over
// the kept ones equals the minimum over all.
//
// Work is cut in tiles: all x, rows [y0, y1), layers [z0, z1), y0 and z0
// multiples of 4, at most BRICK_MAX sub-bricks.  One thread classifies one
// sub-brick.  A group of four sub-bricks along x (32 x 4 x 4 points, one
// sign word in each of 16 rows) that is wholly decided gets its sign words
// at once; in a mixed group the decided sub-bricks get their sign bytes and
// every sample of the mixed ones is evaluated, four mixed sub-bricks to a
// warp (eight lanes each, one sign byte per row), so that no lane idles on a
// decided sub-brick.  Two schedules:
//  * one lattice (brick_classify + brick_rows): one block per tile
//    classifies and appends its mixed sub-bricks to a list; a persistent
//    grid then samples the list, so the evaluation is spread evenly however
//    the surface falls;
//  * many small lattices (brick_tile, the chunk batch): a block takes whole
//    tiles from a work queue and samples its own mixed sub-bricks from a list
//    in shared memory.
//
// The evaluator `Ev` provides value(p) and, for pruned unions, prunable(),
// nprims(), point(p) (the point after a leading domain map), prim(i, q) and
// value_kept(keep, p).
#pragma once

namespace iso {

constexpr uint32_t BRICK_MAX = 1024;        // sub-bricks per tile
constexpr uint32_t BRICK_PRUNE_MAX = 64;    // primitives a keep mask covers
constexpr uint32_t BRICK_ERR_CAPACITY = 2u;  // error bit: a list ran out of room
enum : uint32_t { BRICK_MIXED = 0, BRICK_OUT = 1, BRICK_IN = 2 };

struct BrickLattice {
    float lip;    // Lipschitz bound of the program's value in the sample point
    float slack;  // rounding slack of two values the evaluator computes
    uint32_t nx, ny, nz;  // samples per axis
    float inv;            // lattice step in sample coordinates
    float* field;
    uint64_t pitch;
    uint32_t* bits;
    uint32_t W;     // sign words per row
    uint32_t zoff;  // lattice z of layer 0 (a slab of a larger lattice)
    float reach_steps;  // values are needed within this many lattice steps' worth of change of zero
};

// One tile: the lattice and its rows / layers.
struct BrickTile {
    BrickLattice g;
    uint32_t y0, y1, z0, z1;
};

// A mixed sub-brick: tile * BRICK_MAX + sub-brick, and the primitives it keeps.
struct BrickTask {
    uint32_t tile_sb, unused;
    uint64_t keep;
};

// The tiles of one lattice: 4 layers x `rows` rows each.
struct GridTiles {
    BrickLattice g;
    uint32_t rows, ytiles;
    __device__ __forceinline__ BrickTile tile(uint32_t t) const {
        const uint32_t y0 = (t % ytiles) * rows, z0 = 4 * (t / ytiles);
        return BrickTile{g, y0, min(y0 + rows, g.ny), z0, min(z0 + 4, g.nz)};
    }
};

// OR of a 64-bit mask over the warp (every lane calls it).
__device__ __forceinline__ uint64_t warp_or64(uint64_t m) {
    const uint32_t lo = __reduce_or_sync(0xFFFFFFFFu, (uint32_t)m);
    const uint32_t hi = __reduce_or_sync(0xFFFFFFFFu, (uint32_t)(m >> 32));
    return ((uint64_t)hi << 32) | lo;
}

// Sub-bricks of a tile covering `rows` rows and `layers` layers.
__host__ __device__ __forceinline__ uint32_t brick_count(uint32_t W, uint32_t rows, uint32_t layers) {
    return 4 * W * ((rows + 3) / 4) * ((layers + 3) / 4);
}

// Class and kept primitives of every sub-brick of a tile, into shared memory
// (every thread of the block calls it; no barrier at the end).
template <class Ev>
__device__ __forceinline__ void brick_classes(const Ev& ev, const BrickTile& T, uint8_t* s_cls, uint64_t* s_keep) {
    const BrickLattice& g = T.g;
    const uint32_t SX = 4 * g.W, SY = (T.y1 - T.y0 + 3) / 4, SZ = (T.z1 - T.z0 + 3) / 4;
    const uint32_t nsb = SX * SY * SZ;
    const bool cull = g.lip > 0.0f;
    const bool prune = cull && ev.prunable();
    // both ends of a crossing edge lie within lip * inv of zero (rounded up);
    // a caller may need values further out (reach_steps > 1)
    const float reach = g.lip * g.inv * g.reach_steps * (1.0f + 1.0f / 1024.0f) + g.slack;
    for (uint32_t s = threadIdx.x; s < nsb; s += blockDim.x) {
        uint32_t cls = BRICK_MIXED;
        uint64_t keep = ~0ull;
        if (cull) {
            const uint32_t sx = s % SX, sy = (s / SX) % SY, sz = s / (SX * SY);
            const uint32_t xa = 8 * sx, ya = T.y0 + 4 * sy, za = T.z0 + 4 * sz;
            if (xa >= g.nx) {
                cls = BRICK_OUT;  // no samples: sign bits stay clear
            } else {
                const uint32_t xb = min(xa + 7, g.nx - 1), yb = min(ya + 3, T.y1 - 1), zb = min(za + 3, T.z1 - 1);
                const float hx = 0.5f * (float)(xb - xa), hy = 0.5f * (float)(yb - ya), hz = 0.5f * (float)(zb - za);
                const V3 c = v3(((float)xa + hx) * g.inv, ((float)ya + hy) * g.inv, ((float)(za + g.zoff) + hz) * g.inv);
                // the largest change of any value over the sub-brick, rounded up
                const float spread = g.lip * sqrtf((hx * hx + hy * hy) + hz * hz) * g.inv * (1.0f + 1.0f / 1024.0f) +
                                     g.slack;
                float v;
                if (prune) {
                    const V3 q = ev.point(c);
                    const uint32_t n = ev.nprims();
                    float upper = __int_as_float(0x7F800000);  // +infinity
                    v = 0.0f;
                    for (uint32_t i = 0; i < n; ++i) {
                        const float d = ev.prim(i, q);
                        v = (i == 0) ? d : fminf(v, d);
                        upper = fminf(upper, d + spread);
                    }
                    keep = 0;
                    for (uint32_t i = 0; i < n; ++i)
                        if (!(ev.prim(i, q) - spread > upper)) keep |= 1ull << i;
                } else {
                    v = ev.value(c);
                }
                if (v - spread > reach) cls = BRICK_OUT;
                else if (v + spread < -reach) cls = BRICK_IN;
            }
        }
        s_cls[s] = (uint8_t)cls;
        s_keep[s] = keep;
    }
}

// Sign word of a wholly decided group: its sub-bricks' classes, bits past
// the row's last sample clear.
__device__ __forceinline__ uint32_t decided_word(uint32_t cls4, uint32_t nx, uint32_t w) {
    uint32_t word = 0;
    for (uint32_t j = 0; j < 4; ++j)
        if (((cls4 >> (8 * j)) & 0xFFu) == BRICK_IN) word |= 0xFFu << (8 * j);
    const uint32_t valid = nx - 32 * w;  // samples of this word (> 0)
    return valid < 32 ? word & ((1u << valid) - 1u) : word;
}

// The sign byte (8 samples from x = 8 sx) of a decided sub-brick.
__device__ __forceinline__ uint8_t decided_byte(uint32_t cls, uint32_t nx, uint32_t sx) {
    if (cls != BRICK_IN || 8 * sx >= nx) return 0;
    const uint32_t valid = nx - 8 * sx;
    return valid < 8 ? (uint8_t)((1u << valid) - 1u) : (uint8_t)0xFFu;
}

// The sign bits of group gi of tile T (four sub-bricks along x, one sign
// word in each of 16 rows), written by one thread: a wholly decided group
// gets its words; in a mixed group the decided sub-bricks get their bytes
// and the mixed ones are left to brick_quad.  Returns the mask of mixed
// sub-bricks (bit j: sub-brick 4 gi + j).
__device__ __forceinline__ uint32_t brick_group_bits(const BrickTile& T, uint32_t gi, const uint8_t* s_cls) {
    const BrickLattice& g = T.g;
    const uint32_t SY = (T.y1 - T.y0 + 3) / 4;
    const uint32_t w = gi % g.W, gy = (gi / g.W) % SY, gz = gi / (g.W * SY);
    uint32_t cls4 = 0, mixed = 0;
    for (uint32_t j = 0; j < 4; ++j) {
        const uint32_t c = s_cls[4 * gi + j];
        cls4 |= c << (8 * j);
        if (c == BRICK_MIXED) mixed |= 1u << j;
    }
    const uint32_t word = decided_word(cls4, g.nx, w);
    for (uint32_t r = 0; r < 16; ++r) {
        const uint32_t y = T.y0 + 4 * gy + (r & 3), z = T.z0 + 4 * gz + (r >> 2);
        if (y >= T.y1 || z >= T.z1) continue;
        uint32_t* at = g.bits + ((uint64_t)z * g.ny + y) * g.W + w;
        if (!mixed) {
            *at = word;
        } else {
            for (uint32_t j = 0; j < 4; ++j)
                if (!((mixed >> j) & 1u))
                    reinterpret_cast<uint8_t*>(at)[j] = decided_byte((cls4 >> (8 * j)) & 0xFFu, g.nx, 4 * w + j);
        }
    }
    return mixed;
}

// The 16 rows of up to four mixed sub-bricks, one per eight lanes: lane l
// samples x = 8 sx + l % 8 of sub-brick `sb` of tile `T` (both its own; sb
// = ~0u: none) and the eight lanes' signs go out as one byte of the row's
// sign word.  `keep` (the same in every lane) holds every primitive any of
// the sub-bricks keeps.  Every lane of the warp calls it.
template <class Ev>
__device__ __forceinline__ void brick_quad(const Ev& ev, const BrickTile& T, uint32_t sb, uint64_t keep) {
    const BrickLattice& g = T.g;
    const uint32_t lane = threadIdx.x & 31;
    const bool have = sb != 0xFFFFFFFFu;
    uint32_t sx = 0, ya = 0, za = 0;
    if (have) {
        const uint32_t SX = 4 * g.W, SY = (T.y1 - T.y0 + 3) / 4;
        sx = sb % SX;
        ya = T.y0 + 4 * ((sb / SX) % SY);
        za = T.z0 + 4 * (sb / (SX * SY));
    }
    const uint32_t x = 8 * sx + (lane & 7);
    const bool prune = g.lip > 0.0f && ev.prunable();
    for (uint32_t r = 0; r < 16; ++r) {
        const uint32_t y = ya + (r & 3), z = za + (r >> 2);
        const bool row_ok = have && y < T.y1 && z < T.z1;
        const uint64_t row = (uint64_t)z * g.ny + y;
        bool inside = false;
        if (row_ok && x < g.nx) {
            const V3 p = v3((float)x * g.inv, (float)y * g.inv, (float)(z + g.zoff) * g.inv);
            const float v = prune ? ev.value_kept(keep, p) : ev.value(p);
            g.field[row * g.pitch + x] = v;
            inside = !(v > 0.0f);
        }
        const uint32_t b = __ballot_sync(0xFFFFFFFFu, inside);
        if (row_ok && (lane & 7) == 0)
            reinterpret_cast<uint8_t*>(g.bits + row * g.W + sx / 4)[sx % 4] = (uint8_t)(b >> (lane & ~7u));
    }
}

// Classify one tile, write its decided sign bits and list its mixed
// sub-bricks (every thread of the block calls it).
template <class Ev>
__device__ __forceinline__ void brick_classify_tile(const Ev& ev, const BrickTile& T, uint32_t tile, uint8_t* s_cls,
                                                    uint64_t* s_keep, BrickTask* list, uint32_t* count,
                                                    uint32_t cap, uint32_t* err) {
    brick_classes(ev, T, s_cls, s_keep);
    __syncthreads();
    const uint32_t groups = brick_count(T.g.W, T.y1 - T.y0, T.z1 - T.z0) / 4, lane = threadIdx.x & 31;
    for (uint32_t gb = 0; gb < groups; gb += blockDim.x) {
        const uint32_t gi = gb + threadIdx.x;
        const uint32_t mixed = gi < groups ? brick_group_bits(T, gi, s_cls) : 0u;
        // warp-aggregated append of the mixed sub-bricks
        const uint32_t n = __popc(mixed);
        uint32_t incl = n;
        for (uint32_t d = 1; d < 32; d <<= 1) {
            const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= d) incl += o;
        }
        const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
        if (total) {
            uint32_t base = 0;
            if (lane == 31) base = atomicAdd(count, total);
            base = __shfl_sync(0xFFFFFFFFu, base, 31) + incl - n;
            for (uint32_t m = mixed; m; m &= m - 1, ++base) {
                const uint32_t sb = 4 * gi + (uint32_t)(__ffs(m) - 1);
                if (base < cap) list[base] = BrickTask{tile * BRICK_MAX + sb, 0, s_keep[sb]};
                else atomicOr(err, BRICK_ERR_CAPACITY);
            }
        }
    }
}

// Sample a whole tile in the block: classes, decided sign bits, then the
// mixed sub-bricks four to a warp from a list in shared memory (every thread
// of the block calls it).
template <class Ev>
__device__ __forceinline__ void brick_tile(const Ev& ev, const BrickTile& T, uint8_t* s_cls, uint64_t* s_keep,
                                           uint32_t* s_list, uint32_t* s_n) {
    if (threadIdx.x == 0) *s_n = 0;
    brick_classes(ev, T, s_cls, s_keep);
    __syncthreads();
    const uint32_t groups = brick_count(T.g.W, T.y1 - T.y0, T.z1 - T.z0) / 4;
    for (uint32_t gi = threadIdx.x; gi < groups; gi += blockDim.x) {
        uint32_t mixed = brick_group_bits(T, gi, s_cls);
        if (mixed) {
            uint32_t at = atomicAdd(s_n, (uint32_t)__popc(mixed));
            for (; mixed; mixed &= mixed - 1) s_list[at++] = 4 * gi + (uint32_t)(__ffs(mixed) - 1);
        }
    }
    __syncthreads();
    const uint32_t n = *s_n, lane = threadIdx.x & 31;
    for (uint32_t q = 4 * (threadIdx.x >> 5); q < n; q += 4 * (blockDim.x >> 5)) {
        const uint32_t e = q + (lane >> 3);
        const uint32_t sb = e < n ? s_list[e] : 0xFFFFFFFFu;
        const uint64_t keep = warp_or64(e < n ? s_keep[sb] : 0ull);
        brick_quad(ev, T, sb, keep);
    }
}

// The bodies of the two single-lattice kernels (Tiles: a type with
// `BrickTile tile(uint32_t) const` on the device; blocks of 256 threads).
template <class Tiles, class Ev>
__device__ __forceinline__ void brick_classify_body(const Ev& ev, const Tiles& tiles, BrickTask* list,
                                                    uint32_t* count, uint32_t cap, uint32_t* err) {
    __shared__ uint8_t s_cls[BRICK_MAX];
    __shared__ uint64_t s_keep[BRICK_MAX];
    brick_classify_tile(ev, tiles.tile(blockIdx.x), blockIdx.x, s_cls, s_keep, list, count, cap, err);
}

// The listed mixed sub-bricks, four to a warp, over a persistent grid.
template <class Tiles, class Ev>
__device__ __forceinline__ void brick_rows_body(const Ev& ev, const Tiles& tiles, const BrickTask* list,
                                                const uint32_t* count, uint32_t cap) {
    const uint32_t n = min(*count, cap), lane = threadIdx.x & 31;
    const uint32_t warps = gridDim.x * (blockDim.x >> 5);
    for (uint32_t q = 4 * (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)); q < n; q += 4 * warps) {
        const uint32_t e = q + (lane >> 3);
        BrickTask k{0, 0, 0};
        if (e < n) k = list[e];
        const uint64_t keep = warp_or64(k.keep);
        brick_quad(ev, tiles.tile(k.tile_sb / BRICK_MAX), e < n ? k.tile_sb % BRICK_MAX : 0xFFFFFFFFu, keep);
    }
}

// The plain sampler (every point, nothing culled; the lattice's culling
// fields unused): warp gw of the lattice's W * ny * nz takes 32 consecutive
// points of one row, writes their values and, by ballot, the row's sign word.
template <class Ev>
__device__ __forceinline__ void field_warp(const Ev& ev, const BrickLattice& g, uint64_t gw) {
    if (gw >= (uint64_t)g.W * g.ny * g.nz) return;  // warp-uniform
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t w = (uint32_t)(gw % g.W);
    const uint64_t row = gw / g.W;
    const uint32_t y = (uint32_t)(row % g.ny), z = (uint32_t)(row / g.ny);
    const uint32_t x = 32 * w + lane;
    bool inside = false;
    if (x < g.nx) {
        const float v = ev.value(v3((float)x * g.inv, (float)y * g.inv, (float)(z + g.zoff) * g.inv));
        g.field[row * g.pitch + x] = v;
        inside = !(v > 0.0f);
    }
    const uint32_t b = __ballot_sync(0xFFFFFFFFu, inside);
    if (lane == 0) g.bits[row * g.W + w] = b;
}

}  // namespace iso
