// Grid sampling: the sample loops of PrimalGrid::traverse
// (src/traversal/primal_grid.rs:44-70) as kernels that write the f32 field
// and, with warp ballots, the packed sign bits (bit set iff !(v > 0),
// classify_corners, marching_cubes_impl.rs:26-37) that the marching-cubes
// passes classify from.  launch_sample_grid picks one of three samplers:
// for the extractors (near_only) on a hard union of spheres, the per-tile
// sphere culling below; on another program with a Lipschitz bound and a
// lattice of at least one tile per SM, the culled sampler of bricks_core.cuh
// (compiled for the program by jit.cu when it can be, else interpreted);
// otherwise every point (field_warp): for a full field with the program's
// compiled evaluator when it has one (jit.cu), else interpreted
// (sample_generic).
//
// Point (x, y, z) sits at (x*inv, y*inv, z*inv), inv = 1/(size-1) in f32, as
// in the reference.  Built with -fmad=false: the values are bit-identical to
// the reference's f32 evaluation.
#include <cuda_runtime.h>

#include <algorithm>
#include <utility>

#include "bricks.cuh"
#include "internal.h"
#include "vm.cuh"

namespace iso {
namespace {

constexpr uint32_t FULL = 0xFFFFFFFFu;

// One warp per (32-point chunk, row): the interpreter at every point
// (field_warp, bricks_core.cuh).
__global__ void __launch_bounds__(256) sample_generic(VmEval ev, BrickLattice g) {
    field_warp(ev, g, (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5));
}

// Union of spheres, hard min, optionally behind a domain map.  Each block
// samples a 32 x 8 x TZ tile of points; it first keeps only the spheres that
// can attain the minimum somewhere in the tile:
//   lower_i = dist(c_i, tile box) - r_i - margin
//   upper_i = maxdist(c_i, tile corners) - r_i + margin
//   keep i  iff lower_i <= min_j upper_j
// A dropped sphere's value exceeds the kept minimum at every point of the
// tile (the margin covers f32 rounding of both bounds and values), and min is
// exact, so the field equals the full fold over all spheres bit for bit.
constexpr int TZ = 16;

struct SetArgs {
    const float* spheres;  // n x (cx, cy, cz, r)
    uint32_t n;
    bool domain;
    float sx, sy, sz, ox, oy, oz;
    uint32_t nx, ny, nz;
    float inv;
    float* field;
    uint64_t pitch;
    uint32_t* bits;
    uint32_t W;
    // near-only mode: values are written only where |v| <= reach (a world
    // distance at least one lattice step plus rounding slack); signs everywhere
    bool near_only;
    float reach;
    uint32_t zoff;  // global lattice z of layer 0 (a slab of a larger grid)
};

__device__ __forceinline__ float world(float g, float s, float o, bool dom) { return dom ? g * s + o : g; }

// Thresholds that decide a sample from its squared distance s to a sphere
// (s = (dx*dx + dy*dy) + dz*dz in f32, as vector.rs's length computes it):
//   T: the largest f32 s with sqrt_rn(s) <= r, so sqrt(s) - r <= 0, i.e. the
//      sample is inside this sphere, exactly when s <= T (f32 subtraction of
//      finite values keeps the sign of the exact difference);
//   U: sqrt(s) - r <= reach implies s <= U (a rounded-up bound);
//   L: s < L implies sqrt(s) - r < -reach (a rounded-down bound, -1 if none).
// A sample whose value lies within reach of zero has some s <= U and no
// s < L; only those samples need their exact value (see sphere_column).
__device__ __forceinline__ float4 sphere_thresholds(float r, float reach) {
    float T = -1.0f;
    if (r >= 0.0f) {
        T = r * r;
        while (T > 0.0f && sqrtf(T) > r) T = nextafterf(T, 0.0f);
        for (int i = 0; i < 16; ++i) {  // fl(r*r) is within a few ulps of the bound
            const float up = nextafterf(T, 3.0e38f);
            if (sqrtf(up) > r) break;
            T = up;
        }
    }
    const float hi = fmaxf(r + reach, 0.0f);
    const float U = hi * hi * 1.0001f + 1e-30f;
    const float lo = r - reach;
    const float L = lo > 0.0f ? lo * lo * 0.9999f : -1.0f;
    return make_float4(T, U, L, 0.0f);
}

__device__ __forceinline__ uint32_t lane_incl_scan(uint32_t v, int lane) {
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(FULL, v, o);
        if (lane >= o) v += t;
    }
    return v;
}

// Near-only mode, one warp on 32 columns (lane = x) of row y, layers z0..z1
// (at most TZ): the sign of every sample from the thresholds, collected as the
// layers' sign words in lanes 0..z1-z0 and stored once; each lane notes its
// samples within reach (some sphere with s <= U and none with s < L) in a bit
// mask, and after the layers the warp evaluates those samples 32 at a time
// (lane = sample, found by a shuffle search over the lanes' counts) with the
// same fold as the full field.  (dx*dx + dy*dy) is shared by a column and is
// exactly len_sq's first partial sum.
template <int N>
__device__ __forceinline__ void near_column(const SetArgs& A, const float* dxy, const float* cz, const float* cr,
                                            const float* T, const float* U, const float* L, uint32_t x, uint32_t y,
                                            uint32_t z0, uint32_t z1, bool valid, int lane, uint32_t wx) {
    const uint32_t nzt = z1 - z0 + 1;
    const float pzl = world((float)((z0 + lane) + A.zoff) * A.inv, A.sz, A.oz, A.domain);  // lane k: layer z0 + k
    uint32_t nearmask = 0, word = 0;
    auto layer = [&](uint32_t k) {
        const float pz = __shfl_sync(FULL, pzl, k);
        bool in = false, hi = false, deep = false;
#pragma unroll
        for (int i = 0; i < N; ++i) {
            const float dz = pz - cz[i];
            const float sq = dxy[i] + dz * dz;
            in |= sq <= T[i];
            hi |= sq <= U[i];
            deep |= sq < L[i];
        }
        nearmask |= (uint32_t)(valid && hi && !deep) << k;
        const uint32_t b = __ballot_sync(FULL, valid && in);
        if ((uint32_t)lane == k) word = b;
    };
#pragma unroll 4
    for (uint32_t k = 0; k < nzt; ++k) layer(k);
    if ((uint32_t)lane < nzt) A.bits[((size_t)(z0 + lane) * A.ny + y) * A.W + wx] = word;
    const uint32_t cnt = __popc(nearmask);
    const uint32_t incl = lane_incl_scan(cnt, lane), excl = incl - cnt;
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    for (uint32_t b0 = 0; b0 < total; b0 += 32) {
        const uint32_t kk = b0 + lane;
        uint32_t src = 0;
#pragma unroll
        for (uint32_t step = 16; step > 0; step >>= 1) {
            const uint32_t cand = src + step;
            const uint32_t e = __shfl_sync(FULL, excl, cand & 31);
            if (cand < 32 && e <= kk) src = cand;
        }
        const uint32_t smask = __shfl_sync(FULL, nearmask, src), sexcl = __shfl_sync(FULL, excl, src);
        float sdxy[N];
#pragma unroll
        for (int i = 0; i < N; ++i) sdxy[i] = __shfl_sync(FULL, dxy[i], src);
        if (kk < total) {
            const uint32_t z = z0 + __fns(smask, 0, (int)(kk - sexcl) + 1);
            const float pz = world((float)(z + A.zoff) * A.inv, A.sz, A.oz, A.domain);
            float dz = pz - cz[0];
            float v = sqrtf(sdxy[0] + dz * dz) - cr[0];
#pragma unroll
            for (int i = 1; i < N; ++i) {
                dz = pz - cz[i];
                v = fminf(v, sqrtf(sdxy[i] + dz * dz) - cr[i]);
            }
            A.field[((size_t)z * A.ny + y) * A.pitch + (x - lane + src)] = v;
        }
    }
}

// One thread's z column with the N kept spheres in registers (one warp on 32
// columns of a row).  Full mode: the exact value of every sample.  Near-only
// mode: near_column.
template <int N>
__device__ __forceinline__ void sphere_column(const SetArgs& A, const float4* keep, const float4* thr, float px,
                                              float py, uint32_t x, uint32_t y, uint32_t z0, uint32_t z1, bool valid,
                                              int lane, uint32_t wx) {
    float dxy[N], cz[N], cr[N], T[N], U[N], L[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const float4 c = keep[i];
        const float dx = px - c.x, dy = py - c.y;
        dxy[i] = dx * dx + dy * dy;
        cz[i] = c.z;
        cr[i] = c.w;
        if (A.near_only) {
            const float4 t = thr[i];
            T[i] = t.x;
            U[i] = t.y;
            L[i] = t.z;
        }
    }
    if (A.near_only) {
        near_column<N>(A, dxy, cz, cr, T, U, L, x, y, z0, z1, valid, lane, wx);
        return;
    }
#pragma unroll 2
    for (uint32_t z = z0; z <= z1; ++z) {
        const float pz = world((float)(z + A.zoff) * A.inv, A.sz, A.oz, A.domain);
        const size_t row = (size_t)z * A.ny + y;
        float dz = pz - cz[0];
        float v = sqrtf(dxy[0] + dz * dz) - cr[0];
#pragma unroll
        for (int i = 1; i < N; ++i) {
            dz = pz - cz[i];
            v = fminf(v, sqrtf(dxy[i] + dz * dz) - cr[i]);
        }
        if (valid) A.field[row * A.pitch + x] = v;
        const uint32_t b = __ballot_sync(0xFFFFFFFFu, valid && !(v > 0.0f));
        if (lane == 0) A.bits[row * A.W + wx] = b;
    }
}

// The samples of column (x, y), layers z0..z1, from the nk kept spheres;
// sign words go to word wx of each row.
__device__ __forceinline__ void sample_column(const SetArgs& A, const float4* keep, const float4* thr, uint32_t nk,
                                              float px, float py, uint32_t x, uint32_t y, uint32_t z0, uint32_t z1,
                                              bool valid, int lane, uint32_t wx) {
    switch (nk) {
    case 1: sphere_column<1>(A, keep, thr, px, py, x, y, z0, z1, valid, lane, wx); return;
    case 2: sphere_column<2>(A, keep, thr, px, py, x, y, z0, z1, valid, lane, wx); return;
    case 3: sphere_column<3>(A, keep, thr, px, py, x, y, z0, z1, valid, lane, wx); return;
    case 4: sphere_column<4>(A, keep, thr, px, py, x, y, z0, z1, valid, lane, wx); return;
    default: break;
    }
    for (uint32_t z = z0; z <= z1; ++z) {
        const float pz = world((float)(z + A.zoff) * A.inv, A.sz, A.oz, A.domain);
        float v = 0.0f;
        for (uint32_t i = 0; i < nk; ++i) {
            float4 c = keep[i];
            float d = vlen(v3(px - c.x, py - c.y, pz - c.z)) - c.w;
            v = (i == 0) ? d : fminf(v, d);
        }
        const uint64_t row = (uint64_t)z * A.ny + y;
        if (valid) A.field[row * A.pitch + x] = v;  // near-only mode writes all values here: a superset
        uint32_t b = __ballot_sync(FULL, valid && !(v > 0.0f));
        if (lane == 0) A.bits[row * A.W + wx] = b;
    }
}

__global__ void __launch_bounds__(256) sample_sphere_set(SetArgs A) {
    extern __shared__ float4 s_keep[];
    __shared__ float s_red[8];
    __shared__ uint32_t s_cnt[8];
    __shared__ uint32_t s_nkeep;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t x0 = blockIdx.x * 32, y0 = blockIdx.y * 8, z0 = blockIdx.z * TZ;
    const uint32_t x1 = min(x0 + 31, A.nx - 1), y1 = min(y0 + 7, A.ny - 1), z1 = min(z0 + TZ - 1, A.nz - 1);
    // tile box in world coordinates (the map is affine, so the box's images are the extremes)
    float ax = world((float)x0 * A.inv, A.sx, A.ox, A.domain), bx = world((float)x1 * A.inv, A.sx, A.ox, A.domain);
    float ay = world((float)y0 * A.inv, A.sy, A.oy, A.domain), by = world((float)y1 * A.inv, A.sy, A.oy, A.domain);
    float az = world((float)(z0 + A.zoff) * A.inv, A.sz, A.oz, A.domain), bz = world((float)(z1 + A.zoff) * A.inv, A.sz, A.oz, A.domain);
    const float lox = fminf(ax, bx), hix = fmaxf(ax, bx), loy = fminf(ay, by), hiy = fmaxf(ay, by);
    const float loz = fminf(az, bz), hiz = fmaxf(az, bz);
    const float4* sp = reinterpret_cast<const float4*>(A.spheres);

    float best = 3.0e38f;
    for (uint32_t i = threadIdx.x; i < A.n; i += blockDim.x) {
        float4 c = sp[i];
        float fx = fmaxf(fabsf(c.x - lox), fabsf(c.x - hix));
        float fy = fmaxf(fabsf(c.y - loy), fabsf(c.y - hiy));
        float fz = fmaxf(fabsf(c.z - loz), fabsf(c.z - hiz));
        float far = sqrtf(fx * fx + fy * fy + fz * fz);
        float margin = 1e-4f + 1e-5f * (far + fabsf(c.w));
        best = fminf(best, far - c.w + margin);
    }
    for (int o = 16; o > 0; o >>= 1) best = fminf(best, __shfl_xor_sync(FULL, best, o));
    if (lane == 0) s_red[warp] = best;
    __syncthreads();
    float U = s_red[0];
    for (int i = 1; i < 8; ++i) U = fminf(U, s_red[i]);
    // stable compaction of the kept spheres
    uint32_t base = 0;
    float lbl = 3.0e38f;  // lower bound of the field over the tile
    for (uint32_t r0 = 0; r0 < A.n; r0 += blockDim.x) {
        uint32_t i = r0 + threadIdx.x;
        bool keep = false;
        float4 c = make_float4(0, 0, 0, 0);
        if (i < A.n) {
            c = sp[i];
            float dx = fmaxf(fmaxf(lox - c.x, c.x - hix), 0.0f);
            float dy = fmaxf(fmaxf(loy - c.y, c.y - hiy), 0.0f);
            float dz = fmaxf(fmaxf(loz - c.z, c.z - hiz), 0.0f);
            float near = sqrtf(dx * dx + dy * dy + dz * dz);
            float margin = 1e-4f + 1e-5f * (near + fabsf(c.w) + 4.0f);
            keep = near - c.w - margin <= U;
            lbl = fminf(lbl, near - c.w - margin);
        }
        uint32_t m = __ballot_sync(FULL, keep);
        if (lane == 0) s_cnt[warp] = __popc(m);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int wv = 0; wv < 8; ++wv) {
            if (wv < warp) before += s_cnt[wv];
            total += s_cnt[wv];
        }
        if (keep) {
            const uint32_t at = base + before + __popc(m & ((1u << lane) - 1u));
            s_keep[at] = c;
            if (A.near_only) s_keep[A.n + at] = sphere_thresholds(c.w, A.reach);
        }
        base += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) s_nkeep = base;
    for (int o = 16; o > 0; o >>= 1) lbl = fminf(lbl, __shfl_xor_sync(FULL, lbl, o));
    if (lane == 0) s_red[warp] = lbl;  // s_red's first use ended at the loop's barriers
    __syncthreads();
    const uint32_t nk = s_nkeep;
    if (A.near_only) {
        // every sample v of the tile satisfies LB <= v <= U: a tile wholly
        // beyond reach on one side needs sign words only
        float LB = s_red[0];
        for (int i = 1; i < 8; ++i) LB = fminf(LB, s_red[i]);
        const bool far_out = LB > A.reach, deep_in = U < -A.reach;
        if (far_out || deep_in) {
            const uint32_t y = y0 + warp;
            const uint32_t word = __ballot_sync(FULL, deep_in && x0 + lane < A.nx);
            if (y < A.ny && lane <= z1 - z0) A.bits[((size_t)(z0 + lane) * A.ny + y) * A.W + blockIdx.x] = word;
            return;
        }
    }

    const uint32_t x = x0 + lane, y = y0 + warp;
    if (y >= A.ny) return;
    const float px = world((float)x * A.inv, A.sx, A.ox, A.domain);
    const float py = world((float)y * A.inv, A.sy, A.oy, A.domain);
    const bool valid = x < A.nx;
    sample_column(A, s_keep, s_keep + A.n, nk, px, py, x, y, z0, z1, valid, lane, blockIdx.x);
}

// Sign bits of a caller-supplied field (one warp per 32-point chunk of a row).
__global__ void __launch_bounds__(256) sign_bits(const float* field, uint32_t nx, uint32_t ny, uint32_t nz,
                                                 uint64_t pitch, uint32_t* bits, uint32_t W) {
    const int lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (gw >= (uint64_t)W * ny * nz) return;
    const uint32_t w = (uint32_t)(gw % W);
    const uint64_t row = gw / W;
    const uint32_t x = 32 * w + lane;
    bool inside = false;
    if (x < nx) inside = !(__ldg(field + row * pitch + x) > 0.0f);
    uint32_t b = __ballot_sync(FULL, inside);
    if (lane == 0) bits[row * W + w] = b;
}

__global__ void sample_points(ProgView pv, const float* pts, uint64_t n, float* vals, float* normals) {
    uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    V3 p = v3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]);
    if (normals) {
        V3 nn;
        vals[i] = eval_hermite(pv, p, &nn);
        normals[3 * i] = nn.x;
        normals[3 * i + 1] = nn.y;
        normals[3 * i + 2] = nn.z;
    } else {
        vals[i] = eval_scalar(pv, p);
    }
}

// Unions of at most WARP_SET_MAX spheres take two barrier-free kernels over
// the same 32 x 8 x TZ tiles:
//   set_tiles: one warp per tile computes the culling bounds with shuffles and
//     writes a TileRec: the tile's class (mixed, or wholly beyond reach
//     outside / inside, near-only mode) and the indices of the kept spheres
//     (more than KEEP_MAX: all spheres);
//   set_rows:  one warp per tile row (8 per block) reads its record; a
//     uniform row writes its sign words, a mixed row stages its kept spheres
//     (and thresholds) in shared memory and samples its 32 x TZ points.
constexpr uint32_t WARP_SET_MAX = 256;
constexpr uint32_t KEEP_MAX = 30;
constexpr int TILE_WARPS = 4;

struct TileRec {
    uint16_t cls;  // 0 mixed, 1 far outside, 2 deep inside
    uint16_t nk;   // kept spheres; > KEEP_MAX: use all
    uint16_t idx[KEEP_MAX];
};
static_assert(sizeof(TileRec) == 64, "TileRec is one 64-byte record");

struct TileBox {
    uint32_t x0, y0, z0, x1, y1, z1;
};

__device__ __forceinline__ TileBox tile_box(const SetArgs& A, uint32_t wx, uint32_t ty, uint32_t tz) {
    TileBox b;
    b.x0 = wx * 32;
    b.y0 = ty * 8;
    b.z0 = tz * TZ;
    b.x1 = min(b.x0 + 31, A.nx - 1);
    b.y1 = min(b.y0 + 7, A.ny - 1);
    b.z1 = min(b.z0 + TZ - 1, A.nz - 1);
    return b;
}

__global__ void __launch_bounds__(32 * TILE_WARPS) set_tiles(SetArgs A, uint32_t tiles_y, uint32_t tiles_z,
                                                            TileRec* recs, uint32_t* mixed, uint32_t* nmixed,
                                                            float4* thr) {
    const int lane = threadIdx.x & 31;
    // near-only mode: the first block also writes every sphere's thresholds
    // (they depend on r and the reach only), which set_rows reads after this
    // grid in stream order
    if (thr && blockIdx.x == 0)
        for (uint32_t i = threadIdx.x; i < A.n; i += blockDim.x) thr[i] = sphere_thresholds(A.spheres[4 * i + 3], A.reach);
    const uint64_t t = (uint64_t)blockIdx.x * TILE_WARPS + (threadIdx.x >> 5);
    if (t >= (uint64_t)A.W * tiles_y * tiles_z) return;
    const uint32_t wx = (uint32_t)(t % A.W), rt = (uint32_t)(t / A.W);
    const TileBox tb = tile_box(A, wx, rt % tiles_y, rt / tiles_y);
    float ax = world((float)tb.x0 * A.inv, A.sx, A.ox, A.domain), bx = world((float)tb.x1 * A.inv, A.sx, A.ox, A.domain);
    float ay = world((float)tb.y0 * A.inv, A.sy, A.oy, A.domain), by = world((float)tb.y1 * A.inv, A.sy, A.oy, A.domain);
    float az = world((float)(tb.z0 + A.zoff) * A.inv, A.sz, A.oz, A.domain), bz = world((float)(tb.z1 + A.zoff) * A.inv, A.sz, A.oz, A.domain);
    const float lox = fminf(ax, bx), hix = fmaxf(ax, bx), loy = fminf(ay, by), hiy = fmaxf(ay, by);
    const float loz = fminf(az, bz), hiz = fmaxf(az, bz);
    const float4* sp = reinterpret_cast<const float4*>(A.spheres);
    // bounds of each sphere's value over the tile box (margins as in sample_sphere_set)
    float U = 3.0e38f, LB = 3.0e38f, low[WARP_SET_MAX / 32];
#pragma unroll
    for (int k = 0; k < (int)(WARP_SET_MAX / 32); ++k) {
        const uint32_t i = 32 * k + lane;
        low[k] = 3.0e38f;
        if (i < A.n) {
            const float4 c = __ldg(sp + i);
            const float fx = fmaxf(fabsf(c.x - lox), fabsf(c.x - hix));
            const float fy = fmaxf(fabsf(c.y - loy), fabsf(c.y - hiy));
            const float fz = fmaxf(fabsf(c.z - loz), fabsf(c.z - hiz));
            const float far = sqrtf(fx * fx + fy * fy + fz * fz);
            U = fminf(U, far - c.w + (1e-4f + 1e-5f * (far + fabsf(c.w))));
            const float dx = fmaxf(fmaxf(lox - c.x, c.x - hix), 0.0f);
            const float dy = fmaxf(fmaxf(loy - c.y, c.y - hiy), 0.0f);
            const float dz = fmaxf(fmaxf(loz - c.z, c.z - hiz), 0.0f);
            const float near = sqrtf(dx * dx + dy * dy + dz * dz);
            low[k] = near - c.w - (1e-4f + 1e-5f * (near + fabsf(c.w) + 4.0f));
            LB = fminf(LB, low[k]);
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        U = fminf(U, __shfl_xor_sync(FULL, U, o));
        LB = fminf(LB, __shfl_xor_sync(FULL, LB, o));
    }
    if (A.near_only && (LB > A.reach || U < -A.reach)) {
        // wholly beyond reach on one side: the tile's sign words, and done
        const uint32_t word = __ballot_sync(FULL, U < -A.reach && tb.x0 + lane < A.nx);
        const uint32_t ny_t = tb.y1 - tb.y0 + 1, rows = ny_t * (tb.z1 - tb.z0 + 1);
        for (uint32_t j = lane; j < rows; j += 32)
            A.bits[((size_t)(tb.z0 + j / ny_t) * A.ny + tb.y0 + j % ny_t) * A.W + wx] = word;
        return;
    }
    TileRec* rec = recs + t;
    uint32_t nk = 0;
#pragma unroll
    for (int k = 0; k < (int)(WARP_SET_MAX / 32); ++k) {
        if (32u * k >= A.n) break;
        const bool keep = low[k] <= U;
        const uint32_t m = __ballot_sync(FULL, keep);
        const uint32_t at = nk + __popc(m & ((1u << lane) - 1u));
        if (keep && at < KEEP_MAX) rec->idx[at] = (uint16_t)(32 * k + lane);
        nk += __popc(m);
    }
    if (lane == 0) {
        rec->cls = 0;
        rec->nk = (uint16_t)min(nk, 0xFFFFu);
        mixed[atomicAdd(nmixed, 1u)] = (uint32_t)t;
    }
}

// persistent: warps stride over (mixed tile, row) items.  A row is first
// bounded against the tile's kept spheres alone (they decide the minimum
// everywhere in the tile): a row wholly beyond reach writes its sign words.
constexpr int SET_ROWS_BLOCKS = 3;  // resident blocks of set_rows per SM (4 measured slower)

__global__ void __launch_bounds__(256, SET_ROWS_BLOCKS) set_rows(SetArgs A, uint32_t tiles_y, const TileRec* recs,
                                                   const uint32_t* mixed, const uint32_t* nmixed, const float4* thr_all) {
    __shared__ float4 s_keep[8][KEEP_MAX];
    __shared__ float4 s_thr[8][KEEP_MAX];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const float4* sp = reinterpret_cast<const float4*>(A.spheres);
    const uint32_t items = 8 * *nmixed;
    for (uint32_t it = blockIdx.x * 8 + warp; it < items; it += gridDim.x * 8) {
        const uint32_t t = mixed[it >> 3];
        const uint32_t wx = t % A.W, rt = t / A.W;
        const TileBox tb = tile_box(A, wx, rt % tiles_y, rt / tiles_y);
        const uint32_t y = tb.y0 + (it & 7);
        if (y > tb.y1) continue;
        const TileRec* rec = recs + t;
        const uint32_t nk = rec->nk;
        const uint32_t x = tb.x0 + lane;
        const bool valid = x < A.nx;
        const float px = world((float)x * A.inv, A.sx, A.ox, A.domain);
        const float py = world((float)y * A.inv, A.sy, A.oy, A.domain);
        if (nk > KEEP_MAX) {  // the fold over every sphere: the same minimum
            sample_column(A, sp, nullptr, A.n, px, py, x, y, tb.z0, tb.z1, valid, lane, wx);
            continue;
        }
        __syncwarp();  // the previous item's reads of the staging slots are done
        float up = 3.0e38f, lo = 3.0e38f;
        if (lane < (int)nk) {
            const uint32_t i = rec->idx[lane];
            const float4 c = __ldg(sp + i);
            s_keep[warp][lane] = c;
            if (A.near_only) {
                s_thr[warp][lane] = __ldg(thr_all + i);
                // bounds of this sphere's value over the row box
                const float ax = world((float)tb.x0 * A.inv, A.sx, A.ox, A.domain);
                const float bx = world((float)tb.x1 * A.inv, A.sx, A.ox, A.domain);
                const float az = world((float)(tb.z0 + A.zoff) * A.inv, A.sz, A.oz, A.domain);
                const float bz = world((float)(tb.z1 + A.zoff) * A.inv, A.sz, A.oz, A.domain);
                const float lox = fminf(ax, bx), hix = fmaxf(ax, bx), loz = fminf(az, bz), hiz = fmaxf(az, bz);
                const float fx = fmaxf(fabsf(c.x - lox), fabsf(c.x - hix)), fy = fabsf(c.y - py);
                const float fz = fmaxf(fabsf(c.z - loz), fabsf(c.z - hiz));
                const float far = sqrtf(fx * fx + fy * fy + fz * fz);
                up = far - c.w + (1e-4f + 1e-5f * (far + fabsf(c.w)));
                const float dx = fmaxf(fmaxf(lox - c.x, c.x - hix), 0.0f);
                const float dz = fmaxf(fmaxf(loz - c.z, c.z - hiz), 0.0f);
                const float near = sqrtf(dx * dx + fy * fy + dz * dz);
                lo = near - c.w - (1e-4f + 1e-5f * (near + fabsf(c.w) + 4.0f));
            }
        }
        if (A.near_only) {
            for (int o = 16; o > 0; o >>= 1) {
                up = fminf(up, __shfl_xor_sync(FULL, up, o));
                lo = fminf(lo, __shfl_xor_sync(FULL, lo, o));
            }
            if (lo > A.reach || up < -A.reach) {
                const uint32_t word = __ballot_sync(FULL, up < -A.reach && valid);
                if (lane <= (int)(tb.z1 - tb.z0)) A.bits[((size_t)(tb.z0 + lane) * A.ny + y) * A.W + wx] = word;
                continue;
            }
        }
        __syncwarp();
        sample_column(A, s_keep[warp], s_thr[warp], nk, px, py, x, y, tb.z0, tb.z1, valid, lane, wx);
    }
}

// IndexedInterleavedNormals / OnlyInterleavedNormals (extractor.rs:46-69,
// 97-127): each emitted vertex followed by source.sample_normal(vertex),
// unnormalised, x y z nx ny nz per vertex.
__global__ void vertex_normals(ProgView pv, const float* v, uint64_t n, float* out) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const V3 p = v3(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    V3 nn;
    eval_hermite(pv, p, &nn);
    float* o = out + 6 * i;
    o[0] = p.x;
    o[1] = p.y;
    o[2] = p.z;
    o[3] = nn.x;
    o[4] = nn.y;
    o[5] = nn.z;
}

}  // namespace

iso_status launch_vertex_normals(iso_ctx* ctx, const iso_program* prog, const float* v, uint64_t n, float* out) {
    if (n == 0) return ISO_OK;
    {
        StageTimer timer(ctx, ISO_STAGE_OTHER);
        vertex_normals<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(prog->view(), v, n, out);
    }
    ctx->launches++;
    return check_launch(ctx, "vertex normals");
}

iso_status attach_normals(iso_ctx* ctx, const iso_program* prog) {
    const uint64_t nv = ctx->last.num_vertices;
    iso_status s;
    if (nv) {
        if ((s = ensure(ctx, ctx->aux3, 24 * nv)) != ISO_OK) return s;
        if ((s = launch_vertex_normals(ctx, prog, (const float*)ctx->mesh_v.p, nv, (float*)ctx->aux3.p)) != ISO_OK)
            return s;
        std::swap(ctx->mesh_v, ctx->aux3);
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "vertex normals");
    }
    ctx->last_flags |= ISO_FLAG_NORMALS;
    ctx->last_vertex_floats = 6;
    return ISO_OK;
}

// Tiles of the culled sampler over one lattice: 4 layers x 4 * ty rows, ty
// = brick_tile_groups (at most 8 groups of 4 rows, at most BRICK_MAX
// sub-bricks).
uint32_t brick_tile_groups(uint32_t W, uint32_t ny) {
    return std::max(1u, std::min(std::min(8u, (ny + 3) / 4), BRICK_MAX / (4 * W)));
}
uint64_t brick_tiles(uint32_t W, uint32_t ny, uint32_t nz) {
    const uint32_t rows = 4 * brick_tile_groups(W, ny);
    return (uint64_t)((ny + rows - 1) / rows) * ((nz + 3) / 4);
}

iso_status launch_sample_grid(iso_ctx* ctx, const iso_program* prog, uint32_t nx, uint32_t ny, uint32_t nz, float inv,
                              float* field, uint64_t pitch, uint32_t* bits, bool near_only, uint32_t zoff,
                              float reach_steps) {
    const uint32_t W = words_per_row(nx);
    // the culled sampler (bricks.cuh) for the extractors on general
    // programs; hard sphere unions have their own culling below
    const bool bricks = near_only && prog->lip > 0.0f && 4 * W <= BRICK_MAX &&
                        brick_tiles(W, ny, nz) >= (uint64_t)ctx->sms && brick_tiles(W, ny, nz) < (1ull << 22) &&
                        !(prog->kind == PK_SPHERE_SET_HARD && prog->set_n <= 8192);
    if (bricks) {
        // values only where marching cubes can read them (bricks.cuh): tiles
        // of 4 layers x up to 32 rows, one block each, then the mixed
        // sub-bricks over a persistent grid.  A grid with fewer tiles than
        // SMs takes the plain sampler, whose one launch has less latency.
        const uint32_t ty = brick_tile_groups(W, ny);
        const uint32_t rows = 4 * ty, ytiles = (ny + rows - 1) / rows;
        const uint64_t ntiles = brick_tiles(W, ny, nz);
        const uint64_t cap = ntiles * 4 * W * ty;  // every sub-brick of every tile
        iso_status s = ensure(ctx, ctx->tiles, sizeof(BrickTask) * cap + 256);
        if (s != ISO_OK) return s;
        BrickTask* list = (BrickTask*)ctx->tiles.p;
        uint32_t* count = (uint32_t*)((char*)ctx->tiles.p + sizeof(BrickTask) * cap);
        cudaError_t e = cudaMemsetAsync(count, 0, 4, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "brick list count");
        const GridTiles gt{brick_lattice(prog, nx, ny, nz, inv, field, pitch, bits, W, zoff, reach_steps), rows, ytiles};
        StageTimer timer(ctx, ISO_STAGE_SAMPLE);
        cudaError_t je = cudaSuccess;
        if (jit_sample_bricks(ctx, prog, gt, (uint32_t)ntiles, list, count, (uint32_t)cap, &je)) {
            // the program's compiled evaluator (jit.cu)
            if (je != cudaSuccess) return cuda_fail(ctx, je, "compiled sampler launch");
        } else {
            const VmEval ev{prog->view()};
            brick_classify<GridTiles><<<(unsigned)ntiles, 256, 0, ctx->stream>>>(ev, gt, list, count,
                                                                                  (uint32_t)cap, ctx->d_err);
            brick_rows<GridTiles><<<brick_rows_blocks<GridTiles>(ctx->sms), 256, 0, ctx->stream>>>(
                ev, gt, list, count, (uint32_t)cap);
        }
        ctx->launches++;
    } else if (prog->kind == PK_SPHERE_SET_HARD && prog->set_n <= 8192) {
        near_only = near_only && prog->set_n <= 4096 && nx > 1;
        SetArgs a;
        a.spheres = prog->d_set;
        a.n = prog->set_n;
        a.domain = prog->has_domain;
        a.sx = prog->domain[0]; a.sy = prog->domain[1]; a.sz = prog->domain[2];
        a.ox = prog->domain[3]; a.oy = prog->domain[4]; a.oz = prog->domain[5];
        a.nx = nx; a.ny = ny; a.nz = nz; a.inv = inv;
        a.field = field; a.pitch = pitch; a.bits = bits; a.W = W;
        a.near_only = near_only;
        a.zoff = zoff;
        // a crossing edge joins samples one lattice step apart, and the field
        // is 1-Lipschitz in world units: both ends lie within one step (the
        // largest axis step after the domain map) of zero, plus rounding slack
        const float step = inv * (prog->has_domain ? fmaxf(fabsf(a.sx), fmaxf(fabsf(a.sy), fabsf(a.sz))) : 1.0f);
        a.reach = step * reach_steps * 1.001f + 1e-4f;
        size_t smem = (near_only ? 32 : 16) * (size_t)prog->set_n;
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(sample_sphere_set, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "sphere-set smem attribute");
        }
        const uint32_t ty = (ny + 7) / 8, tz = (nz + TZ - 1) / TZ;
        const uint64_t tiles = (uint64_t)W * ty * tz;
        if (prog->set_n <= WARP_SET_MAX && tiles < (1ull << 31)) {
            // records | mixed-tile list | its length | sphere thresholds
            const size_t rec_bytes = sizeof(TileRec) * tiles, list_bytes = (4 * tiles + 255) & ~(size_t)255;
            iso_status s = ensure(ctx, ctx->tiles, rec_bytes + list_bytes + 256 + 16 * (size_t)prog->set_n);
            if (s != ISO_OK) return s;
            TileRec* recs = (TileRec*)ctx->tiles.p;
            uint32_t* mixed = (uint32_t*)((char*)ctx->tiles.p + rec_bytes);
            uint32_t* nmixed = (uint32_t*)((char*)mixed + list_bytes);
            float4* thr = (float4*)((char*)nmixed + 256);
            cudaError_t e = cudaMemsetAsync(nmixed, 0, 4, ctx->stream);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "mixed-tile count");
            StageTimer timer(ctx, ISO_STAGE_SAMPLE);
            set_tiles<<<(unsigned)((tiles + TILE_WARPS - 1) / TILE_WARPS), 32 * TILE_WARPS, 0, ctx->stream>>>(
                a, ty, tz, recs, mixed, nmixed, near_only ? thr : nullptr);
            set_rows<<<(unsigned)ctx->sms * SET_ROWS_BLOCKS, 256, 0, ctx->stream>>>(a, ty, recs, mixed, nmixed, thr);
            ctx->launches++;
        } else {
            dim3 grid(W, (ny + 7) / 8, (nz + TZ - 1) / TZ);
            StageTimer timer(ctx, ISO_STAGE_SAMPLE);
            sample_sphere_set<<<grid, 256, smem, ctx->stream>>>(a);
        }
    } else {
        const uint64_t warps = (uint64_t)W * ny * nz;
        const BrickLattice g = brick_lattice(prog, nx, ny, nz, inv, field, pitch, bits, W, zoff, reach_steps);
        StageTimer timer(ctx, ISO_STAGE_SAMPLE);
        cudaError_t je = cudaSuccess;
        // a full field: the program's compiled evaluator when it has one
        // (jit.cu; the extractors' small lattices stay interpreted, as a
        // compilation would cost more than it saves there)
        if (!near_only && jit_sample_field(ctx, prog, g, (warps + 7) / 8, &je)) {
            if (je != cudaSuccess) return cuda_fail(ctx, je, "compiled field sampler launch");
        } else {
            sample_generic<<<(unsigned)((warps + 7) / 8), 256, 0, ctx->stream>>>(VmEval{prog->view()}, g);
        }
    }
    ctx->launches++;
    return check_launch(ctx, "sample_grid");
}

iso_status launch_sign_bits(iso_ctx* ctx, const float* field, uint32_t nx, uint32_t ny, uint32_t nz, uint64_t pitch,
                            uint32_t* bits) {
    const uint32_t W = words_per_row(nx);
    uint64_t warps = (uint64_t)W * ny * nz;
    StageTimer timer(ctx, ISO_STAGE_SIGNS);
    sign_bits<<<(unsigned)((warps + 7) / 8), 256, 0, ctx->stream>>>(field, nx, ny, nz, pitch, bits, W);
    ctx->launches++;
    return check_launch(ctx, "sign_bits");
}

cudaError_t launch_sign_bits_on(cudaStream_t stream, const float* field, uint32_t nx, uint32_t ny, uint32_t nz,
                                uint64_t pitch, uint32_t* bits) {
    const uint32_t W = words_per_row(nx);
    uint64_t warps = (uint64_t)W * ny * nz;
    sign_bits<<<(unsigned)((warps + 7) / 8), 256, 0, stream>>>(field, nx, ny, nz, pitch, bits, W);
    return cudaGetLastError();
}

iso_status launch_sample_points(iso_ctx* ctx, const iso_program* prog, const float* d_pts, uint64_t n, float* d_vals,
                                float* d_normals) {
    if (n == 0) return ISO_OK;
    StageTimer timer(ctx, ISO_STAGE_OTHER);
    sample_points<<<(unsigned)((n + 127) / 128), 128, 0, ctx->stream>>>(prog->view(), d_pts, n, d_vals, d_normals);
    ctx->launches++;
    return check_launch(ctx, "sample_points");
}

}  // namespace iso
