// Learned-surrogate marching cubes, and the distances that score it.
//
// iso_surrogate_field builds the field of MarchingCubes::new(size) for an
// expensive exact program from a trained network (mlp.cu / mlp_infer.cu):
//   1. the network (bf16 tensor cores) on every step-th lattice point;
//   2. every fine point takes the trilinear interpolation of that coarse grid;
//      points whose interpolated value lies within band_cells fine cells of
//      zero are listed (warp-aggregated append);
//   3. the listed points are re-sampled with the exact program, at the same
//      f32 lattice coordinates as the grid sampler, so inside the band the
//      field is bit-identical to the exact field.
// Marching cubes then runs on the field as on any caller field.  Cells whose
// corners all lie in the band produce exactly the exact mesh's triangles;
// elsewhere the surface is the network's.
//
// iso_mesh_distance scores two vertex sets by nearest-neighbour distances
// (Chamfer = mean of the two directed means, Hausdorff = the larger max) with
// a bucket grid built by counting sort and a ring search; iso_field_case_
// disagreement counts cells whose corner signs differ between two fields.
//
// Built with -fmad=false (the exact re-sampling must round as the sampler).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "internal.h"
#include "mlp.h"
#include "vm.cuh"

namespace iso {
namespace {

constexpr uint32_t FULL = 0xFFFFFFFFu;

struct BandArgs {
    const float* coarse;  // cx x cy x cz network values, x fastest
    uint32_t cx, cy, cz, step;
    uint32_t nx, ny, nz;
    float inv_step;
    float tau;            // band half-width in field units
    float* field;
    uint64_t pitch;
    uint32_t* list;       // fine point ids (z*ny + y)*nx + x of band points
    uint32_t* count;
    const uint32_t* forced;  // null, or one bit per fine point id: re-sample it exactly
};

__device__ __forceinline__ float lerp1(float a, float b, float t) { return a + (b - a) * t; }

// grid (ceil(nx / 128), ny, nz) x 128 threads
__global__ void __launch_bounds__(128) band_mark(BandArgs A) {
    const uint32_t x = blockIdx.x * 128 + threadIdx.x, y = blockIdx.y, z = blockIdx.z;
    bool band = false;
    if (x < A.nx) {
        const uint32_t ix = x / A.step, iy = y / A.step, iz = z / A.step;
        const float tx = (float)(x - ix * A.step) * A.inv_step, ty = (float)(y - iy * A.step) * A.inv_step,
                    tz = (float)(z - iz * A.step) * A.inv_step;
        const uint32_t jx = min(ix + 1, A.cx - 1), jy = min(iy + 1, A.cy - 1), jz = min(iz + 1, A.cz - 1);
        const float* c = A.coarse;
        auto at = [&](uint32_t i, uint32_t j, uint32_t k) { return __ldg(c + ((size_t)k * A.cy + j) * A.cx + i); };
        const float v00 = lerp1(at(ix, iy, iz), at(jx, iy, iz), tx), v10 = lerp1(at(ix, jy, iz), at(jx, jy, iz), tx);
        const float v01 = lerp1(at(ix, iy, jz), at(jx, iy, jz), tx), v11 = lerp1(at(ix, jy, jz), at(jx, jy, jz), tx);
        const float v = lerp1(lerp1(v00, v10, ty), lerp1(v01, v11, ty), tz);
        band = fabsf(v) <= A.tau;
        if (!band && A.forced) {
            const uint32_t id = ((uint32_t)z * A.ny + y) * A.nx + x;
            band = (__ldg(A.forced + (id >> 5)) >> (id & 31)) & 1u;
        }
        if (!band) A.field[((size_t)z * A.ny + y) * A.pitch + x] = v;
    }
    const uint32_t m = __ballot_sync(FULL, band);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(A.count, (uint32_t)__popc(m));
    base = __shfl_sync(FULL, base, 0);
    if (band) A.list[base + __popc(m & ((1u << lane) - 1u))] = ((uint32_t)z * A.ny + y) * A.nx + x;
}

struct ExactArgs {
    ProgView pv;
    const uint32_t* list;
    const uint32_t* count;
    uint32_t nx, ny;
    float inv;
    float* field;
    uint64_t pitch;
};

// grid-stride over the band list: the grid sampler's evaluation of the same points
__global__ void __launch_bounds__(256) band_exact(ExactArgs A) {
    const uint32_t n = *A.count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t id = A.list[i];
        const uint32_t x = id % A.nx, r = id / A.nx;
        const uint32_t y = r % A.ny, z = r / A.ny;
        const float v = eval_scalar(A.pv, v3((float)x * A.inv, (float)y * A.inv, (float)z * A.inv));
        A.field[((size_t)z * A.ny + y) * A.pitch + x] = v;
    }
}

// The coarse grid from the exact program instead of the network (the same
// pipeline without the network, for comparison): coarse point (i, j, k) is
// fine lattice point (i, j, k) * step, as the network sees it.
__global__ void __launch_bounds__(256) coarse_exact(ProgView pv, uint32_t cx, uint32_t cy, uint32_t cz,
                                                     uint32_t step, float inv, float* coarse) {
    const uint64_t n = (uint64_t)cx * cy * cz;
    for (uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(t % cx), r = (uint32_t)(t / cx);
        const uint32_t j = r % cy, k = r / cy;
        coarse[t] = eval_scalar(pv, v3((float)(i * step) * inv, (float)(j * step) * inv, (float)(k * step) * inv));
    }
}

// Spot checks of the surrogate against the exact source at witness points of
// each sphere of a sphere-set source: its centre (inside the exact surface)
// and the six points of its own surface on the axes.  A sphere is flagged
// when the interpolated network value says "outside" at its centre, or when
// at a surface witness that lies near the exact surface (|exact| within two
// cells) the two differ by more than `tol`: there the band around the
// network's surface may miss the exact one.
struct WitnessArgs {
    ProgView pv;
    const float* spheres;   // n x (cx, cy, cz, r) in the source's frame
    uint32_t n;
    float scale[3], offset[3];  // sample frame -> source frame
    float inv;              // 1 / (size - 1)
    const float* coarse;
    uint32_t cx, cy, cz, step;
    float near, tol;        // field units
    uint32_t* flags;        // per sphere: 1 shell, 2 ball (or both); flags[n] counts the flagged
};

__device__ __forceinline__ float coarse_at(const WitnessArgs& A, float u, float v, float w) {
    // trilinear interpolation of the coarse grid at fine lattice coordinates
    const float fu = fminf(fmaxf(u / (float)A.step, 0.0f), (float)(A.cx - 1));
    const float fv = fminf(fmaxf(v / (float)A.step, 0.0f), (float)(A.cy - 1));
    const float fw = fminf(fmaxf(w / (float)A.step, 0.0f), (float)(A.cz - 1));
    const uint32_t i = min((uint32_t)fu, A.cx - 1), j = min((uint32_t)fv, A.cy - 1), k = min((uint32_t)fw, A.cz - 1);
    const uint32_t i1 = min(i + 1, A.cx - 1), j1 = min(j + 1, A.cy - 1), k1 = min(k + 1, A.cz - 1);
    const float tx = fu - (float)i, ty = fv - (float)j, tz = fw - (float)k;
    auto at = [&](uint32_t a, uint32_t b, uint32_t c) { return __ldg(A.coarse + ((size_t)c * A.cy + b) * A.cx + a); };
    const float v00 = lerp1(at(i, j, k), at(i1, j, k), tx), v10 = lerp1(at(i, j1, k), at(i1, j1, k), tx);
    const float v01 = lerp1(at(i, j, k1), at(i1, j, k1), tx), v11 = lerp1(at(i, j1, k1), at(i1, j1, k1), tx);
    return lerp1(lerp1(v00, v10, ty), lerp1(v01, v11, ty), tz);
}

__global__ void __launch_bounds__(256) witness_check(WitnessArgs A) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 7 * A.n) return;
    const uint32_t s = t / 7, k = t % 7;
    const float* q = A.spheres + 4 * (size_t)s;
    const float4 sp = make_float4(q[0], q[1], q[2], q[3]);
    float w[3] = {sp.x, sp.y, sp.z};
    if (k > 0) w[(k - 1) >> 1] += (k & 1) ? sp.w : -sp.w;
    float p[3], u[3];
    for (int a = 0; a < 3; ++a) {
        p[a] = (w[a] - A.offset[a]) / A.scale[a];  // sample frame
        u[a] = p[a] / A.inv;                        // fine lattice coordinates
    }
    const float sv = coarse_at(A, u[0], u[1], u[2]);
    uint32_t flag = 0;
    if (k == 0) {
        flag = sv > 0.0f ? 2u : 0u;  // missed at its centre: the whole ball
    } else {
        const float ev = eval_scalar(A.pv, v3(p[0], p[1], p[2]));
        flag = fabsf(ev) <= A.near && fabsf(sv - ev) > A.tol ? 1u : 0u;  // off near its surface: the shell
    }
    if (flag && atomicOr(A.flags + s, flag) == 0u) atomicAdd(A.flags + A.n, 1u);  // count each sphere once
}

// Fine points within `shell` (field units) of a flagged sphere's surface are
// forced into the band, and for a sphere missed at its centre every point
// inside it as well (the network's signs there are wrong): one block per
// sphere (unflagged ones return at once).
struct ShellArgs {
    const float* spheres;
    const uint32_t* flags;
    float scale[3], offset[3];
    float inv, shell;
    uint32_t nx, ny, nz;
    uint32_t* forced;
};

__global__ void __launch_bounds__(256) witness_shells(ShellArgs A) {
    const uint32_t flag = A.flags[blockIdx.x];
    if (!flag) return;
    const bool ball = flag & 2u;
    const float* q4 = A.spheres + 4 * (size_t)blockIdx.x;
    const float4 sp = make_float4(q4[0], q4[1], q4[2], q4[3]);
    const float c[3] = {sp.x, sp.y, sp.z};
    const float reach = sp.w + A.shell;
    int32_t lo[3], hi[3];
    const uint32_t dims[3] = {A.nx, A.ny, A.nz};
    for (int a = 0; a < 3; ++a) {
        // lattice coordinates of c -/+ reach (the scale may be negative)
        const float e0 = (c[a] - reach - A.offset[a]) / A.scale[a] / A.inv;
        const float e1 = (c[a] + reach - A.offset[a]) / A.scale[a] / A.inv;
        lo[a] = max((int32_t)floorf(fminf(e0, e1)) - 1, 0);
        hi[a] = min((int32_t)ceilf(fmaxf(e0, e1)) + 1, (int32_t)dims[a] - 1);
        if (lo[a] > hi[a]) return;
    }
    const uint32_t ex = hi[0] - lo[0] + 1, ey = hi[1] - lo[1] + 1, ez = hi[2] - lo[2] + 1;
    const uint64_t total = (uint64_t)ex * ey * ez;
    for (uint64_t t = threadIdx.x; t < total; t += blockDim.x) {
        const uint32_t x = lo[0] + (uint32_t)(t % ex), r = (uint32_t)(t / ex);
        const uint32_t y = lo[1] + r % ey, z = lo[2] + r / ey;
        const float qx = (float)x * A.inv * A.scale[0] + A.offset[0] - c[0];
        const float qy = (float)y * A.inv * A.scale[1] + A.offset[1] - c[1];
        const float qz = (float)z * A.inv * A.scale[2] + A.offset[2] - c[2];
        const float d = sqrtf(qx * qx + qy * qy + qz * qz) - sp.w;
        if (ball ? d <= A.shell : fabsf(d) <= A.shell) {
            const uint32_t id = (z * A.ny + y) * A.nx + x;
            atomicOr(A.forced + (id >> 5), 1u << (id & 31));
        }
    }
}

// ------------------------------------------------------------ distances ---
struct Buckets {
    float lo[3];
    float inv_b;          // 1 / bucket edge
    uint32_t g[3];        // buckets per axis
};

__device__ __forceinline__ uint32_t bucket_axis(float v, float lo, float inv_b, uint32_t g) {
    const float f = (v - lo) * inv_b;
    const int i = (int)floorf(f);
    return (uint32_t)min(max(i, 0), (int)g - 1);
}

__global__ void bucket_count(const float* p, uint32_t n, Buckets B, uint32_t* counts, uint32_t* bucket_of) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t bx = bucket_axis(p[3 * i], B.lo[0], B.inv_b, B.g[0]);
    const uint32_t by = bucket_axis(p[3 * i + 1], B.lo[1], B.inv_b, B.g[1]);
    const uint32_t bz = bucket_axis(p[3 * i + 2], B.lo[2], B.inv_b, B.g[2]);
    const uint32_t b = (bz * B.g[1] + by) * B.g[0] + bx;
    bucket_of[i] = b;
    atomicAdd(counts + b, 1u);
}

__global__ void bucket_fill(const float* p, uint32_t n, const uint32_t* bucket_of, uint32_t* cursor, float4* sorted) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t at = atomicAdd(cursor + bucket_of[i], 1u);
    sorted[at] = make_float4(p[3 * i], p[3 * i + 1], p[3 * i + 2], 0.0f);
}

struct QueryArgs {
    const float* q;
    uint32_t nq;
    Buckets B;
    const uint32_t* start;  // exclusive scan of counts (nb + 1 entries: total at the end)
    const float4* pts;
    uint32_t max_rings;
    double* sum;            // sum of distances
    unsigned int* max_bits; // max distance as f32 bits (non-negative)
    unsigned long long* capped;
};

// Nearest point of the bucketed set for each query: rings of buckets at
// Chebyshev distance r = 0, 1, ... around the query's bucket; every point in
// ring r + 1 or beyond is at least r bucket edges away, so the search stops
// once the best distance is within that.  Past max_rings the distance is
// reported as max_rings bucket edges (counted in `capped`).
__global__ void __launch_bounds__(256) nearest(QueryArgs A) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float d = 0.0f;
    if (i < A.nq) {
        const float qx = A.q[3 * i], qy = A.q[3 * i + 1], qz = A.q[3 * i + 2];
        const int bx = (int)bucket_axis(qx, A.B.lo[0], A.B.inv_b, A.B.g[0]);
        const int by = (int)bucket_axis(qy, A.B.lo[1], A.B.inv_b, A.B.g[1]);
        const int bz = (int)bucket_axis(qz, A.B.lo[2], A.B.inv_b, A.B.g[2]);
        const float edge = 1.0f / A.B.inv_b;
        float best = INFINITY;
        bool done = false;
        for (int r = 0; r <= (int)A.max_rings && !done; ++r) {
            for (int dz = -r; dz <= r; ++dz) {
                const int z = bz + dz;
                if (z < 0 || z >= (int)A.B.g[2]) continue;
                for (int dy = -r; dy <= r; ++dy) {
                    const int y = by + dy;
                    if (y < 0 || y >= (int)A.B.g[1]) continue;
                    const bool face = (dz == -r || dz == r || dy == -r || dy == r);
                    for (int dx = -r; dx <= r; dx += (face || r == 0) ? 1 : 2 * r) {
                        const int x = bx + dx;
                        if (x < 0 || x >= (int)A.B.g[0]) continue;
                        const uint32_t b = ((uint32_t)z * A.B.g[1] + (uint32_t)y) * A.B.g[0] + (uint32_t)x;
                        for (uint32_t k = A.start[b]; k < A.start[b + 1]; ++k) {
                            const float4 p = A.pts[k];
                            const float ex = p.x - qx, ey = p.y - qy, ez = p.z - qz;
                            best = fminf(best, ex * ex + ey * ey + ez * ez);
                        }
                    }
                }
            }
            const float reach = (float)r * edge;
            if (best <= reach * reach) done = true;
        }
        if (done) {
            d = sqrtf(best);
        } else {  // an upper bound when something was seen, else the searched radius
            d = best < INFINITY ? sqrtf(best) : (float)A.max_rings * edge;
            atomicAdd(A.capped, 1ull);
        }
    }
    // block reduction of sum and max
    __shared__ double s_sum[8];
    __shared__ float s_max[8];
    double s = d;
    float m = d;
    for (int o = 16; o; o >>= 1) {
        s += __shfl_down_sync(FULL, s, o);
        m = fmaxf(m, __shfl_down_sync(FULL, m, o));
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_sum[warp] = s;
        s_max[warp] = m;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        float mm = 0.0f;
        for (int w = 0; w < 8; ++w) {
            t += s_sum[w];
            mm = fmaxf(mm, s_max[w]);
        }
        atomicAdd(A.sum, t);
        atomicMax(A.max_bits, __float_as_uint(mm));
    }
}

// cells (x < nx-1, y < ny-1, z < nz-1) whose eight corner signs differ
// between two fields, from the XOR of their sign-bit rows
__global__ void case_diff(const uint32_t* ba, const uint32_t* bb, uint32_t nx, uint32_t ny, uint32_t nz, uint32_t W,
                          unsigned long long* cells) {
    const uint64_t t = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const uint64_t rows = (uint64_t)(ny - 1) * (nz - 1);
    uint32_t c = 0;
    if (t < rows * W) {
        const uint32_t w = (uint32_t)(t % W);
        const uint64_t r = t / W;
        const uint32_t y = (uint32_t)(r % (ny - 1)), z = (uint32_t)(r / (ny - 1));
        auto dx = [&](uint32_t yy, uint32_t zz, uint32_t ww) {
            const size_t at = ((size_t)zz * ny + yy) * W + ww;
            return ww < W ? (ba[at] ^ bb[at]) : 0u;
        };
        const uint32_t d = dx(y, z, w) | dx(y + 1, z, w) | dx(y, z + 1, w) | dx(y + 1, z + 1, w);
        const uint32_t dn = dx(y, z, w + 1) | dx(y + 1, z, w + 1) | dx(y, z + 1, w + 1) | dx(y + 1, z + 1, w + 1);
        uint32_t cellmask = d | (d >> 1) | (dn << 31);  // cell x: corner x or x + 1 differs
        const uint32_t first = 32 * w;
        const uint32_t ncell = nx - 1;  // cells along x
        if (first + 32 > ncell) cellmask &= first >= ncell ? 0u : ((1u << (ncell - first)) - 1u);
        c = __popc(cellmask);
    }
    for (int o = 16; o; o >>= 1) c += __shfl_down_sync(FULL, c, o);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(cells, (unsigned long long)c);
}

inline unsigned blocks_for(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

iso_status check_args(iso_ctx* ctx, iso_mlp* net, const iso_program* exact, uint32_t size, uint32_t step,
                      float band, bool need_net = true) {
    if (!ctx || !exact || (need_net && !net)) return ISO_ERR_INVALID_ARG;
    if (net && net->ctx != ctx) return fail(ctx, ISO_ERR_INVALID_ARG, "network belongs to another context");
    if (exact->ctx != ctx) return fail(ctx, ISO_ERR_INVALID_ARG, "program belongs to another context");
    if (size < 2 || size > 2048) return fail(ctx, ISO_ERR_INVALID_ARG, "size must be in [2, 2048]");
    if (step < 1 || step > 64) return fail(ctx, ISO_ERR_INVALID_ARG, "coarse step must be in [1, 64]");
    if (!(band >= 0.0f) || band > 1.0e6f) return fail(ctx, ISO_ERR_INVALID_ARG, "band must be >= 0");
    return set_device(ctx);
}

// The sphere list of a sphere-set program ([domain map] SPHERE_SET, hard or
// smooth) on the device, its size, smooth k (0 for a hard union) and frame.
bool sphere_list(const iso_program* p, const float** d_spheres, uint32_t* n, float* k) {
    const auto& o = p->ops;
    size_t at = SIZE_MAX;
    if (o.size() == 1 && (o[0] & 0xFF) == OP_SPHERE_SET) at = o[0] >> 8;
    if (o.size() == 3 && (o[0] & 0xFF) == OP_PT_DOMAIN && (o[1] & 0xFF) == OP_SPHERE_SET &&
        (o[2] & 0xFF) == OP_PT_POP)
        at = o[1] >> 8;
    if (at == SIZE_MAX) return false;
    *n = (uint32_t)p->consts[at];
    *k = p->consts[at + 1] != 0.0f ? p->consts[at + 2] : 0.0f;
    *d_spheres = p->d_consts + at + 3;
    return true;
}

// field into `field`; uses ctx->aux (band list), ctx->aux2 (coarse grid) and,
// for the witness checks, ctx->aux3 (forced-point mask and sphere flags)
iso_status surrogate_field(iso_ctx* ctx, iso_mlp* net, const iso_program* exact, uint32_t size, uint32_t step,
                           float band, uint32_t flags, float* field, uint64_t pitch, iso_surrogate_stats* stats,
                           uint64_t* flagged) {
    const uint32_t nx = size, ny = size, nz = size + 1;
    const uint64_t npts = (uint64_t)nx * ny * nz;
    if (npts >= (1ull << 32)) return fail(ctx, ISO_ERR_TOO_LARGE, "more than 2^32 lattice points");
    const float inv = 1.0f / (float)(size - 1);
    MlpGrid g;
    g.nx = (nx - 1 + step - 1) / step + 1;
    g.ny = (ny - 1 + step - 1) / step + 1;
    g.nz = (nz - 1 + step - 1) / step + 1;
    g.step = step;
    g.inv = inv;
    float cell = inv;
    for (int i = 0; i < 3; ++i) {
        g.scale[i] = exact->has_domain ? exact->domain[i] : 1.0f;
        g.offset[i] = exact->has_domain ? exact->domain[3 + i] : 0.0f;
    }
    if (exact->has_domain)
        cell = inv * std::min(std::fabs(g.scale[0]), std::min(std::fabs(g.scale[1]), std::fabs(g.scale[2])));
    const uint64_t ncoarse = (uint64_t)g.nx * g.ny * g.nz;
    iso_status s;
    if ((s = ensure(ctx, ctx->aux2, 4 * ncoarse + 256)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->aux, 4 * npts + 256)) != ISO_OK) return s;
    float* coarse = (float*)ctx->aux2.p;
    uint32_t* count = (uint32_t*)((char*)ctx->aux2.p + ((4 * ncoarse + 255) & ~255ull));
    uint32_t* list = (uint32_t*)ctx->aux.p;
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (flags & ISO_SURROGATE_EXACT_COARSE) {
        StageTimer timer(ctx, ISO_STAGE_SAMPLE);
        coarse_exact<<<(unsigned)sms * 8, 256, 0, ctx->stream>>>(exact->view(), g.nx, g.ny, g.nz, step, inv, coarse);
        ctx->launches++;
        if ((s = check_launch(ctx, "coarse exact")) != ISO_OK) return s;
    } else if ((s = mlp_infer_launch(net, nullptr, 0, &g, coarse)) != ISO_OK) {
        return s;
    }
    cudaError_t e = cudaMemsetAsync(count, 0, 4, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "band count");
    uint32_t* forced = nullptr;
    uint32_t* sphere_flags = nullptr;
    uint32_t nsph = 0;
    if (flags & ISO_SURROGATE_WITNESS) {
        const float* d_sph = nullptr;
        float sk = 0.0f;
        if (!sphere_list(exact, &d_sph, &nsph, &sk))
            return fail(ctx, ISO_ERR_UNSUPPORTED, "witness checks need a sphere-set source");
        const size_t mask_words = (npts + 31) / 32;
        const size_t bytes = 4 * mask_words + 4 * ((size_t)nsph + 1) + 256;
        if ((s = ensure(ctx, ctx->aux3, bytes)) != ISO_OK) return s;
        forced = (uint32_t*)ctx->aux3.p;
        sphere_flags = forced + ((mask_words + 63) & ~(size_t)63);
        e = cudaMemsetAsync(ctx->aux3.p, 0, bytes, ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "witness scratch");
        WitnessArgs w{exact->view(), d_sph, nsph, {g.scale[0], g.scale[1], g.scale[2]},
                      {g.offset[0], g.offset[1], g.offset[2]}, inv, coarse, g.nx, g.ny, g.nz, step,
                      2.0f * cell, std::max(band - 1.0f, 0.25f) * cell, sphere_flags};
        ShellArgs sh{d_sph, sphere_flags, {g.scale[0], g.scale[1], g.scale[2]}, {g.offset[0], g.offset[1], g.offset[2]},
                     inv, (band + 1.0f) * cell + 0.5f * sk, nx, ny, nz, forced};
        StageTimer timer(ctx, ISO_STAGE_OTHER);
        witness_check<<<blocks_for(7ull * nsph, 256), 256, 0, ctx->stream>>>(w);
        witness_shells<<<nsph, 256, 0, ctx->stream>>>(sh);
        ctx->launches += 2;
        if ((s = check_launch(ctx, "witness checks")) != ISO_OK) return s;
    }
    BandArgs b{coarse, g.nx, g.ny, g.nz, step, nx, ny, nz, 1.0f / (float)step, band * cell, field, pitch, list, count,
               forced};
    {
        StageTimer timer(ctx, ISO_STAGE_OTHER);
        band_mark<<<dim3(blocks_for(nx, 128), ny, nz), 128, 0, ctx->stream>>>(b);
    }
    ctx->launches++;
    if ((s = check_launch(ctx, "band mark")) != ISO_OK) return s;
    ExactArgs x{exact->view(), list, count, nx, ny, inv, field, pitch};
    {
        StageTimer timer(ctx, ISO_STAGE_SAMPLE);
        band_exact<<<(unsigned)sms * 8, 256, 0, ctx->stream>>>(x);
    }
    ctx->launches++;
    if ((s = check_launch(ctx, "band exact")) != ISO_OK) return s;
    if (stats || flagged) {
        e = cudaMemcpyAsync(ctx->h_pinned, count, 4, cudaMemcpyDeviceToHost, ctx->stream);
        if (e == cudaSuccess && sphere_flags)
            e = cudaMemcpyAsync((uint32_t*)ctx->h_pinned + 1, sphere_flags + nsph, 4, cudaMemcpyDeviceToHost,
                                ctx->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "band stats");
        if (stats) {
            stats->coarse_points = ncoarse;
            stats->band_points = *(uint32_t*)ctx->h_pinned;
            stats->total_points = npts;
        }
        if (flagged) *flagged = sphere_flags ? ((uint32_t*)ctx->h_pinned)[1] : 0;
    }
    return ISO_OK;
}

}  // namespace
}  // namespace iso

using namespace iso;

extern "C" {

iso_status iso_surrogate_field(iso_ctx* ctx, iso_mlp* net, const iso_program* exact, uint32_t size,
                               uint32_t coarse_step, float band_cells, float* field, uint64_t pitch,
                               iso_surrogate_stats* stats) {
    iso::NvtxRange nvtx_range("iso_surrogate_field");
    iso_status s = check_args(ctx, net, exact, size, coarse_step, band_cells);
    if (s != ISO_OK) return s;
    if (!field || pitch < size) return fail(ctx, ISO_ERR_INVALID_ARG, "need a field with pitch >= size");
    if ((s = surrogate_field(ctx, net, exact, size, coarse_step, band_cells, 0, field, pitch, stats, nullptr)) !=
        ISO_OK)
        return s;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "surrogate field");
    return read_device_errors(ctx);
}

iso_status iso_surrogate_field_ex(iso_ctx* ctx, iso_mlp* net, const iso_program* exact, uint32_t size,
                                  uint32_t coarse_step, float band_cells, uint32_t flags, float* field, uint64_t pitch,
                                  iso_surrogate_stats* stats, uint64_t* flagged_primitives) {
    iso::NvtxRange nvtx_range("iso_surrogate_field_ex");
    if (flags & ~(uint32_t)(ISO_SURROGATE_EXACT_COARSE | ISO_SURROGATE_WITNESS)) {
        if (ctx) fail(ctx, ISO_ERR_INVALID_ARG, "unknown flags");
        return ISO_ERR_INVALID_ARG;
    }
    iso_status s = check_args(ctx, net, exact, size, coarse_step, band_cells,
                              !(flags & ISO_SURROGATE_EXACT_COARSE));
    if (s != ISO_OK) return s;
    if (!field || pitch < size) return fail(ctx, ISO_ERR_INVALID_ARG, "need a field with pitch >= size");
    if ((s = surrogate_field(ctx, net, exact, size, coarse_step, band_cells, flags, field, pitch, stats,
                             flagged_primitives)) != ISO_OK)
        return s;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "surrogate field");
    return read_device_errors(ctx);
}

iso_status iso_surrogate_extract(iso_ctx* ctx, iso_mlp* net, const iso_program* exact, uint32_t size,
                                 uint32_t coarse_step, float band_cells, uint32_t flags, iso_surrogate_stats* stats,
                                 iso_mesh_info* info) {
    iso::NvtxRange nvtx_range("iso_surrogate_extract");
    iso_status s = check_args(ctx, net, exact, size, coarse_step, band_cells);
    if (s != ISO_OK) return s;
    if (flags & ~(uint32_t)ISO_FLAG_KEYS) return fail(ctx, ISO_ERR_INVALID_ARG, "unknown flags");
    const uint32_t nx = size, ny = size, nz = size + 1;
    const uint64_t pitch = default_pitch(nx);
    const uint32_t W = words_per_row(nx);
    if ((s = ensure(ctx, ctx->field, 4 * pitch * ny * nz)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->bits, 4ull * W * ny * nz)) != ISO_OK) return s;
    float* field = (float*)ctx->field.p;
    if ((s = surrogate_field(ctx, net, exact, size, coarse_step, band_cells, 0, field, pitch, stats, nullptr)) !=
        ISO_OK)
        return s;
    if ((s = launch_sign_bits(ctx, field, nx, ny, nz, pitch, (uint32_t*)ctx->bits.p)) != ISO_OK) return s;
    Lattice L{nx, ny, nz, pitch, field, (const uint32_t*)ctx->bits.p, W, 1.0f / (float)(nx - 1), nullptr};
    return mc_extract_lattice(ctx, L, flags, info);
}

iso_status iso_mesh_distance(iso_ctx* ctx, const float* a, uint64_t na, const float* b, uint64_t nb, float bucket,
                             uint32_t max_rings, iso_mesh_distance_result* out) {
    iso::NvtxRange nvtx_range("iso_mesh_distance");
    if (!ctx || !out || (!a && na) || (!b && nb) || !(bucket > 0.0f) || max_rings == 0 || max_rings > 1024)
        return ISO_ERR_INVALID_ARG;
    if (na == 0 || nb == 0) return fail(ctx, ISO_ERR_INVALID_ARG, "both vertex sets must be non-empty");
    if (na >= (1ull << 31) || nb >= (1ull << 31)) return fail(ctx, ISO_ERR_TOO_LARGE, "too many vertices");
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    // common bucket grid over the bounding box of both sets
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (const float* p : {a, b}) {
        const uint64_t n = p == a ? na : nb;
        for (uint64_t i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                const float v = p[3 * i + k];
                if (!std::isfinite(v)) return fail(ctx, ISO_ERR_INVALID_ARG, "non-finite vertex");
                lo[k] = std::min(lo[k], v);
                hi[k] = std::max(hi[k], v);
            }
    }
    Buckets B;
    uint64_t nbk = 1;
    for (int k = 0; k < 3; ++k) {
        const double g = std::floor((double)(hi[k] - lo[k]) / bucket) + 1.0;
        if (g > 4096.0) return fail(ctx, ISO_ERR_TOO_LARGE, "more than 4096 buckets along an axis: use larger buckets");
        B.lo[k] = lo[k];
        B.g[k] = (uint32_t)g;
        nbk *= B.g[k];
    }
    B.inv_b = 1.0f / bucket;
    if (nbk > (1ull << 28)) return fail(ctx, ISO_ERR_TOO_LARGE, "bucket grid too large: use larger buckets");
    const uint64_t nmax = std::max(na, nb);
    // aux: points (a, b), sorted float4 copy, bucket ids, counts/starts, scan sums, accumulators
    const size_t bytes = 12 * (na + nb) + 16 * nmax + 4 * nmax + 8 * (nbk + 1) + 4 * ((nbk + 1023) / 1024 + 64) + 4096;
    if ((s = ensure(ctx, ctx->aux, bytes)) != ISO_OK) return s;
    char* base = (char*)ctx->aux.p;
    size_t at = 0;
    auto take = [&](size_t n) {
        at = (at + 255) & ~(size_t)255;
        char* p = base + at;
        at += n;
        return p;
    };
    float* da = (float*)take(12 * na);
    float* db = (float*)take(12 * nb);
    float4* sorted = (float4*)take(16 * nmax);
    uint32_t* bucket_of = (uint32_t*)take(4 * nmax);
    uint32_t* counts = (uint32_t*)take(4 * (nbk + 1));
    uint32_t* start = (uint32_t*)take(4 * (nbk + 1));
    uint32_t* sums = (uint32_t*)take(4 * ((nbk + 1 + 1023) / 1024 + 64));
    double* acc = (double*)take(64);  // sum, max bits, capped
    cudaStream_t st = ctx->stream;
    cudaError_t e = cudaMemcpyAsync(da, a, 12 * na, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(db, b, 12 * nb, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "upload vertices");
    double res_sum[2], res_max[2];
    uint64_t capped = 0;
    for (int dir = 0; dir < 2; ++dir) {
        const float* set = dir == 0 ? db : da;  // bucketed
        const float* qry = dir == 0 ? da : db;
        const uint32_t ns = (uint32_t)(dir == 0 ? nb : na), nq = (uint32_t)(dir == 0 ? na : nb);
        e = cudaMemsetAsync(counts, 0, 4 * (nbk + 1), st);
        if (e == cudaSuccess) e = cudaMemsetAsync(acc, 0, 64, st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "distance scratch");
        bucket_count<<<blocks_for(ns, 256), 256, 0, st>>>(set, ns, B, counts, bucket_of);
        ctx->launches++;
        if ((s = scan_u32(ctx, counts, start, (uint32_t)(nbk + 1), sums, (uint32_t*)(acc + 7))) != ISO_OK) return s;
        e = cudaMemcpyAsync(counts, start, 4 * (nbk + 1), cudaMemcpyDeviceToDevice, st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "bucket cursor");
        bucket_fill<<<blocks_for(ns, 256), 256, 0, st>>>(set, ns, bucket_of, counts, sorted);
        QueryArgs q{qry, nq, B, start, sorted, max_rings, acc, (unsigned int*)(acc + 1),
                    (unsigned long long*)(acc + 2)};
        nearest<<<blocks_for(nq, 256), 256, 0, st>>>(q);
        ctx->launches += 2;
        if ((s = check_launch(ctx, "nearest")) != ISO_OK) return s;
        double h[3];
        e = cudaMemcpyAsync(h, acc, 24, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "distance results");
        res_sum[dir] = h[0] / (double)nq;
        unsigned int mb;
        std::memcpy(&mb, &h[1], 4);
        float mf;
        std::memcpy(&mf, &mb, 4);
        res_max[dir] = mf;
        uint64_t c;
        std::memcpy(&c, &h[2], 8);
        capped += c;
    }
    out->mean_ab = res_sum[0];
    out->mean_ba = res_sum[1];
    out->max_ab = res_max[0];
    out->max_ba = res_max[1];
    out->capped = capped;
    return ISO_OK;
}

iso_status iso_field_case_disagreement(iso_ctx* ctx, const float* fa, const float* fb, uint32_t nx, uint32_t ny,
                                       uint32_t nz, uint64_t pitch, uint64_t* cells) {
    iso::NvtxRange nvtx_range("iso_field_case_disagreement");
    if (!ctx || !fa || !fb || !cells) return ISO_ERR_INVALID_ARG;
    if (nx < 2 || ny < 2 || nz < 2 || pitch < nx) return fail(ctx, ISO_ERR_INVALID_ARG, "need n >= 2, pitch >= nx");
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    const uint32_t W = words_per_row(nx);
    const uint64_t words = (uint64_t)W * ny * nz;
    if ((s = ensure(ctx, ctx->aux3, 8 * words + 256)) != ISO_OK) return s;
    uint32_t* ba = (uint32_t*)ctx->aux3.p;
    uint32_t* bb = ba + words;
    unsigned long long* acc = (unsigned long long*)(bb + words);  // byte offset 8 * words
    if ((s = launch_sign_bits(ctx, fa, nx, ny, nz, pitch, ba)) != ISO_OK) return s;
    if ((s = launch_sign_bits(ctx, fb, nx, ny, nz, pitch, bb)) != ISO_OK) return s;
    cudaError_t e = cudaMemsetAsync(acc, 0, 8, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "case count");
    const uint64_t threads = (uint64_t)(ny - 1) * (nz - 1) * W;
    case_diff<<<blocks_for(threads, 256), 256, 0, ctx->stream>>>(ba, bb, nx, ny, nz, W, acc);
    ctx->launches++;
    if ((s = check_launch(ctx, "case disagreement")) != ISO_OK) return s;
    e = cudaMemcpyAsync(ctx->h_pinned, acc, 8, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "case count");
    *cells = *(uint64_t*)ctx->h_pinned;
    return ISO_OK;
}

}  // extern "C"
