// Grid sampling: the sample loops of PrimalGrid::traverse
// (src/traversal/primal_grid.rs:44-70) as one kernel that writes the f32 field
// and, with warp ballots, the packed sign bits (bit set iff !(v > 0),
// classify_corners, marching_cubes_impl.rs:26-37) that the marching-cubes
// passes classify from.
//
// Point (x, y, z) sits at (x*inv, y*inv, z*inv), inv = 1/(size-1) in f32, as
// in the reference.  Built with -fmad=false: the values are bit-identical to
// the reference's f32 evaluation.
#include <cuda_runtime.h>

#include <utility>

#include "internal.h"
#include "vm.cuh"

namespace iso {
namespace {

constexpr uint32_t FULL = 0xFFFFFFFFu;

// One warp per (32-point chunk, row): generic program evaluator.
__global__ void __launch_bounds__(256) sample_generic(ProgView pv, uint32_t nx, uint32_t ny, uint32_t nz, float inv,
                                                      float* field, uint64_t pitch, uint32_t* bits, uint32_t W) {
    const int lane = threadIdx.x & 31;
    const uint64_t gw = (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5);
    if (gw >= (uint64_t)W * ny * nz) return;
    const uint32_t w = (uint32_t)(gw % W);
    const uint64_t row = gw / W;
    const uint32_t y = (uint32_t)(row % ny), z = (uint32_t)(row / ny);
    const uint32_t x = 32 * w + lane;
    bool inside = false;
    if (x < nx) {
        float v = eval_scalar(pv, v3((float)x * inv, (float)y * inv, (float)z * inv));
        field[row * pitch + x] = v;
        inside = !(v > 0.0f);
    }
    uint32_t b = __ballot_sync(FULL, inside);
    if (lane == 0) bits[row * W + w] = b;
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
constexpr int KEEP_REGS = 6;  // kept spheres held in registers (more: shared-memory loop)

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
};

__device__ __forceinline__ float world(float g, float s, float o, bool dom) { return dom ? g * s + o : g; }

// One thread's z column with the N kept spheres in registers.  (dx*dx + dy*dy)
// is shared by the whole column and is exactly len_sq's first partial sum.
template <int N>
__device__ __forceinline__ void sphere_column(const SetArgs& A, const float4* keep, float px, float py, uint32_t x,
                                              uint32_t y, uint32_t z0, uint32_t z1, bool valid, int lane) {
    float dxy[N], cz[N], cr[N];
#pragma unroll
    for (int i = 0; i < N; ++i) {
        const float4 c = keep[i];
        const float dx = px - c.x, dy = py - c.y;
        dxy[i] = dx * dx + dy * dy;
        cz[i] = c.z;
        cr[i] = c.w;
    }
#pragma unroll 2
    for (uint32_t z = z0; z <= z1; ++z) {
        const float pz = world((float)z * A.inv, A.sz, A.oz, A.domain);
        float dz = pz - cz[0];
        float v = sqrtf(dxy[0] + dz * dz) - cr[0];
#pragma unroll
        for (int i = 1; i < N; ++i) {
            dz = pz - cz[i];
            v = fminf(v, sqrtf(dxy[i] + dz * dz) - cr[i]);
        }
        const size_t row = (size_t)z * A.ny + y;
        if (valid) A.field[row * A.pitch + x] = v;
        const uint32_t b = __ballot_sync(0xFFFFFFFFu, valid && !(v > 0.0f));
        if (lane == 0) A.bits[row * A.W + blockIdx.x] = b;
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
    float az = world((float)z0 * A.inv, A.sz, A.oz, A.domain), bz = world((float)z1 * A.inv, A.sz, A.oz, A.domain);
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
        }
        uint32_t m = __ballot_sync(FULL, keep);
        if (lane == 0) s_cnt[warp] = __popc(m);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int wv = 0; wv < 8; ++wv) {
            if (wv < warp) before += s_cnt[wv];
            total += s_cnt[wv];
        }
        if (keep) s_keep[base + before + __popc(m & ((1u << lane) - 1u))] = c;
        base += total;
        __syncthreads();
    }
    if (threadIdx.x == 0) s_nkeep = base;
    __syncthreads();
    const uint32_t nk = s_nkeep;

    const uint32_t x = x0 + lane, y = y0 + warp;
    if (y >= A.ny) return;
    const float px = world((float)x * A.inv, A.sx, A.ox, A.domain);
    const float py = world((float)y * A.inv, A.sy, A.oy, A.domain);
    const bool valid = x < A.nx;
    switch (nk) {
    case 1: sphere_column<1>(A, s_keep, px, py, x, y, z0, z1, valid, lane); return;
    case 2: sphere_column<2>(A, s_keep, px, py, x, y, z0, z1, valid, lane); return;
    case 3: sphere_column<3>(A, s_keep, px, py, x, y, z0, z1, valid, lane); return;
    case 4: sphere_column<4>(A, s_keep, px, py, x, y, z0, z1, valid, lane); return;
    case 5: sphere_column<5>(A, s_keep, px, py, x, y, z0, z1, valid, lane); return;
    case 6: sphere_column<6>(A, s_keep, px, py, x, y, z0, z1, valid, lane); return;
    default: break;
    }
    for (uint32_t z = z0; z <= z1; ++z) {
        const float pz = world((float)z * A.inv, A.sz, A.oz, A.domain);
        float v = 0.0f;
        for (uint32_t i = 0; i < nk; ++i) {
            float4 c = s_keep[i];
            float d = vlen(v3(px - c.x, py - c.y, pz - c.z)) - c.w;
            v = (i == 0) ? d : fminf(v, d);
        }
        const uint64_t row = (uint64_t)z * A.ny + y;
        if (valid) A.field[row * A.pitch + x] = v;
        uint32_t b = __ballot_sync(FULL, valid && !(v > 0.0f));
        if (lane == 0) A.bits[row * A.W + blockIdx.x] = b;
    }
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

iso_status launch_sample_grid(iso_ctx* ctx, const iso_program* prog, uint32_t nx, uint32_t ny, uint32_t nz, float inv,
                              float* field, uint64_t pitch, uint32_t* bits) {
    const uint32_t W = words_per_row(nx);
    if (prog->kind == PK_SPHERE_SET_HARD && prog->set_n <= 8192) {
        SetArgs a;
        a.spheres = prog->d_set;
        a.n = prog->set_n;
        a.domain = prog->has_domain;
        a.sx = prog->domain[0]; a.sy = prog->domain[1]; a.sz = prog->domain[2];
        a.ox = prog->domain[3]; a.oy = prog->domain[4]; a.oz = prog->domain[5];
        a.nx = nx; a.ny = ny; a.nz = nz; a.inv = inv;
        a.field = field; a.pitch = pitch; a.bits = bits; a.W = W;
        size_t smem = 16 * (size_t)prog->set_n;
        if (smem > 48 * 1024) {
            cudaError_t e = cudaFuncSetAttribute(sample_sphere_set, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e != cudaSuccess) return cuda_fail(ctx, e, "sphere-set smem attribute");
        }
        dim3 grid(W, (ny + 7) / 8, (nz + TZ - 1) / TZ);
        StageTimer timer(ctx, ISO_STAGE_SAMPLE);
        sample_sphere_set<<<grid, 256, smem, ctx->stream>>>(a);
    } else {
        uint64_t warps = (uint64_t)W * ny * nz;
        StageTimer timer(ctx, ISO_STAGE_SAMPLE);
        sample_generic<<<(unsigned)((warps + 7) / 8), 256, 0, ctx->stream>>>(prog->view(), nx, ny, nz, inv, field, pitch,
                                                                          bits, W);
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
