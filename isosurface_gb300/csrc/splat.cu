// Deferred point-splat rendering of a PointCloud with interleaved normals: the
// technique of examples/deferred_rasterisation.rs (its GLSL passes, lines
// 95-127 and 131-213, driven as in lines 342-421), as CUDA kernels writing a
// headless float RGBA image instead of a GL framebuffer.
//
//   splat_points   every point to the pixel its clip position falls in,
//                  depth-tested as GL_LESS does (nearest depth, then earliest
//                  point) with a 64-bit atomicMin of (depth bits, index);
//   splat_gbuffer  position (xyz, 1) and normalised normal of each pixel's
//                  point, zeros for empty pixels;
//   splat_gather   along one image axis, 16 taps either side: the pixel's eye
//                  ray (from the near-plane centre through its far-plane
//                  point) against the cube of half-size `voxel` around each
//                  tap's point, the nearest hit kept (ties: the later tap);
//                  three passes along x, y, x, then a last one along y that
//                  shades hits with the hemisphere term and composites over
//                  the clear colour.
// Row 0 is the bottom row (GL's window convention); taps outside the image
// read as empty, or, with ISO_SPLAT_MIRROR_EDGES, through mirrored-repeat
// addressing (the wrap of the sampler the example reads its buffers with).  Every expression has a fixed f32 operation order (this unit
// is compiled without FMA contraction), restated by the numpy oracle.
#include <cuda_runtime.h>

#include "internal.h"

namespace iso {
namespace {

struct Mat4 {
    float m[16];  // column-major: element (row r, column c) at m[4 c + r]
};

struct Vec4 {
    float x, y, z, w;
};

__device__ __forceinline__ Vec4 mat_vec(const Mat4& M, float x, float y, float z, float w) {
    Vec4 r;
    r.x = ((M.m[0] * x + M.m[4] * y) + M.m[8] * z) + M.m[12] * w;
    r.y = ((M.m[1] * x + M.m[5] * y) + M.m[9] * z) + M.m[13] * w;
    r.z = ((M.m[2] * x + M.m[6] * y) + M.m[10] * z) + M.m[14] * w;
    r.w = ((M.m[3] * x + M.m[7] * y) + M.m[11] * z) + M.m[15] * w;
    return r;
}

constexpr unsigned long long EMPTY = ~0ull;
constexpr int TAPS = 16;
constexpr float NO_HIT = 9999999.0f;

__global__ void splat_points(const float* pn, uint64_t n, Mat4 mvp, uint32_t width, uint32_t height,
                             unsigned long long* zbuf) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float* q = pn + 6 * i;
    const Vec4 c = mat_vec(mvp, q[0], q[1], q[2], 1.0f);
    if (!(c.w > 0.0f)) return;
    const float nx = c.x / c.w, ny = c.y / c.w, nz = c.z / c.w;
    if (!(nx >= -1.0f && nx <= 1.0f && ny >= -1.0f && ny <= 1.0f && nz >= -1.0f && nz <= 1.0f)) return;
    const float xw = (nx + 1.0f) * ((float)width * 0.5f), yw = (ny + 1.0f) * ((float)height * 0.5f);
    const uint32_t ix = min((uint32_t)floorf(xw), width - 1), iy = min((uint32_t)floorf(yw), height - 1);
    const float depth = nz * 0.5f + 0.5f;  // in [0, 1], so its bits order like its values
    atomicMin(zbuf + (size_t)iy * width + ix, ((unsigned long long)__float_as_uint(depth) << 32) | i);
}

__global__ void splat_gbuffer(const float* pn, const unsigned long long* zbuf, uint64_t npix, float4* pos,
                              float4* nrm) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npix) return;
    const unsigned long long key = zbuf[p];
    if (key == EMPTY) {
        pos[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        nrm[p] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float* q = pn + 6 * (key & 0xFFFFFFFFull);
    pos[p] = make_float4(q[0], q[1], q[2], 1.0f);
    const float len = sqrtf((q[3] * q[3] + q[4] * q[4]) + q[5] * q[5]);
    nrm[p] = make_float4(q[3] / len, q[4] / len, q[5] / len, 0.0f);
}

struct GatherArgs {
    const float4* spos;
    const float4* snrm;
    float4* dpos;  // non-last passes
    float4* dnrm;
    float4* out;   // last pass: composited RGBA
    uint32_t width, height;
    Mat4 vpinv;
    float voxel;
    int dx, dy, last;
    int mirror;    // taps past the edge: 0 empty, 1 mirrored repeat
    float clear[3];
};

// mirrored-repeat addressing of texel i in a row of n: -1 -> 0, n -> n - 1, ...
__device__ __forceinline__ int mirror_index(int i, int n) {
    int m = i % (2 * n);
    if (m < 0) m += 2 * n;
    return m >= n ? 2 * n - 1 - m : m;
}

__global__ void splat_gather(GatherArgs A) {
    const uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= (uint64_t)A.width * A.height) return;
    const int ix = (int)(p % A.width), iy = (int)(p / A.width);
    const Vec4 e = mat_vec(A.vpinv, 0.0f, 0.0f, -1.0f, 1.0f);
    const float ex = e.x / e.w, ey = e.y / e.w, ez = e.z / e.w;
    const float ndx = (float)(2 * ix + 1) / (float)A.width - 1.0f;
    const float ndy = (float)(2 * iy + 1) / (float)A.height - 1.0f;
    const Vec4 s = mat_vec(A.vpinv, ndx, ndy, 1.0f, 1.0f);
    const float sx = s.x / s.w - ex, sy = s.y / s.w - ey, sz = s.z / s.w - ez;
    const float len = sqrtf((sx * sx + sy * sy) + sz * sz);
    const float ix_ = 1.0f / (sx / len), iy_ = 1.0f / (sy / len), iz_ = 1.0f / (sz / len);
    float best = NO_HIT;
    float3 res = make_float3(0.0f, 0.0f, 0.0f), rn = make_float3(0.0f, 0.0f, 0.0f);
    for (int t = -TAPS; t <= TAPS; ++t) {
        int tx = ix + t * A.dx, ty = iy + t * A.dy;
        if (A.mirror) {
            tx = mirror_index(tx, (int)A.width);
            ty = mirror_index(ty, (int)A.height);
        } else if (tx < 0 || tx >= (int)A.width || ty < 0 || ty >= (int)A.height) {
            continue;
        }
        const size_t at = (size_t)ty * A.width + tx;
        const float4 q = A.spos[at];
        if (!((fabsf(q.x) + fabsf(q.y)) + fabsf(q.z) > 0.0f)) continue;
        const float bx = ix_ * ((q.x - A.voxel) - ex), tx_ = ix_ * ((q.x + A.voxel) - ex);
        const float by = iy_ * ((q.y - A.voxel) - ey), ty_ = iy_ * ((q.y + A.voxel) - ey);
        const float bz = iz_ * ((q.z - A.voxel) - ez), tz_ = iz_ * ((q.z + A.voxel) - ez);
        const float mnx = fminf(tx_, bx), mny = fminf(ty_, by), mnz = fminf(tz_, bz);
        const float mxx = fmaxf(tx_, bx), mxy = fmaxf(ty_, by), mxz = fmaxf(tz_, bz);
        const float t0 = fmaxf(fmaxf(mnx, mny), fmaxf(mnx, mnz));
        const float t1 = fminf(fminf(mxx, mxy), fminf(mxx, mxz));
        if (t0 <= t1 && t0 <= best) {
            best = t0;
            res = make_float3(q.x, q.y, q.z);
            const float4 nn = A.snrm[at];
            rn = make_float3(nn.x, nn.y, nn.z);
        }
    }
    if (!A.last) {
        A.dpos[p] = make_float4(res.x, res.y, res.z, 0.0f);
        A.dnrm[p] = make_float4(rn.x, rn.y, rn.z, 0.0f);
        return;
    }
    if (best < NO_HIT) {
        // hemisphere(normal), light (0.1, -1, 0), mix(c1, c2, N.L * 0.5 + 0.5)
        const float ndl = ((rn.x * 0.1f + rn.y * -1.0f) + rn.z * 0.0f) * 0.5f + 0.5f;
        const float om = 1.0f - ndl;
        A.out[p] = make_float4(0.886f * om + 0.518f * ndl, 0.757f * om + 0.169f * ndl, 0.337f * om + 0.0f * ndl,
                               1.0f);
    } else {
        A.out[p] = make_float4(A.clear[0], A.clear[1], A.clear[2], 0.0f);
    }
}

}  // namespace
}  // namespace iso

using namespace iso;

extern "C" {

iso_status iso_point_splat_render_ex(iso_ctx* ctx, const float* view_proj, const float* view_proj_inverse,
                                     uint32_t width, uint32_t height, float voxel_half, const float* clear_rgb,
                                     uint32_t flags, float* rgba) {
    iso::NvtxRange nvtx_range("iso_point_splat_render");
    if (!ctx) return ISO_ERR_INVALID_ARG;
    if (flags & ~(uint32_t)ISO_SPLAT_MIRROR_EDGES) return fail(ctx, ISO_ERR_INVALID_ARG, "unsupported flags");
    if (!view_proj || !view_proj_inverse || !clear_rgb || !rgba)
        return fail(ctx, ISO_ERR_INVALID_ARG, "null matrix, colour or image pointer");
    if (width == 0 || height == 0 || width > 16384 || height > 16384)
        return fail(ctx, ISO_ERR_INVALID_ARG, "image size must be 1..16384 per side");
    if (ctx->last_vertex_floats != 6 || ctx->last.num_triangles != 0)
        return fail(ctx, ISO_ERR_INVALID_ARG, "the last extraction is not a point cloud with normals");
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    const uint64_t npix = (uint64_t)width * height, n = ctx->last.num_vertices;
    // the depth test's 64-bit key holds the point index in its low 32 bits
    if (n > 0xFFFFFFFFull) return fail(ctx, ISO_ERR_TOO_LARGE, "point cloud above 2^32 points");
    // z-buffer | two position + normal buffer pairs | composited image
    const size_t zbytes = (8 * npix + 255) & ~(size_t)255, fbytes = 16 * npix;
    if ((s = ensure(ctx, ctx->aux, zbytes + 5 * fbytes)) != ISO_OK) return s;
    unsigned long long* zbuf = (unsigned long long*)ctx->aux.p;
    float4* posA = (float4*)((char*)ctx->aux.p + zbytes);
    float4* nrmA = posA + npix;
    float4* posB = nrmA + npix;
    float4* nrmB = posB + npix;
    float4* out = nrmB + npix;
    Mat4 vp, vpi;
    for (int i = 0; i < 16; ++i) {
        vp.m[i] = view_proj[i];
        vpi.m[i] = view_proj_inverse[i];
    }
    StageTimer timer(ctx, ISO_STAGE_OTHER);
    cudaError_t e = cudaMemsetAsync(zbuf, 0xFF, 8 * npix, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "clear depth buffer");
    const unsigned pix_blocks = (unsigned)((npix + 255) / 256);
    if (n) splat_points<<<(unsigned)((n + 255) / 256), 256, 0, ctx->stream>>>((const float*)ctx->mesh_v.p, n, vp,
                                                                              width, height, zbuf);
    splat_gbuffer<<<pix_blocks, 256, 0, ctx->stream>>>((const float*)ctx->mesh_v.p, zbuf, npix, posA, nrmA);
    // three gathers along x, y, x (A -> B -> A -> B), then the last along y
    GatherArgs g{};
    g.width = width;
    g.height = height;
    g.vpinv = vpi;
    g.voxel = voxel_half;
    g.mirror = (flags & ISO_SPLAT_MIRROR_EDGES) ? 1 : 0;
    for (int k = 0; k < 3; ++k) g.clear[k] = clear_rgb[k];
    for (int i = 0; i < 4; ++i) {
        const bool from_a = (i % 2) == 0;
        g.spos = from_a ? posA : posB;
        g.snrm = from_a ? nrmA : nrmB;
        g.dpos = from_a ? posB : posA;
        g.dnrm = from_a ? nrmB : nrmA;
        g.out = out;
        g.dx = i < 3 ? (i + 1) % 2 : 0;
        g.dy = i < 3 ? i % 2 : 1;
        g.last = i == 3;
        splat_gather<<<pix_blocks, 256, 0, ctx->stream>>>(g);
    }
    ctx->launches += (n ? 6 : 5);
    if ((s = check_launch(ctx, "point splat")) != ISO_OK) return s;
    e = cudaMemcpyAsync(rgba, out, fbytes, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, "image readback");
}

iso_status iso_point_splat_render(iso_ctx* ctx, const float* view_proj, const float* view_proj_inverse,
                                  uint32_t width, uint32_t height, float voxel_half, const float* clear_rgb,
                                  float* rgba) {
    return iso_point_splat_render_ex(ctx, view_proj, view_proj_inverse, width, height, voxel_half, clear_rgb, 0,
                                     rgba);
}

}  // extern "C"
