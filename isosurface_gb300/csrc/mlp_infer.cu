// BF16 tensor-core inference of the surrogate MLP on sm_103a (tcgen05).
//
// One CTA of 128 threads runs tiles of M = 128 points through the whole
// network:
//   * features / activations: the A operand, 128 rows x K bf16 in shared
//     memory, K-major with the 128-byte swizzle, as K-blocks of 64 columns
//     (16 KB each; layer 0's 96 features are padded to 128);
//   * weights of the current layer: the B operand, 256 rows (N) x K bf16, the
//     same layout; they are copied from a pre-swizzled bf16 image made once
//     per parameter update (prepare_images);
//   * one thread issues tcgen05.mma.cta_group::1.kind::f16 (M=128, N=256,
//     K=16, fp32 accumulate) into a 256-column TMEM accumulator and commits to
//     an mbarrier; every wait on it is bounded (error flag, TMEM still freed);
//   * epilogue: each warp reads its 32 TMEM lanes (rows) with tcgen05.ld,
//     adds the bias, applies softplus_beta and writes the bf16 operand of the
//     next layer; after the last layer it dots with w_out (fp32) instead.
// Descriptor formats (tcgen05 shared-memory matrix descriptor and the
// kind::f16 instruction descriptor) follow the PTX ISA for sm_100-class MMA.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <vector>

#include "internal.h"
#include "mlp.h"

using namespace iso;
using namespace iso::mlp;

struct MlpImages {
    __nv_bfloat16* w = nullptr;  // per layer: NK/64 K-blocks of 256 rows x 128 B, swizzled
    float* bias = nullptr;       // NLAYERS x 256
    float* wout = nullptr;       // 256 + 1
    bool valid = false;
};

namespace {

constexpr int KB0 = 2;                 // layer 0: K padded 96 -> 128
constexpr int KB = HID / 64;           // layers 1..5: K = 256
constexpr size_t KBLOCK_BYTES_B = 256 * 128;   // 256 rows x 64 bf16
constexpr size_t KBLOCK_BYTES_A = 128 * 128;   // 128 rows x 64 bf16
constexpr uint32_t WAIT_LIMIT = 1u << 26;

__host__ __device__ constexpr size_t image_offset(int l) {  // in bf16 elements
    return l == 0 ? 0 : (size_t)KB0 * 256 * 64 + (size_t)(l - 1) * KB * 256 * 64;
}
constexpr size_t IMAGE_ELEMS = image_offset(NLAYERS);

// byte offset of element (row, k) in a swizzled K-major operand of `rows` rows
__host__ __device__ __forceinline__ uint32_t swz(uint32_t row, uint32_t k, uint32_t rows) {
    const uint32_t kb = k >> 6, c = (k & 63) >> 3, e = k & 7;
    return kb * rows * 128 + row * 128 + ((c ^ (row & 7)) << 4) + e * 2;
}

__global__ void prepare_images(const float* params, __nv_bfloat16* w, float* bias, float* wout) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    // weights
    if (i < IMAGE_ELEMS) {
        int l = 0;
        while (l + 1 < NLAYERS && i >= image_offset(l + 1)) ++l;
        const uint32_t local = i - (uint32_t)image_offset(l);
        const uint32_t K = l == 0 ? FF : HID;
        const uint32_t row = local / (l == 0 ? KB0 * 64 : KB * 64), k = local % (l == 0 ? KB0 * 64 : KB * 64);
        const float v = k < K ? params[weight_offset(l) + (size_t)row * K + k] : 0.0f;
        unsigned char* base = reinterpret_cast<unsigned char*>(w + image_offset(l));
        *reinterpret_cast<__nv_bfloat16*>(base + swz(row, k, 256)) = __float2bfloat16_rn(v);
    }
    if (i < NLAYERS * HID) bias[i] = params[bias_offset(i / HID) + i % HID];
    if (i < HID + 1) wout[i] = params[OUT_W + i];
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFF) >> 4);  // start address
    d |= (uint64_t)1 << 16;                   // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset: 8 rows x 128 B
    d |= (uint64_t)1 << 46;                   // descriptor version
    d |= (uint64_t)2 << 61;                   // 128-byte swizzle
    return d;
}

// kind::f16: fp32 D, bf16 A and B, both K-major, N = 256, M = 128
constexpr uint32_t IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((256u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ void mma(uint32_t tmem, uint64_t a, uint64_t b, uint32_t acc) {
    asm volatile(
        "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
        "l"(a), "l"(b), "r"(IDESC), "r"(acc));
}

__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t phase) {
    for (uint32_t it = 0; it < WAIT_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(phase)
            : "memory");
        if (done) return true;
    }
    return false;
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float softplus_b(float z) {
    return fmaxf(z, 0.0f) + log1pf(__expf(-BETA * fabsf(z))) * (1.0f / BETA);
}

__device__ __forceinline__ float ffreq(int j) { return 3.14159265358979f * exp2f((float)(7 * j) / 15.0f); }

struct InferArgs {
    const __nv_bfloat16* w;
    const float* bias;
    const float* wout;
    // points: either explicit (pts != null, n points, out[i]) or a grid of
    // nx x ny x nz lattice points (i, j, k) at p = (i*step*inv, j*step*inv,
    // k*step*inv) mapped by q = p * scale + offset, out[(k*ny + j)*nx + i]
    const float* pts;
    uint64_t n;
    uint32_t nx, ny, nz, step;
    float inv;
    float scale[3], offset[3];
    float* out;
    uint32_t* err;
};

__device__ __forceinline__ void point_of(const InferArgs& A, uint64_t i, float* q) {
    if (A.pts) {
        q[0] = A.pts[3 * i];
        q[1] = A.pts[3 * i + 1];
        q[2] = A.pts[3 * i + 2];
        return;
    }
    const uint32_t x = (uint32_t)(i % A.nx);
    const uint64_t r = i / A.nx;
    const uint32_t y = (uint32_t)(r % A.ny), z = (uint32_t)(r / A.ny);
    // unfused, so that a host computing the same points in f32 feeds the
    // network identical coordinates
    q[0] = __fadd_rn(__fmul_rn(__fmul_rn((float)(x * A.step), A.inv), A.scale[0]), A.offset[0]);
    q[1] = __fadd_rn(__fmul_rn(__fmul_rn((float)(y * A.step), A.inv), A.scale[1]), A.offset[1]);
    q[2] = __fadd_rn(__fmul_rn(__fmul_rn((float)(z * A.step), A.inv), A.scale[2]), A.offset[2]);
}

constexpr size_t SMEM_A = 4 * KBLOCK_BYTES_A;          // 64 KB
constexpr size_t SMEM_B = 4 * KBLOCK_BYTES_B;          // 128 KB
constexpr size_t SMEM_TOTAL = SMEM_A + SMEM_B + 1024;  // + alignment slack

__global__ void __launch_bounds__(128, 1) mlp_infer_kernel(InferArgs A) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t s_mbar;
    __shared__ uint32_t s_tmem;
    unsigned char* smem = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = smem;
    unsigned char* sB = smem + SMEM_A;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;\n" ::"r"(smem_u32(&s_tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_u32(&s_mbar)));
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = s_tmem;
    const uint32_t mbar = smem_u32(&s_mbar);
    uint32_t phase = 0;
    bool aborted = false;
    const uint64_t ntiles = (A.n + 127) / 128;
    for (uint64_t tile = blockIdx.x; tile < ntiles && !aborted; tile += gridDim.x) {
        const uint64_t pidx = tile * 128 + tid;
        float q[3] = {0.0f, 0.0f, 0.0f};
        if (pidx < A.n) point_of(A, pidx, q);
        // Fourier features of this thread's point into row tid of A (K padded to 128)
        for (int k = 0; k < KB0 * 64; k += 2) {
            float v0 = 0.0f, v1 = 0.0f;
            if (k < FF) {
                const int a = k / 32, j = (k % 32) / 2;
                float s, c;
                sincosf(ffreq(j) * q[a], &s, &c);
                v0 = s;
                v1 = c;
            }
            *reinterpret_cast<__nv_bfloat162*>(sA + swz(tid, k, 128)) = __floats2bfloat162_rn(v0, v1);
        }
        float y = 0.0f;
        for (int l = 0; l < NLAYERS; ++l) {
            const int kblocks = l == 0 ? KB0 : KB;
            // weights of layer l into B (plain 16-byte copies of the swizzled image)
            const uint4* src = reinterpret_cast<const uint4*>(A.w + image_offset(l));
            uint4* dst = reinterpret_cast<uint4*>(sB);
            const int n16 = (int)(kblocks * KBLOCK_BYTES_B / 16);
            for (int i = tid; i < n16; i += 128) dst[i] = __ldg(src + i);
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            if (tid == 0) {
                for (int kb = 0; kb < kblocks; ++kb)
                    for (int s = 0; s < 4; ++s) {
                        const uint64_t ad = sdesc(smem_u32(sA + kb * KBLOCK_BYTES_A + s * 32));
                        const uint64_t bd = sdesc(smem_u32(sB + kb * KBLOCK_BYTES_B + s * 32));
                        mma(tmem, ad, bd, (kb | s) ? 1u : 0u);
                    }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 mbar)
                             : "memory");
            }
            const bool ok = mbar_wait(mbar, phase);
            if (__syncthreads_or(!ok)) {  // block-uniform: every thread leaves together
                if (tid == 0) atomicOr(A.err, DERR_QUEUE_TIMEOUT);
                if (ok == false) mbar_wait(mbar, phase);  // bounded: let the MMAs drain before TMEM is freed
                aborted = true;
                break;
            }
            phase ^= 1;
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            // epilogue: row tid of the accumulator
            const float* bias = A.bias + l * HID;
            const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
            for (int c0 = 0; c0 < HID; c0 += 16) {
                float v[16];
                tmem_ld16(lane_base + c0, v);
#pragma unroll
                for (int i = 0; i < 16; ++i) v[i] = softplus_b(v[i] + __ldg(bias + c0 + i));
                if (l + 1 < NLAYERS) {
#pragma unroll
                    for (int i = 0; i < 16; i += 2)
                        *reinterpret_cast<__nv_bfloat162*>(sA + swz(tid, c0 + i, 128)) =
                            __floats2bfloat162_rn(v[i], v[i + 1]);
                } else {
#pragma unroll
                    for (int i = 0; i < 16; ++i) y += v[i] * __ldg(A.wout + c0 + i);
                }
            }
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncthreads();
        }
        if (pidx < A.n && !aborted) {
            A.out[pidx] = y + __ldg(A.wout + HID);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;\n" ::"r"(tmem));
}

}  // namespace

namespace iso {

static MlpImages* images_of(iso_mlp* net) {
    if (!net->infer) net->infer = new MlpImages();
    return (MlpImages*)net->infer;
}

void mlp_infer_release(iso_mlp* net) {
    MlpImages* m = (MlpImages*)net->infer;
    if (!m) return;
    if (m->w) cudaFree(m->w);
    delete m;
    net->infer = nullptr;
}

void mlp_infer_invalidate(iso_mlp* net) {
    if (net->infer) ((MlpImages*)net->infer)->valid = false;
}

static iso_status ready(iso_mlp* net, MlpImages** out) {
    iso_ctx* ctx = net->ctx;
    MlpImages* m = images_of(net);
    if (!m->w) {
        void* p = nullptr;
        cudaError_t e = cudaMalloc(&p, IMAGE_ELEMS * 2 + 4 * (NLAYERS * HID + HID + 1) + 256);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "mlp images");
        m->w = (__nv_bfloat16*)p;
        m->bias = (float*)((char*)p + ((IMAGE_ELEMS * 2 + 255) & ~(size_t)255));
        m->wout = m->bias + NLAYERS * HID;
    }
    if (!m->valid) {
        prepare_images<<<(unsigned)((IMAGE_ELEMS + 255) / 256), 256, 0, ctx->stream>>>(net->params, m->w,
                                                                                     m->bias, m->wout);
        ctx->launches++;
        iso_status s = check_launch(ctx, "prepare images");
        if (s != ISO_OK) return s;
        m->valid = true;
    }
    *out = m;
    return ISO_OK;
}

iso_status mlp_infer_launch(iso_mlp* net, const float* d_pts, uint64_t n, const MlpGrid* grid, float* d_out) {
    iso_ctx* ctx = net->ctx;
    MlpImages* m;
    iso_status s = ready(net, &m);
    if (s != ISO_OK) return s;
    InferArgs a{};
    a.w = m->w;
    a.bias = m->bias;
    a.wout = m->wout;
    a.pts = d_pts;
    a.n = n;
    if (grid) {
        a.nx = grid->nx;
        a.ny = grid->ny;
        a.nz = grid->nz;
        a.step = grid->step;
        a.inv = grid->inv;
        for (int i = 0; i < 3; ++i) {
            a.scale[i] = grid->scale[i];
            a.offset[i] = grid->offset[i];
        }
        a.n = (uint64_t)grid->nx * grid->ny * grid->nz;
    }
    a.out = d_out;
    a.err = ctx->d_err;
    cudaError_t e = cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)SMEM_TOTAL);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mlp smem attribute");
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (a.n == 0) return ISO_OK;
    const uint64_t tiles = (a.n + 127) / 128;
    const unsigned blocks = (unsigned)std::min<uint64_t>(tiles, (uint64_t)sms);
    {
        StageTimer timer(ctx, ISO_STAGE_MLP);
        mlp_infer_kernel<<<blocks, 128, SMEM_TOTAL, ctx->stream>>>(a);
    }
    ctx->launches++;
    return check_launch(ctx, "mlp infer");
}

}  // namespace iso

extern "C" iso_status iso_mlp_forward_bf16(iso_mlp* net, const float* pts, uint32_t n, float* values) {
    if (!net || (!pts && n) || (!values && n)) return ISO_ERR_INVALID_ARG;
    if (n == 0) return ISO_OK;
    iso_ctx* ctx = net->ctx;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->aux, 16ull * n + 256)) != ISO_OK) return s;
    float* d_pts = (float*)ctx->aux.p;
    float* d_out = d_pts + 3ull * n;
    cudaError_t e = cudaMemcpyAsync(d_pts, pts, 12ull * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "upload points");
    if ((s = mlp_infer_launch(net, d_pts, n, nullptr, d_out)) != ISO_OK) return s;
    e = cudaMemcpyAsync(values, d_out, 4ull * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mlp bf16 forward");
    return read_device_errors(ctx);
}
