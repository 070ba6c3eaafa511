// BF16 tensor-core inference of the surrogate MLP on sm_103a (tcgen05).
//
// One CTA of 256 threads per SM runs tiles of M = 128 points through the whole
// network:
//   * features / activations: the A operand, 128 rows x K bf16 in shared
//     memory, K-major with the 128-byte swizzle, as K-blocks of 64 columns
//     (16 KB each; layer 0's 96 features are padded to 128);
//   * weights: the B operand, 256 rows (N) x 64 K bf16 per K-block (32 KB),
//     the same layout, copied by TMA bulk copies from a pre-swizzled bf16
//     image made once per parameter update (prepare_images) into four slots;
//     the next layer's copies run during the current layer's epilogue;
//   * one thread issues tcgen05.mma.cta_group::1.kind::f16 (M=128, N=256,
//     K=16, fp32 accumulate) into a 256-column TMEM accumulator and commits to
//     an mbarrier; every wait is bounded (error flag, copies drained, TMEM
//     freed);
//   * epilogue: eight warps read the accumulator with tcgen05.ld (warp w: 32
//     lanes = rows, 128 columns), add the bias, apply softplus_beta and write
//     the bf16 operand of the next layer; after the last layer they dot with
//     w_out (fp32) instead.
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
constexpr uint64_t WAIT_NS = 1000000000ull;  // 1 s

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

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// parity wait on an mbarrier, bounded in polls and in time (about a second)
__device__ __forceinline__ bool mbar_wait(uint32_t addr, uint32_t phase) {
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; it < WAIT_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(phase)
            : "memory");
        if (done) return true;
        if ((it & 255u) == 255u && global_ns() - t0 > WAIT_NS) return false;
    }
    return false;
}

// 32 lanes x 16 columns of 32 bits from TMEM, without waiting
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

// wait for this thread's TMEM loads; the registers are tied to the wait so
// that no use of them moves above it
__device__ __forceinline__ void tmem_wait(uint32_t (&r)[16]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;\n"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15])
                 :
                 : "memory");
}

// packed f32x2 arithmetic (two lanes per instruction on sm_100-class SMs)
__device__ __forceinline__ uint64_t f2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void uf2(uint64_t v, float& a, float& b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v)); }
__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// softplus_beta of z + b for two lanes at once:
//   max(x, 0) + log1p(u) / beta,  u = exp(-beta |x|) = 2^(-|x| beta log2(e)),
// u from the MUFU, log1p(u) / beta = u * P(u) with P a degree-4 polynomial
// fitted here to log1p(u) / (beta u) on [0, 1] (least squares at Chebyshev
// nodes; maximum absolute error 1e-7 after the 1/beta scaling, far below the
// bf16 rounding of the result)
__device__ __forceinline__ uint64_t softplus2(uint64_t z, uint64_t b) {
    constexpr float K = BETA * 1.4426950408889634f;
    const uint64_t x = add2(z, b);
    float t0, t1;
    uf2(mul2(x, f2(K, K)), t0, t1);
    const uint64_t u = f2(ex2_approx(-fabsf(t0)), ex2_approx(-fabsf(t1)));
    uint64_t p = fma2(f2(0.000321511645f, 0.000321511645f), u, f2(-0.00136042002f, -0.00136042002f));
    p = fma2(p, u, f2(0.00289453869f, 0.00289453869f));
    p = fma2(p, u, f2(-0.00491900276f, -0.00491900276f));
    p = fma2(p, u, f2(0.00999494363f, 0.00999494363f));
    float x0, x1;
    uf2(x, x0, x1);
    return fma2(u, p, f2(fmaxf(x0, 0.0f), fmaxf(x1, 0.0f)));
}


__device__ __forceinline__ float ffreq(int j) { return 3.14159265358979f * exp2f((float)(7 * j) / 15.0f); }

// sin and cos of a = w_j x (|a| < ~500): Cody-Waite reduction by 2 pi with a
// two-term constant (the high term has 8 significant bits, so n * hi is exact
// for |n| < 2^16), then the MUFU sine / cosine on [-pi, pi]
__device__ __forceinline__ void sincos_reduced(float a, float* s, float* c) {
    constexpr float TWO_PI_HI = 6.28125f;
    constexpr float TWO_PI_LO = 1.9353071795864769e-3f;
    const float n = rintf(a * 0.15915494309189535f);
    float r = fmaf(-n, TWO_PI_HI, a);
    r = fmaf(-n, TWO_PI_LO, r);
    __sincosf(r, s, c);
}

struct InferArgs {
    const unsigned char* w;  // swizzled bf16 weight image (K-blocks of 32 KB)
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

constexpr int THREADS = 256;
constexpr size_t SMEM_A = 4 * KBLOCK_BYTES_A;          // 64 KB: activations, 4 K-blocks
constexpr size_t SMEM_B = 4 * KBLOCK_BYTES_B;          // 128 KB: weight slots, one K-block each
constexpr size_t SMEM_TOTAL = SMEM_A + SMEM_B + 1024;  // + alignment slack

__host__ __device__ constexpr int kblocks_of(int l) { return l == 0 ? KB0 : KB; }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count));
}

// weights of layer l into the slots: one bulk copy per K-block, completing
// on that slot's barrier
__device__ __forceinline__ void load_layer(const InferArgs& A, int l, uint32_t sB, uint32_t full0) {
    const unsigned char* src = A.w + 2 * image_offset(l);
    for (int kb = 0; kb < kblocks_of(l); ++kb) {
        const uint32_t bar = full0 + 8 * kb;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar),
                     "r"((uint32_t)KBLOCK_BYTES_B)
                     : "memory");
        asm volatile(
            "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                sB + kb * (uint32_t)KBLOCK_BYTES_B),
            "l"(src + kb * KBLOCK_BYTES_B), "r"((uint32_t)KBLOCK_BYTES_B), "r"(bar)
            : "memory");
    }
}

// One CTA per SM, 8 warps.  Warp w reads TMEM lanes 32*(w%4).. (rows) and
// accumulator columns 128*(w/4).. in the epilogue; thread 0 also issues the
// weight copies and the MMAs.  Per layer:
//   thread 0: wait for each weight K-block, 4 MMAs (K = 16) per K-block,
//             commit to `done`;
//   all:      wait `done`; thread 0 starts copying the next layer's weights
//             (the slots are free once the MMAs completed), which overlaps
//             the epilogue; epilogue from TMEM into the next A operand.
// Every wait is bounded; a timeout anywhere ends the CTA's loop uniformly
// (the decision is a block-wide OR), drains what it started and frees TMEM.
__global__ void __launch_bounds__(THREADS, 1) mlp_infer_kernel(InferArgs A) {
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t s_full[4];
    __shared__ uint64_t s_done;
    __shared__ uint32_t s_tmem;
    __shared__ float s_part[128];
    unsigned char* smem = reinterpret_cast<unsigned char*>(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    unsigned char* sA = smem;
    const uint32_t sB = smem_u32(smem + SMEM_A);
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const uint32_t full0 = smem_u32(&s_full[0]), done = smem_u32(&s_done);
    const uint64_t ntiles = (A.n + 127) / 128;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;\n" ::"r"(smem_u32(&s_tmem)));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
    if (tid == 0) {
        for (int i = 0; i < 4; ++i) mbar_init(full0 + 8 * i, 1);
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
        if ((uint64_t)blockIdx.x < ntiles) load_layer(A, 0, sB, full0);
    }
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = s_tmem;
    uint32_t full_phase = 0;   // thread 0: parity per slot
    uint32_t pending = 0;      // thread 0: slots with a copy not yet waited on
    if (tid == 0 && (uint64_t)blockIdx.x < ntiles) pending = (1u << KB0) - 1u;
    uint32_t done_phase = 0;
    bool aborted = false;
    const int row = tid & 127, half = tid >> 7;  // features: point row, 64-feature half
    const int erow = 32 * (warp & 3) + lane, ecol0 = 128 * (warp >> 2);  // epilogue
    for (uint64_t tile = blockIdx.x; tile < ntiles && !aborted; tile += gridDim.x) {
        const uint64_t pidx = tile * 128 + row;
        float q[3] = {0.0f, 0.0f, 0.0f};
        if (pidx < A.n) point_of(A, pidx, q);
        // Fourier features k in [64*half, 64*half + 64) of row `row` (96..127 zero)
        for (int k0 = 64 * half; k0 < 64 * half + 64; k0 += 8) {
            uint32_t packed[4] = {0u, 0u, 0u, 0u};
            if (k0 < FF) {
                const int a = k0 / 32;
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int j = (k0 % 32) / 2 + i;
                    float s, c;
                    sincos_reduced(ffreq(j) * q[a], &s, &c);
                    __nv_bfloat162 h = __floats2bfloat162_rn(s, c);
                    packed[i] = *reinterpret_cast<uint32_t*>(&h);
                }
            }
            *reinterpret_cast<uint4*>(sA + swz(row, k0, 128)) = make_uint4(packed[0], packed[1], packed[2], packed[3]);
        }
        float y = 0.0f;
        for (int l = 0; l < NLAYERS; ++l) {
            asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
            __syncthreads();
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            bool ok = true;
            if (tid == 0) {
                for (int kb = 0; kb < kblocks_of(l) && ok; ++kb) {
                    ok = mbar_wait(full0 + 8 * kb, (full_phase >> kb) & 1u);
                    if (!ok) break;
                    full_phase ^= 1u << kb;
                    pending &= ~(1u << kb);
                    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
                    for (int s = 0; s < 4; ++s) {
                        const uint64_t ad = sdesc(smem_u32(sA + kb * KBLOCK_BYTES_A + s * 32));
                        const uint64_t bd = sdesc(sB + kb * (uint32_t)KBLOCK_BYTES_B + s * 32);
                        mma(tmem, ad, bd, (kb | s) ? 1u : 0u);
                    }
                }
                // commit even after a failed wait: `done` then tracks the MMAs issued so far
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                                 done)
                             : "memory");
            }
            const bool ok_done = mbar_wait(done, done_phase);
            done_phase ^= 1;
            if (__syncthreads_or(!(ok && ok_done))) {
                if (tid == 0) atomicOr(A.err, DERR_QUEUE_TIMEOUT);
                if (!ok_done) mbar_wait(done, done_phase ^ 1);  // bounded: let issued MMAs drain
                aborted = true;
                break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            // the slots are free: copy the next layer's weights during the epilogue
            if (tid == 0) {
                const bool more = l + 1 < NLAYERS || tile + gridDim.x < ntiles;
                if (more) {
                    const int nl = (l + 1) % NLAYERS;
                    load_layer(A, nl, sB, full0);
                    pending |= (1u << kblocks_of(nl)) - 1u;
                }
            }
            // epilogue: row erow, columns [ecol0, ecol0 + 128), 16 at a time;
            // the TMEM load of the next 16 overlaps the arithmetic on these
            const float* bias = A.bias + l * HID;
            const uint32_t taddr = tmem + ((uint32_t)(32 * (warp & 3)) << 16);
            uint32_t ra[16], rb[16];
            uint64_t acc = f2(0.0f, 0.0f);
            tmem_ld16(taddr + ecol0, ra);
            tmem_wait(ra);
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                uint32_t(&cur)[16] = (c & 1) ? rb : ra;
                uint32_t(&nxt)[16] = (c & 1) ? ra : rb;
                const int c0 = ecol0 + 16 * c;
                if (c + 1 < 8) tmem_ld16(taddr + c0 + 16, nxt);
                uint64_t r[8];
#pragma unroll
                for (int i = 0; i < 8; ++i) {
                    const float2 bb = __ldg(reinterpret_cast<const float2*>(bias + c0) + i);
                    r[i] = softplus2(f2(__uint_as_float(cur[2 * i]), __uint_as_float(cur[2 * i + 1])), f2(bb.x, bb.y));
                }
                if (l + 1 < NLAYERS) {
                    uint32_t p[8];
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        float a0, a1;
                        uf2(r[i], a0, a1);
                        __nv_bfloat162 h = __floats2bfloat162_rn(a0, a1);
                        p[i] = *reinterpret_cast<uint32_t*>(&h);
                    }
                    *reinterpret_cast<uint4*>(sA + swz(erow, c0, 128)) = make_uint4(p[0], p[1], p[2], p[3]);
                    *reinterpret_cast<uint4*>(sA + swz(erow, c0 + 8, 128)) = make_uint4(p[4], p[5], p[6], p[7]);
                } else {
#pragma unroll
                    for (int i = 0; i < 8; ++i) {
                        const float2 ww = __ldg(reinterpret_cast<const float2*>(A.wout + c0) + i);
                        acc = fma2(r[i], f2(ww.x, ww.y), acc);
                    }
                }
                if (c + 1 < 8) tmem_wait(nxt);
            }
            if (l + 1 == NLAYERS) {
                float a0, a1;
                uf2(acc, a0, a1);
                y = a0 + a1;
            }
        }
        if (aborted) break;
        // output: the two column halves of each row
        if (ecol0) s_part[erow] = y;
        __syncthreads();
        if (!ecol0) {
            const uint64_t o = tile * 128 + erow;
            if (o < A.n) A.out[o] = y + s_part[erow] + __ldg(A.wout + HID);
        }
    }
    if (tid == 0) {  // bounded drain of copies started and not consumed (after an abort)
        for (int kb = 0; kb < 4; ++kb)
            if ((pending >> kb) & 1u) mbar_wait(full0 + 8 * kb, (full_phase >> kb) & 1u);
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
    MlpImages* m = nullptr;
    iso_status s = ready(net, &m);
    if (s != ISO_OK) return s;
    InferArgs a{};
    a.w = reinterpret_cast<const unsigned char*>(m->w);
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
        mlp_infer_kernel<<<blocks, THREADS, SMEM_TOTAL, ctx->stream>>>(a);
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
