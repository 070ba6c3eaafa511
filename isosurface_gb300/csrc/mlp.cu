// Learned SDF surrogate: a Fourier-feature MLP trained on the GPU by this
// file's own kernels (forward, backward, Adam), with no library GEMM.
//
// Network (no counterpart in the reference; it stands in for an expensive
// many-primitive Source):
//   x (3, the source's world coordinates)
//   -> Fourier features, 16 frequencies per axis: sin(w_j x_a), cos(w_j x_a),
//      w_j = pi * 2^(7 j / 15), feature a*32 + 2j (+1 for cos)        96
//   -> 6 hidden layers of 256, softplus_beta(z) = log(1 + exp(beta z)) / beta
//      with beta = 100 (computed as max(z,0) + log1p(exp(-beta |z|)) / beta)
//   -> linear output (signed distance)                                  1
// Parameters (fp32 master copy, this order): W0[256][96], b0[256],
// W1..W5[256][256], b1..b5[256], w_out[256], b_out.
//
// Training data: points drawn uniformly in the domain box, kept with
// probability 1 near the surface (|f| < 0.05) and 0.25 elsewhere, labelled by
// the exact program (the same evaluator as the grid sampler).  Loss: L1
// against the target truncated to [-d, d] (one-sided where it saturates,
// see loss_l1), d = 0.1 by default.  Optimiser: Adam.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "internal.h"
#include "mlp.h"
#include "vm.cuh"

namespace iso {
namespace mlp {

// ---------------------------------------------------------------- helpers ---
__host__ __device__ __forceinline__ uint64_t splitmix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__host__ __device__ __forceinline__ float unit_float(uint64_t h) { return (float)(h >> 40) * (1.0f / 16777216.0f); }

__device__ __forceinline__ float softplus(float z) {
    return fmaxf(z, 0.0f) + log1pf(expf(-BETA * fabsf(z))) * (1.0f / BETA);
}
// d softplus_beta / dz = sigmoid(beta z)
__device__ __forceinline__ float sigmoid(float z) { return 1.0f / (1.0f + expf(-BETA * z)); }

__host__ __device__ __forceinline__ float freq(int j) { return 3.14159265358979f * exp2f((float)(7 * j) / 15.0f); }

// ------------------------------------------------------------ fp32 GEMM ---
// C[M x N] (ldc) (+)= op(A)[M x K] * op(B)[K x N], element (i,k) of op(A) at
// A[i*sa0 + k*sa1], element (k,j) of op(B) at B[k*sb0 + j*sb1].  64x64 tiles,
// 256 threads, 4x4 per thread.  Split-K over gridDim.z accumulates with
// atomicAdd (accumulate must be set then).  bias (nullable) is added per column
// by the z == 0 slice.
constexpr int TM = 64, TN = 64, TK = 16;

__global__ void __launch_bounds__(256) sgemm(int M, int N, int K, const float* __restrict__ A, int64_t sa0,
                                             int64_t sa1, const float* __restrict__ B, int64_t sb0, int64_t sb1,
                                             float* __restrict__ C, int64_t ldc, const float* __restrict__ bias,
                                             int accumulate) {
    __shared__ float As[TK][TM + 4];
    __shared__ float Bs[TK][TN + 4];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int i0 = blockIdx.y * TM, j0 = blockIdx.x * TN;
    const int kslices = gridDim.z;
    const int kper = ((K + kslices - 1) / kslices + TK - 1) / TK * TK;
    const int kbeg = blockIdx.z * kper, kend = min(K, kbeg + kper);
    float acc[4][4] = {};
    for (int k0 = kbeg; k0 < kend; k0 += TK) {
        for (int t = threadIdx.x; t < TK * TM; t += 256) {
            const int kk = t / TM, ii = t % TM;
            const int gi = i0 + ii, gk = k0 + kk;
            As[kk][ii] = (gi < M && gk < kend) ? A[(int64_t)gi * sa0 + (int64_t)gk * sa1] : 0.0f;
        }
        for (int t = threadIdx.x; t < TK * TN; t += 256) {
            const int kk = t / TN, jj = t % TN;
            const int gj = j0 + jj, gk = k0 + kk;
            Bs[kk][jj] = (gj < N && gk < kend) ? B[(int64_t)gk * sb0 + (int64_t)gj * sb1] : 0.0f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) a[r] = As[kk][ty * 4 + r];
#pragma unroll
            for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx * 4 + c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(a[r], b[c], acc[r][c]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int gi = i0 + ty * 4 + r;
        if (gi >= M) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int gj = j0 + tx * 4 + c;
            if (gj >= N) continue;
            float v = acc[r][c];
            if (bias && blockIdx.z == 0) v += bias[gj];
            float* dst = C + (int64_t)gi * ldc + gj;
            if (accumulate) atomicAdd(dst, v);
            else *dst = v;
        }
    }
}

void gemm(cudaStream_t s, int M, int N, int K, const float* A, int64_t sa0, int64_t sa1, const float* B, int64_t sb0,
          int64_t sb1, float* C, int64_t ldc, const float* bias, bool accumulate, int ksplit = 1) {
    dim3 grid((N + TN - 1) / TN, (M + TM - 1) / TM, ksplit);
    sgemm<<<grid, 256, 0, s>>>(M, N, K, A, sa0, sa1, B, sb0, sb1, C, ldc, bias, accumulate ? 1 : 0);
}

// ------------------------------------------------------- elementwise kernels ---
__global__ void fourier(const float* pts, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * FF) return;
    const uint32_t p = i / FF, f = i % FF;
    const uint32_t a = f / 32, j = (f % 32) / 2;
    const float x = freq(j) * pts[3 * p + a];
    out[i] = (f & 1) ? cosf(x) : sinf(x);
}

__global__ void act_softplus(const float* z, float* a, uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) a[i] = softplus(z[i]);
}

// dz = da * sigmoid(z), in place on da
__global__ void act_backward(const float* z, float* da, uint64_t n) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) da[i] *= sigmoid(z[i]);
}

// y[p] = a[p] . w + b; warp per point
__global__ void out_forward(const float* a, uint32_t n, const float* w, const float* b, float* y) {
    const uint32_t p = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x & 31;
    if (p >= n) return;
    float s = 0.0f;
    for (int k = lane; k < HID; k += 32) s += a[(size_t)p * HID + k] * w[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xFFFFFFFFu, s, o);
    if (lane == 0) y[p] = s + b[0];
}

// Truncated L1: e = y - t inside the band |t| < d; where the target is
// saturated (t >= d or t <= -d) only a prediction on the band's side of +-d
// is penalised (e = min(y - d, 0) or max(y + d, 0)).  loss = mean |e|,
// dy = sign(e) / n; the loss accumulates into *loss.
__global__ void loss_l1(const float* y, const float* t, uint32_t n, float clampd, float* dy, float* loss) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (i < n) {
        const float ti = t[i], yi = y[i];
        const float d = (ti >= clampd) ? fminf(yi - clampd, 0.0f) : (ti <= -clampd) ? fmaxf(yi + clampd, 0.0f) : yi - ti;
        l = fabsf(d);
        dy[i] = (d > 0.0f ? 1.0f : (d < 0.0f ? -1.0f : 0.0f)) / (float)n;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xFFFFFFFFu, l, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l / (float)n);
}

// da[p][k] = dy[p] * w[k]
__global__ void out_backward_act(const float* dy, const float* w, uint32_t n, float* da) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < (uint64_t)n * HID) da[i] = dy[i / HID] * w[i % HID];
}

// column sums: out[j] += sum_p m[p][j]  (block per 256 columns chunk of rows)
__global__ void colsum(const float* m, uint32_t n, uint32_t cols, float* out) {
    const uint32_t j = threadIdx.x;
    if (j >= cols) return;
    const uint32_t rows_per = (n + gridDim.x - 1) / gridDim.x;
    const uint32_t r0 = blockIdx.x * rows_per, r1 = min(n, r0 + rows_per);
    float s = 0.0f;
    for (uint32_t r = r0; r < r1; ++r) s += m[(size_t)r * cols + j];
    atomicAdd(out + j, s);
}

__global__ void adam(float* p, const float* g, float* m, float* v, uint64_t n, float lr, float b1, float b2,
                     float eps, float c1, float c2) {
    const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

// ------------------------------------------------------------- dataset ---
struct SampleArgs {
    ProgView pv;
    uint64_t seed;
    uint64_t base;     // candidate counter offset
    uint32_t ncand;
    float lo, hi;      // world box
    float near, far_keep;
    float* pts;        // world coordinates
    float* labels;
    uint32_t* count;
    uint32_t cap;
};

__global__ void make_samples(SampleArgs A) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.ncand) return;
    const uint64_t id = A.base + i;
    const float x = A.lo + (A.hi - A.lo) * unit_float(splitmix(A.seed ^ (3 * id)));
    const float y = A.lo + (A.hi - A.lo) * unit_float(splitmix(A.seed ^ (3 * id + 1)));
    const float z = A.lo + (A.hi - A.lo) * unit_float(splitmix(A.seed ^ (3 * id + 2)));
    const float f = eval_scalar(A.pv, v3(x, y, z));
    const float u = unit_float(splitmix(A.seed * 31 + id));
    if (!(fabsf(f) < A.near || u < A.far_keep)) return;
    const uint32_t at = atomicAdd(A.count, 1u);
    if (at >= A.cap) return;
    A.pts[3 * at] = x;
    A.pts[3 * at + 1] = y;
    A.pts[3 * at + 2] = z;
    A.labels[at] = f;
}

__global__ void gather_batch(const float* pts, const float* labels, uint32_t n, uint64_t seed, uint32_t b,
                             float* bp, float* bl) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= b) return;
    const uint32_t k = (uint32_t)(splitmix(seed + i) % n);
    bp[3 * i] = pts[3 * k];
    bp[3 * i + 1] = pts[3 * k + 1];
    bp[3 * i + 2] = pts[3 * k + 2];
    bl[i] = labels[k];
}

}  // namespace mlp
}  // namespace iso

using namespace iso;
using namespace iso::mlp;


namespace {

struct Views {
    float *pts, *ff, *z[NLAYERS], *a[NLAYERS], *y, *t, *dy, *da, *db_scratch, *loss;
};

iso_status ensure_work(iso_mlp* net, uint32_t n) {
    if (n <= net->cap && net->work) return ISO_OK;
    if (net->work) cudaFree(net->work);
    net->work = nullptr;
    const size_t floats = (size_t)n * (3 + FF + 2 * NLAYERS * HID + 3 + 2 * HID) + 1024;
    cudaError_t e = cudaMalloc(&net->work, floats * 4);
    if (e != cudaSuccess) return cuda_fail(net->ctx, e, "mlp work");
    net->work_bytes = floats * 4;
    net->cap = n;
    return ISO_OK;
}

Views views(iso_mlp* net) {
    Views w;
    float* p = net->work;
    const size_t n = net->cap;
    w.pts = p; p += 3 * n;
    w.ff = p; p += FF * n;
    for (int l = 0; l < NLAYERS; ++l) { w.z[l] = p; p += HID * n; }
    for (int l = 0; l < NLAYERS; ++l) { w.a[l] = p; p += HID * n; }
    w.y = p; p += n;
    w.t = p; p += n;
    w.dy = p; p += n;
    w.da = p; p += HID * n;
    w.db_scratch = p; p += HID * n;
    w.loss = p;
    return w;
}

inline unsigned blocks(uint64_t n, unsigned t) { return (unsigned)((n + t - 1) / t); }

// forward over w.pts[0..n) into w.y; keeps z/a for backward
void forward(iso_mlp* net, const Views& w, uint32_t n) {
    cudaStream_t s = net->ctx->stream;
    const float* P = net->params;
    fourier<<<blocks((uint64_t)n * FF, 256), 256, 0, s>>>(w.pts, n, w.ff);
    const float* in = w.ff;
    int in_dim = FF;
    for (int l = 0; l < NLAYERS; ++l) {
        const float* W = P + weight_offset(l);
        const float* b = P + bias_offset(l);
        // z = in [n x in_dim] * W^T [in_dim x HID] + b
        gemm(s, n, HID, in_dim, in, in_dim, 1, W, 1, in_dim, w.z[l], HID, b, false);
        act_softplus<<<blocks((uint64_t)n * HID, 256), 256, 0, s>>>(w.z[l], w.a[l], (uint64_t)n * HID);
        in = w.a[l];
        in_dim = HID;
    }
    out_forward<<<blocks(n, 8), 256, 0, s>>>(w.a[NLAYERS - 1], n, P + OUT_W, P + OUT_B, w.y);
    net->ctx->launches += 2 + 2 * NLAYERS;
}

// grads (zeroed first) of the loss over n points with targets w.t; *loss
void backward(iso_mlp* net, const Views& w, uint32_t n, float clampd) {
    cudaStream_t s = net->ctx->stream;
    const float* P = net->params;
    float* G = net->grads;
    cudaMemsetAsync(G, 0, NPARAMS * 4, s);
    cudaMemsetAsync(w.loss, 0, 4, s);
    loss_l1<<<blocks(n, 256), 256, 0, s>>>(w.y, w.t, n, clampd, w.dy, w.loss);
    // output layer
    gemm(s, 1, HID, n, w.dy, 1, 1, w.a[NLAYERS - 1], HID, 1, G + OUT_W, HID, nullptr, true, 64);
    colsum<<<64, 32, 0, s>>>(w.dy, n, 1, G + OUT_B);
    out_backward_act<<<blocks((uint64_t)n * HID, 256), 256, 0, s>>>(w.dy, P + OUT_W, n, w.da);
    for (int l = NLAYERS - 1; l >= 0; --l) {
        act_backward<<<blocks((uint64_t)n * HID, 256), 256, 0, s>>>(w.z[l], w.da, (uint64_t)n * HID);
        const float* in = l ? w.a[l - 1] : w.ff;
        const int in_dim = l ? HID : FF;
        // dW = dz^T [HID x n] * in [n x in_dim]
        gemm(s, HID, in_dim, n, w.da, 1, HID, in, in_dim, 1, G + weight_offset(l), in_dim, nullptr, true, 64);
        colsum<<<64, HID, 0, s>>>(w.da, n, HID, G + bias_offset(l));
        if (l > 0) {
            // d in = dz [n x HID] * W [HID x in_dim]
            gemm(s, n, in_dim, HID, w.da, HID, 1, P + weight_offset(l), in_dim, 1, w.db_scratch, in_dim, nullptr,
                 false);
            cudaMemcpyAsync(w.da, w.db_scratch, (size_t)n * in_dim * 4, cudaMemcpyDeviceToDevice, s);
        }
    }
    net->ctx->launches += 4 + 5 * NLAYERS;
}

}  // namespace

extern "C" {

iso_status iso_mlp_create(iso_ctx* ctx, uint64_t seed, iso_mlp** out) {
    if (!ctx || !out) return ISO_ERR_INVALID_ARG;
    *out = nullptr;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    iso_mlp* net = new iso_mlp();
    net->ctx = ctx;
    cudaError_t e = cudaMalloc(&net->params, 4ull * NPARAMS * 4);
    if (e != cudaSuccess) {
        delete net;
        return cuda_fail(ctx, e, "mlp params");
    }
    net->grads = net->params + NPARAMS;
    net->m = net->grads + NPARAMS;
    net->v = net->m + NPARAMS;
    // uniform(-a, a) with a = sqrt(6 / (fan_in + fan_out)); biases zero
    std::vector<float> h(NPARAMS, 0.0f);
    for (int l = 0; l <= NLAYERS; ++l) {
        const int fin = l == 0 ? FF : HID, fout = l == NLAYERS ? 1 : HID;
        const float a = std::sqrt(6.0f / (float)(fin + fout));
        const size_t off = l == NLAYERS ? OUT_W : weight_offset(l);
        for (size_t k = 0; k < (size_t)fin * fout; ++k)
            h[off + k] = a * (2.0f * unit_float(splitmix(seed * 1000003ull + off + k)) - 1.0f);
    }
    e = cudaMemcpy(net->params, h.data(), 4ull * NPARAMS, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(net->m, 0, 8ull * NPARAMS);
    if (e != cudaSuccess) {
        iso_mlp_destroy(net);
        return cuda_fail(ctx, e, "mlp init");
    }
    *out = net;
    return ISO_OK;
}

iso_status iso_mlp_destroy(iso_mlp* net) {
    if (!net) return ISO_ERR_INVALID_ARG;
    cudaSetDevice(net->ctx->device);
    if (net->params) cudaFree(net->params);
    if (net->work) cudaFree(net->work);
    if (net->data_pts) cudaFree(net->data_pts);
    mlp_infer_release(net);
    delete net;
    return ISO_OK;
}

uint64_t iso_mlp_num_params(void) { return NPARAMS; }

iso_status iso_mlp_get_params(iso_mlp* net, float* host) {
    if (!net || !host) return ISO_ERR_INVALID_ARG;
    cudaError_t e = cudaMemcpy(host, net->params, 4ull * NPARAMS, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? ISO_OK : cuda_fail(net->ctx, e, "get params");
}

iso_status iso_mlp_set_params(iso_mlp* net, const float* host) {
    if (!net || !host) return ISO_ERR_INVALID_ARG;
    cudaError_t e = cudaMemcpy(net->params, host, 4ull * NPARAMS, cudaMemcpyHostToDevice);
    mlp_infer_invalidate(net);
    return e == cudaSuccess ? ISO_OK : cuda_fail(net->ctx, e, "set params");
}

// fp32 forward of n host points (world coordinates) into host values
iso_status iso_mlp_forward(iso_mlp* net, const float* pts, uint32_t n, float* values) {
    if (!net || (!pts && n) || (!values && n)) return ISO_ERR_INVALID_ARG;
    if (n == 0) return ISO_OK;
    iso_status s = set_device(net->ctx);
    if (s != ISO_OK || (s = ensure_work(net, n)) != ISO_OK) return s;
    Views w = views(net);
    cudaStream_t st = net->ctx->stream;
    cudaMemcpyAsync(w.pts, pts, 12ull * n, cudaMemcpyHostToDevice, st);
    {
        StageTimer timer(net->ctx, ISO_STAGE_MLP);
        forward(net, w, n);
    }
    cudaMemcpyAsync(values, w.y, 4ull * n, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? check_launch(net->ctx, "mlp forward") : cuda_fail(net->ctx, e, "mlp forward");
}

// loss and gradient of the training loss over given points/targets (host)
iso_status iso_mlp_loss_grad(iso_mlp* net, const float* pts, const float* targets, uint32_t n, float clampd,
                             float* loss, float* grad_host) {
    if (!net || !pts || !targets || n == 0) return ISO_ERR_INVALID_ARG;
    iso_status s = set_device(net->ctx);
    if (s != ISO_OK || (s = ensure_work(net, n)) != ISO_OK) return s;
    Views w = views(net);
    cudaStream_t st = net->ctx->stream;
    cudaMemcpyAsync(w.pts, pts, 12ull * n, cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(w.t, targets, 4ull * n, cudaMemcpyHostToDevice, st);
    forward(net, w, n);
    backward(net, w, n, clampd);
    if (loss) cudaMemcpyAsync(loss, w.loss, 4, cudaMemcpyDeviceToHost, st);
    if (grad_host) cudaMemcpyAsync(grad_host, net->grads, 4ull * NPARAMS, cudaMemcpyDeviceToHost, st);
    cudaError_t e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? check_launch(net->ctx, "mlp loss/grad") : cuda_fail(net->ctx, e, "mlp loss/grad");
}

// draw n samples in [lo, hi]^3 labelled by `exact` (see file comment)
iso_status iso_mlp_make_dataset(iso_mlp* net, const iso_program* exact, uint32_t n, float lo, float hi,
                                uint64_t seed) {
    iso::NvtxRange nvtx_range("iso_mlp_make_dataset");
    if (!net || !exact || n == 0) return ISO_ERR_INVALID_ARG;
    iso_status s = set_device(net->ctx);
    if (s != ISO_OK) return s;
    if (net->data_pts) cudaFree(net->data_pts);
    net->data_pts = nullptr;
    cudaError_t e = cudaMalloc(&net->data_pts, 16ull * n + 256);
    if (e != cudaSuccess) return cuda_fail(net->ctx, e, "dataset");
    net->data_labels = net->data_pts + 3ull * n;
    uint32_t* count = (uint32_t*)(net->data_labels + n);
    cudaStream_t st = net->ctx->stream;
    cudaMemsetAsync(count, 0, 4, st);
    uint64_t base = 0;
    uint32_t have = 0;
    for (int round = 0; round < 64 && have < n; ++round) {
        const uint32_t cand = std::max<uint32_t>(n, 1u << 20);
        SampleArgs a{exact->view(), seed, base, cand, lo, hi, 0.05f, 0.25f, net->data_pts, net->data_labels, count, n};
        {
            StageTimer timer(net->ctx, ISO_STAGE_MLP);
            make_samples<<<blocks(cand, 128), 128, 0, st>>>(a);
        }
        net->ctx->launches++;
        base += cand;
        e = cudaMemcpyAsync(&have, count, 4, cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) return cuda_fail(net->ctx, e, "dataset");
    }
    net->data_n = std::min(have, n);
    return net->data_n == n ? ISO_OK : fail(net->ctx, ISO_ERR_CAPACITY, "dataset rounds exhausted");
}

// steps of Adam on random batches of the dataset; loss per step into history (nullable)
iso_status iso_mlp_train(iso_mlp* net, uint32_t steps, uint32_t batch, float lr, float clampd, uint64_t seed,
                         float* history) {
    iso::NvtxRange nvtx_range("iso_mlp_train");
    if (!net || batch == 0 || net->data_n == 0) return ISO_ERR_INVALID_ARG;
    iso_status s = set_device(net->ctx);
    if (s != ISO_OK || (s = ensure_work(net, batch)) != ISO_OK) return s;
    Views w = views(net);
    cudaStream_t st = net->ctx->stream;
    std::vector<float> hist(steps, 0.0f);
    float* d_hist = nullptr;
    if (history) {
        cudaError_t e = cudaMalloc(&d_hist, 4ull * std::max<uint32_t>(steps, 1));
        if (e != cudaSuccess) return cuda_fail(net->ctx, e, "history");
    }
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (uint32_t k = 0; k < steps; ++k) {
        StageTimer timer(net->ctx, ISO_STAGE_MLP);
        gather_batch<<<blocks(batch, 256), 256, 0, st>>>(net->data_pts, net->data_labels, net->data_n,
                                                          splitmix(seed + 7919ull * (net->step + 1)), batch, w.pts, w.t);
        forward(net, w, batch);
        backward(net, w, batch, clampd);
        ++net->step;
        const float c1 = 1.0f - std::pow(b1, (float)net->step), c2 = 1.0f - std::pow(b2, (float)net->step);
        // cosine decay to 5% of lr over the call
        const float lr_k = lr * (0.05f + 0.95f * 0.5f * (1.0f + std::cos(3.14159265f * (float)k / (float)steps)));
        adam<<<blocks(NPARAMS, 256), 256, 0, st>>>(net->params, net->grads, net->m, net->v, NPARAMS, lr_k, b1, b2,
                                                    eps, c1, c2);
        if (d_hist) cudaMemcpyAsync(d_hist + k, w.loss, 4, cudaMemcpyDeviceToDevice, st);
        net->ctx->launches += 2;
    }
    mlp_infer_invalidate(net);
    cudaError_t e = cudaSuccess;
    if (d_hist) {
        e = cudaMemcpyAsync(history, d_hist, 4ull * steps, cudaMemcpyDeviceToHost, st);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (d_hist) cudaFree(d_hist);
    return e == cudaSuccess ? check_launch(net->ctx, "mlp train") : cuda_fail(net->ctx, e, "mlp train");
}

// ------------------------------------------------------------- checkpoints ---
// 32-byte header, then NPARAMS fp32 parameters, Adam's first and second
// moments; host byte order (little-endian on both supported machines).
namespace {
constexpr char CKPT_MAGIC[8] = {'I', 'S', 'O', 'M', 'L', 'P', '0', '1'};
struct CkptHeader {
    char magic[8];
    uint32_t version;       // 1
    uint32_t header_bytes;  // 32
    uint64_t nparams;
    uint64_t step;          // Adam steps taken
};
static_assert(sizeof(CkptHeader) == 32, "checkpoint header layout");

// 0 = ok, 1 = cannot open / short file, 2 = not a checkpoint of this network
int read_header(FILE* f, CkptHeader* h) {
    if (std::fread(h, sizeof(*h), 1, f) != 1) return 1;
    if (std::memcmp(h->magic, CKPT_MAGIC, 8) != 0 || h->version != 1 || h->header_bytes != sizeof(*h) ||
        h->nparams != NPARAMS)
        return 2;
    return 0;
}
}  // namespace

iso_status iso_mlp_checkpoint_info(const char* path, uint64_t* nparams, uint64_t* step) {
    if (!path) return ISO_ERR_INVALID_ARG;
    FILE* f = std::fopen(path, "rb");
    if (!f) return ISO_ERR_INVALID_ARG;
    CkptHeader h;
    const int r = read_header(f, &h);
    std::fseek(f, 0, SEEK_END);
    const long size = std::ftell(f);
    std::fclose(f);
    if (r != 0 || size != (long)(sizeof(h) + 12ull * NPARAMS)) return ISO_ERR_INVALID_ARG;
    if (nparams) *nparams = h.nparams;
    if (step) *step = h.step;
    return ISO_OK;
}

iso_status iso_mlp_save(iso_mlp* net, const char* path) {
    if (!net || !path) return ISO_ERR_INVALID_ARG;
    iso_status s = set_device(net->ctx);
    if (s != ISO_OK) return s;
    std::vector<float> host(3 * NPARAMS);
    cudaError_t e = cudaMemcpy(host.data(), net->params, 4ull * NPARAMS, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(host.data() + NPARAMS, net->m, 8ull * NPARAMS, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(net->ctx, e, "checkpoint read");
    CkptHeader h{};
    std::memcpy(h.magic, CKPT_MAGIC, 8);
    h.version = 1;
    h.header_bytes = sizeof(h);
    h.nparams = NPARAMS;
    h.step = net->step;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(net->ctx, ISO_ERR_INVALID_ARG, std::string("cannot write ") + path);
    const bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1 &&
                    std::fwrite(host.data(), 4, host.size(), f) == host.size();
    if (std::fclose(f) != 0 || !ok) return fail(net->ctx, ISO_ERR_INVALID_ARG, std::string("cannot write ") + path);
    return ISO_OK;
}

iso_status iso_mlp_load(iso_mlp* net, const char* path) {
    if (!net || !path) return ISO_ERR_INVALID_ARG;
    iso_status s = iso_mlp_checkpoint_info(path, nullptr, nullptr);
    if (s != ISO_OK) return fail(net->ctx, s, std::string("not a checkpoint of this network: ") + path);
    if ((s = set_device(net->ctx)) != ISO_OK) return s;
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(net->ctx, ISO_ERR_INVALID_ARG, std::string("cannot read ") + path);
    CkptHeader h;
    std::vector<float> host(3 * NPARAMS);
    const bool ok = read_header(f, &h) == 0 && std::fread(host.data(), 4, host.size(), f) == host.size();
    std::fclose(f);
    if (!ok) return fail(net->ctx, ISO_ERR_INVALID_ARG, std::string("cannot read ") + path);
    // parameters | gradients | first moments | second moments, one allocation
    cudaError_t e = cudaMemcpy(net->params, host.data(), 4ull * NPARAMS, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(net->m, host.data() + NPARAMS, 8ull * NPARAMS, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(net->ctx, e, "checkpoint load");
    net->step = h.step;
    mlp_infer_invalidate(net);
    return ISO_OK;
}

}  // extern "C"
