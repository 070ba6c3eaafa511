// Shape and parameter layout of the surrogate MLP (mlp.cu, mlp_infer.cu).
#pragma once
#include <cstddef>
#include <cstdint>

#include "../../include/isosurface_gpu.h"

#ifdef __CUDACC__
#define MLP_HD __host__ __device__
#else
#define MLP_HD
#endif

struct iso_mlp {
    iso_ctx* ctx = nullptr;
    float* params = nullptr;  // NPARAMS
    float* grads = nullptr;
    float* m = nullptr;
    float* v = nullptr;
    uint64_t step = 0;
    // activations for a batch of up to cap points
    uint32_t cap = 0;
    float* work = nullptr;
    size_t work_bytes = 0;
    // dataset
    float* data_pts = nullptr;
    float* data_labels = nullptr;
    uint32_t data_n = 0;
    // bf16 inference copy (mlp_infer.cu)
    void* infer = nullptr;
};

namespace iso {
namespace mlp {

constexpr int FF = 96;       // Fourier features: 3 axes x 16 frequencies x (sin, cos)
constexpr int HID = 256;     // hidden width
constexpr int NLAYERS = 6;   // hidden layers (each followed by softplus)
// softplus_beta(z) = log(1 + exp(beta z)) / beta: close to ReLU, smooth
constexpr float BETA = 100.0f;

// W0 [HID][FF], b0, W1..W5 [HID][HID], b1..b5, w_out [HID], b_out
MLP_HD constexpr size_t weight_offset(int l) {
    return l == 0 ? 0 : (size_t)HID * FF + HID + (size_t)(l - 1) * (HID * HID + HID);
}
MLP_HD constexpr size_t bias_offset(int l) { return weight_offset(l) + (size_t)HID * (l == 0 ? FF : HID); }
constexpr size_t OUT_W = weight_offset(NLAYERS);
constexpr size_t OUT_B = OUT_W + HID;
constexpr size_t NPARAMS = OUT_B + 1;

}  // namespace mlp

// mlp_infer.cu: the bf16 tensor-core copy of the parameters
void mlp_infer_release(iso_mlp* net);
void mlp_infer_invalidate(iso_mlp* net);
// A lattice of nx x ny x nz points (i, j, k) at p = (i, j, k) * step * inv,
// given to the network as q = p * scale + offset.
struct MlpGrid {
    uint32_t nx, ny, nz, step;
    float inv;
    float scale[3], offset[3];
};
// bf16 tcgen05 inference on the net's stream: n explicit device points
// (d_pts, xyz interleaved) into d_out[i], or, with d_pts null, every point of
// *grid into d_out[(k * ny + j) * nx + i]
iso_status mlp_infer_launch(iso_mlp* net, const float* d_pts, uint64_t n, const MlpGrid* grid, float* d_out);

}  // namespace iso
