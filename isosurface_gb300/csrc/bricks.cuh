// Culled sampling in the library: the device code of bricks_core.cuh with
// the library's program evaluator (vm.cuh), and the launch helpers.  The
// same core also runs with a per-program compiled evaluator (jit.cu).
#pragma once
#include <cuda_runtime.h>

#include <atomic>

#include "internal.h"
#include "vm.cuh"
#include "bricks_core.cuh"

namespace iso {

static_assert(BRICK_ERR_CAPACITY == DERR_CAPACITY, "the core's capacity bit is the library's");

// The interpreted evaluator: the program's ops, or its flat list of
// translated primitives (pruned per sub-brick when there are at most 64).
struct VmEval {
    ProgView pv;
    __device__ __forceinline__ float value(V3 p) const { return eval_scalar(pv, p); }
    __device__ __forceinline__ bool prunable() const { return pv.prims != nullptr && pv.nprims <= BRICK_PRUNE_MAX; }
    __device__ __forceinline__ uint32_t nprims() const { return pv.nprims; }
    __device__ __forceinline__ V3 point(V3 p) const { return prims_point(pv, p); }
    __device__ __forceinline__ float prim(uint32_t i, V3 q) const { return prim_at(pv, i, q); }
    __device__ __forceinline__ float value_kept(uint64_t keep, V3 p) const { return eval_prims_kept(pv, keep, p); }
};

// The culling bounds of a program for a lattice.
inline BrickLattice brick_lattice(const iso_program* prog, uint32_t nx, uint32_t ny, uint32_t nz, float inv,
                                  float* field, uint64_t pitch, uint32_t* bits, uint32_t W, uint32_t zoff,
                                  float reach_steps) {
    return BrickLattice{prog->lip, prog->slack, nx, ny, nz, inv, field, pitch, bits, W, zoff, reach_steps};
}

template <class Tiles>
__global__ void __launch_bounds__(256) brick_classify(VmEval ev, Tiles tiles, BrickTask* list, uint32_t* count,
                                                      uint32_t cap, uint32_t* err) {
    brick_classify_body(ev, tiles, list, count, cap, err);
}

template <class Tiles>
__global__ void __launch_bounds__(256) brick_rows(VmEval ev, Tiles tiles, const BrickTask* list,
                                                  const uint32_t* count, uint32_t cap) {
    brick_rows_body(ev, tiles, list, count, cap);
}

// Blocks of a persistent kernel that fill every SM (its occupancy at 256
// threads, looked up once per process and kernel).
inline unsigned persistent_blocks(const void* kernel, std::atomic<int>& per_sm, int sms) {
    int b = per_sm.load(std::memory_order_relaxed);
    if (b == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, 256, 0) != cudaSuccess || b < 1) {
            cudaGetLastError();
            b = 4;
        }
        per_sm.store(b, std::memory_order_relaxed);
    }
    return (unsigned)(b * (sms > 0 ? sms : 1));
}

// jit.cu: the culled sampler over one lattice with the program's compiled
// evaluator; false (nothing launched) when the program has none
bool jit_sample_bricks(iso_ctx* ctx, const iso_program* prog, const GridTiles& tiles, uint32_t ntiles,
                       BrickTask* list, uint32_t* count, uint32_t cap, cudaError_t* err);

// jit.cu: the full field of one lattice (blocks of eight field_warp warps)
// with the program's compiled evaluator; false (nothing launched) when the
// program has none
bool jit_sample_field(iso_ctx* ctx, const iso_program* prog, const BrickLattice& g, uint64_t blocks,
                      cudaError_t* err);

template <class Tiles>
inline unsigned brick_rows_blocks(int sms) {
    static std::atomic<int> per_sm{0};
    return persistent_blocks((const void*)brick_rows<Tiles>, per_sm, sms);
}

}  // namespace iso
