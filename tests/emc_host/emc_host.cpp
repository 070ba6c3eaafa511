// Host build of the library's ExtendedMarchingCubes passes
// (isosurface_gb300/csrc/emc.cuh): the same per-item functions the CUDA
// kernels of emc.cu run, here run one item at a time on the CPU in the
// kernels' pass order, with host copies of the tables and a serial
// exclusive scan in place of scan_u32.  Test infrastructure: tests/ build and
// load it to check the library's own arithmetic, ownership, ordering and
// flips against the oracle on machines without a GPU.  Built by g++ as
// plain C++ (the CUDA keywords expand to nothing) with -ffp-contract=off,
// as the library's units are built with -fmad=false.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

// nvcc's keyword for what gcc spells as an attribute; defined only after the
// system headers, which use the attribute's own name
#ifndef __noinline__
#define __noinline__ __attribute__((noinline))
#endif

#define ISO_TABLE static const
#include "emc_tables.h"
#include "mc_tables.h"

#include "emc.cuh"

using namespace iso;

namespace {

struct HostProgram {
    std::vector<uint32_t> ops;
    std::vector<float> consts;
    std::vector<int32_t> jump;
    ProgView view() const { return ProgView{ops.data(), consts.data(), jump.data(), (uint32_t)ops.size(), nullptr, 0, -1}; }
};

// the program's ops, constants (padded as the library pads them) and CD jump table
bool parse(const uint8_t* bytes, size_t len, HostProgram* p) {
    uint32_t h[4];
    if (len < 16) return false;
    std::memcpy(h, bytes, 16);
    if (h[0] != 0x314F5349u || 16 + 4ull * h[1] + 4ull * h[2] != len) return false;
    p->ops.assign(h[1], 0);
    p->consts.assign(h[2] + 4, 0.0f);
    std::memcpy(p->ops.data(), bytes + 16, 4ull * h[1]);
    if (h[2]) std::memcpy(p->consts.data(), bytes + 16 + 4ull * h[1], 4ull * h[2]);
    // CD_BEGIN -> its CD_END (scopes do not nest)
    p->jump.assign(p->ops.size(), 0);
    for (size_t pc = 0; pc < p->ops.size(); ++pc)
        if ((p->ops[pc] & 0xFF) == OP_CD_BEGIN)
            for (size_t e = pc + 1; e < p->ops.size(); ++e)
                if ((p->ops[e] & 0xFF) == OP_CD_END) {
                    p->jump[pc] = (int32_t)e;
                    break;
                }
    return true;
}

}  // namespace

extern "C" {

// The device's Directed evaluator (emc::eval_vector) at n points, 3 floats each.
int emc_host_sample_vector(const uint8_t* bytes, size_t len, const float* pts, uint64_t n, float* out) {
    HostProgram p;
    if (!parse(bytes, len, &p)) return 2;
    const ProgView pv = p.view();
    for (uint64_t i = 0; i < n; ++i) {
        const V3 v = emc::eval_vector(pv, v3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
        out[3 * i] = v.x;
        out[3 * i + 1] = v.y;
        out[3 * i + 2] = v.z;
    }
    return 0;
}

// counts: vertices, triangles, flips, device error bits.  Returns 0, or 1
// when the output capacities are too small (counts still filled), or 2 for
// a malformed program.
int emc_host_extract(const uint8_t* bytes, size_t len, uint32_t size, float* vout, uint64_t vcap, uint32_t* iout,
                     uint64_t icap, uint64_t* counts) {
    HostProgram prog;
    if (!parse(bytes, len, &prog)) return 2;
    counts[0] = counts[1] = counts[2] = counts[3] = 0;
    if (size < 2) return 0;
    const uint32_t n = size;
    const uint64_t points = emc::num_points(n), cells = emc::num_cells(n);
    std::vector<float4> field(points);
    std::vector<uint16_t> cell(cells);
    std::vector<uint32_t> voff(cells), toff(cells), edge_map(3 * points, 0xFFFFFFFFu);
    uint32_t err = 0;
    emc::Args A{};
    A.prog = prog.view();
    A.g = emc::Grid{n, 1.0f / (float)(n - 1)};
    A.field = field.data();
    A.cell = cell.data();
    A.voff = voff.data();
    A.toff = toff.data();
    A.edge_map = edge_map.data();
    A.err = &err;
    for (uint64_t i = 0; i < points; ++i) emc::sample_item(A, i);
    for (uint64_t c = 0; c < cells; ++c) emc::count_item(A, c);
    uint64_t nv = 0, nt = 0;
    for (uint64_t c = 0; c < cells; ++c) {
        const uint32_t a = voff[c], b = toff[c];
        voff[c] = (uint32_t)nv;
        toff[c] = (uint32_t)nt;
        nv += a;
        nt += b;
    }
    std::vector<float> verts(3 * nv + 3);
    std::vector<uint32_t> idx(3 * nt + 3);
    A.vertices = verts.data();
    A.indices = idx.data();
    A.cap_v = nv;
    A.cap_t = nt;
    for (uint64_t c = 0; c < cells; ++c) emc::vertex_item(A, c);
    for (uint64_t c = 0; c < cells; ++c) emc::triangle_item(A, c);
    uint64_t flips = 0;
    for (uint64_t c = 0; c < cells; ++c) flips += emc::flip_item(A, c);
    counts[0] = nv;
    counts[1] = nt;
    counts[2] = flips;
    counts[3] = err;
    if (nv > vcap || nt > icap) return 1;
    if (nv) std::memcpy(vout, verts.data(), 12 * nv);
    if (nt) std::memcpy(iout, idx.data(), 12 * nt);
    return 0;
}

}  // extern "C"
