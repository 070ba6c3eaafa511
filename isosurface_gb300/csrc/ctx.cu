// Contexts, programs, buffers and the C ABI entry points (include/isosurface_gpu.h).
#include <cuda_runtime.h>

#include <atomic>
#include <mutex>
#include <unordered_set>
#include <utility>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>

#include "internal.h"

namespace iso {

iso_status fail(iso_ctx* ctx, iso_status s, const std::string& msg) {
    if (ctx) ctx->last_error = msg;
    return s;
}

iso_status cuda_fail(iso_ctx* ctx, cudaError_t e, const char* what) {
    if (ctx) ctx->last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return (e == cudaErrorMemoryAllocation) ? ISO_ERR_OUT_OF_MEMORY : ISO_ERR_CUDA;
}

iso_status set_device(iso_ctx* ctx) {
    cudaError_t e = cudaSetDevice(ctx->device);
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, "cudaSetDevice");
}

iso_status fork_side(iso_ctx* ctx, cudaStream_t* side) {
    cudaError_t e = cudaSuccess;
    if (!ctx->side) {
        e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->side_fork, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->side_join, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "side stream");
    }
    e = cudaEventRecord(ctx->side_fork, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->side, ctx->side_fork, 0);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "fork side stream");
    *side = ctx->side;
    return ISO_OK;
}

iso_status join_side(iso_ctx* ctx) {
    cudaError_t e = cudaEventRecord(ctx->side_join, ctx->side);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->stream, ctx->side_join, 0);
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, "join side stream");
}

iso_status ensure(iso_ctx* ctx, DevBuf& b, size_t bytes) {
    if (bytes <= b.bytes) return ISO_OK;
    if (ctx->capturing) return fail(ctx, ISO_ERR_INVALID_ARG, "allocation while recording a graph");
    if (b.p) {
        // the buffer may still be read by queued work of this context
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return cuda_fail(ctx, e, "sync before regrow");
        cudaFree(b.p);
        b.p = nullptr;
        b.bytes = 0;
    }
    if (ctx->fail_alloc_after == 0) {  // iso_debug_fail_allocation: fail here as cudaMalloc would
        ctx->fail_alloc_after = -1;
        return fail(ctx, ISO_ERR_OUT_OF_MEMORY, "injected allocation failure");
    }
    if (ctx->fail_alloc_after > 0) --ctx->fail_alloc_after;
    size_t want = bytes + bytes / 8 + 256;
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
        b.p = nullptr;
        cudaGetLastError();
        return cuda_fail(ctx, e, "cudaMalloc");
    }
    b.bytes = want;
    return ISO_OK;
}

iso_status check_launch(iso_ctx* ctx, const char* what) {
    cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, what);
}

iso_status read_device_errors(iso_ctx* ctx) {
    uint32_t h = 0;
    cudaError_t e = cudaMemcpy(&h, ctx->d_err, 4, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "read error flags");
    if (h == 0) return ISO_OK;
    cudaMemset(ctx->d_err, 0, 4);
    if (h & DERR_SCAN_TIMEOUT) return fail(ctx, ISO_ERR_TIMEOUT, "scan look-back wait gave up");
    if (h & DERR_QUEUE_TIMEOUT) return fail(ctx, ISO_ERR_TIMEOUT, "work-queue wait gave up");
    if (h & DERR_SVD_ITER) return fail(ctx, ISO_ERR_TIMEOUT, "QR iteration bound reached");
    return fail(ctx, ISO_ERR_CAPACITY, "device output capacity exceeded");
}

static cudaEvent_t take_event(iso_ctx* ctx) {
    if (!ctx->event_pool.empty()) {
        cudaEvent_t e = ctx->event_pool.back();
        ctx->event_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return e;
}

StageTimer::StageTimer(iso_ctx* c, int s) : ctx(c), stage(s) {
    ctx->stage_launches[stage]++;
    if (!ctx->timing) return;
    a = take_event(ctx);
    if (a) cudaEventRecord(a, ctx->stream);
}

StageTimer::~StageTimer() {
    if (!a) return;
    cudaEvent_t b = take_event(ctx);
    if (!b) {
        ctx->event_pool.push_back(a);
        return;
    }
    cudaEventRecord(b, ctx->stream);
    ctx->pending.push_back({stage, a, b});
}

}  // namespace iso

using namespace iso;

namespace {

enum : uint32_t {
    OP_PT_DOMAIN = 0x01, OP_PT_TRANSLATE = 0x02, OP_PT_RIGID = 0x03, OP_PT_POP = 0x04,
    OP_SPHERE = 0x10, OP_BOX = 0x11, OP_CYLINDER = 0x12, OP_TORUS = 0x13,
    OP_UNION = 0x20, OP_INTERSECTION = 0x21, OP_DIFFERENCE = 0x22, OP_SMOOTH_UNION = 0x23,
    OP_SPHERE_SET = 0x30, OP_CD_BEGIN = 0x40, OP_CD_END = 0x41,
};

// Validates a program and fills the jump table; mirrors the device evaluator's limits.
bool validate(iso_program* p, std::string* err) {
    const uint32_t nops = (uint32_t)p->ops.size(), nk = (uint32_t)p->consts.size();
    p->jump.assign(nops, 0);
    struct Scope {
        uint32_t op, pc;
        int vdepth;
    };
    std::vector<Scope> scopes;
    int vsp = 0, psp = 0, cd_depth = 0;
    auto need = [&](uint32_t a, uint64_t n) { return (uint64_t)a + n <= nk; };
    for (uint32_t pc = 0; pc < nops; ++pc) {
        uint32_t op = p->ops[pc] & 0xFF, a = p->ops[pc] >> 8;
        switch (op) {
        case OP_PT_DOMAIN: case OP_PT_TRANSLATE: case OP_PT_RIGID: {
            uint32_t n = op == OP_PT_DOMAIN ? 6 : op == OP_PT_TRANSLATE ? 3 : 12;
            if (!need(a, n)) { *err = "constant index out of range"; return false; }
            if (psp + 1 >= PSTACK) { *err = "point scopes nested too deeply"; return false; }
            ++psp;
            scopes.push_back({op, pc, vsp});
            break;
        }
        case OP_PT_POP:
            if (scopes.empty() || scopes.back().op == OP_CD_BEGIN) { *err = "PT_POP without a point scope"; return false; }
            if (vsp != scopes.back().vdepth + 1) { *err = "point scope must leave exactly one value"; return false; }
            scopes.pop_back();
            --psp;
            break;
        case OP_CD_BEGIN:
            if (!need(a, 1)) { *err = "constant index out of range"; return false; }
            if (cd_depth > 0) { *err = "nested CD_BEGIN is not supported"; return false; }
            ++cd_depth;
            scopes.push_back({op, pc, vsp});
            break;
        case OP_CD_END:
            if (scopes.empty() || scopes.back().op != OP_CD_BEGIN) { *err = "CD_END without CD_BEGIN"; return false; }
            if (vsp != scopes.back().vdepth + 1) { *err = "CD scope must leave exactly one value"; return false; }
            p->jump[scopes.back().pc] = (int32_t)pc;
            scopes.pop_back();
            --cd_depth;
            break;
        case OP_SPHERE: case OP_BOX: case OP_CYLINDER: case OP_TORUS: {
            uint32_t n = op == OP_SPHERE ? 1 : op == OP_BOX ? 3 : 2;
            if (!need(a, n)) { *err = "constant index out of range"; return false; }
            if (++vsp > VSTACK) { *err = "value stack deeper than 16"; return false; }
            break;
        }
        case OP_UNION: case OP_INTERSECTION: case OP_DIFFERENCE: case OP_SMOOTH_UNION:
            if (op == OP_SMOOTH_UNION && !need(a, 1)) { *err = "constant index out of range"; return false; }
            if (op == OP_SMOOTH_UNION && !(p->consts[a] > 0.0f)) { *err = "smooth union needs k > 0"; return false; }
            if (vsp - (scopes.empty() ? 0 : scopes.back().vdepth) < 2) { *err = "binary op needs two operands"; return false; }
            --vsp;
            break;
        case OP_SPHERE_SET: {
            if (!need(a, 3)) { *err = "constant index out of range"; return false; }
            float fn = p->consts[a];
            if (!(fn >= 1.0f) || fn != std::floor(fn) || fn > 16777216.0f) { *err = "bad sphere count"; return false; }
            if (!need(a + 3, 4ull * (uint64_t)fn)) { *err = "sphere data out of range"; return false; }
            if (p->consts[a + 1] != 0.0f && !(p->consts[a + 2] > 0.0f)) { *err = "smooth set needs k > 0"; return false; }
            if (++vsp > VSTACK) { *err = "value stack deeper than 16"; return false; }
            break;
        }
        default:
            *err = "unknown opcode";
            return false;
        }
    }
    if (!scopes.empty()) { *err = "unclosed scope"; return false; }
    if (vsp != 1) { *err = "program must leave exactly one value"; return false; }
    return true;
}

void classify(iso_program* p) {
    const auto& o = p->ops;
    auto op = [&](size_t i) { return o[i] & 0xFF; };
    auto arg = [&](size_t i) { return o[i] >> 8; };
    p->kind = PK_GENERIC;
    size_t set_pc = SIZE_MAX;
    if (o.size() == 1 && op(0) == OP_SPHERE_SET) {
        set_pc = 0;
        p->has_domain = false;
    } else if (o.size() == 3 && op(0) == OP_PT_DOMAIN && op(1) == OP_SPHERE_SET && op(2) == OP_PT_POP) {
        set_pc = 1;
        p->has_domain = true;
        for (int i = 0; i < 6; ++i) p->domain[i] = p->consts[arg(0) + i];
    }
    if (set_pc != SIZE_MAX && p->consts[arg(set_pc) + 1] == 0.0f) {
        p->kind = PK_SPHERE_SET_HARD;
        p->set_at = arg(set_pc);
        p->set_n = (uint32_t)p->consts[p->set_at];
    }
    // [DOMAIN] TRANSLATE prim POP (TRANSLATE prim POP UNION)* [POP]: a left
    // fold of hard unions over translated primitives, compiled to a flat list
    // that the evaluator walks with the same operations in the same order
    size_t i = 0;
    int32_t dom = -1;
    if (o.size() > 0 && op(0) == OP_PT_DOMAIN) {
        dom = (int32_t)arg(0);
        i = 1;
    }
    std::vector<float> prims;
    bool ok = true;
    size_t groups = 0;
    while (ok && i + 3 <= o.size() && op(i) == OP_PT_TRANSLATE) {
        const uint32_t pr = op(i + 1);
        if (op(i + 2) != OP_PT_POP || !(pr == OP_SPHERE || pr == OP_BOX || pr == OP_CYLINDER || pr == OP_TORUS)) {
            ok = false;
            break;
        }
        if (groups > 0) {
            if (i + 3 >= o.size() || op(i + 3) != OP_UNION) {
                ok = false;
                break;
            }
        }
        const float* c = p->consts.data() + arg(i);
        const float* a = p->consts.data() + arg(i + 1);
        const int na = pr == OP_SPHERE ? 1 : (pr == OP_BOX ? 3 : 2);
        float rec[8] = {c[0], c[1], c[2], 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        std::memcpy(&rec[3], &pr, 4);
        for (int j = 0; j < na; ++j) rec[4 + j] = a[j];
        prims.insert(prims.end(), rec, rec + 8);
        i += groups > 0 ? 4 : 3;
        ++groups;
    }
    if (ok && groups > 0 && ((dom < 0 && i == o.size()) || (dom >= 0 && i + 1 == o.size() && op(i) == OP_PT_POP))) {
        p->prims = std::move(prims);
        p->prim_dom_at = dom;
    }
}

// Bounds for culled sampling.  Every primitive (sphere.rs, rectangular_prism.rs,
// cylinder.rs, torus.rs) and sphere set is an exact signed distance, so
// 1-Lipschitz in its own coordinates; a translation keeps distances, a domain
// map scales them by at most its largest |scale|, a rigid map by its matrix's
// spectral norm (bounded by Gershgorin's theorem on M^T M); min, max,
// negation and the polynomial smooth minimum (partial derivatives
// non-negative and summing to 1) keep the larger bound of their operands.
// So the value's bound is the largest product of point-map norms above any
// primitive.  The magnitude of every point coordinate and value the
// evaluator meets is tracked alongside, for points in [0, 2]^3; the f32
// rounding error of a value is a few tens of units in the last place of that
// magnitude, and the slack allows 2^10 of them for each of two values.
void cull_bounds(iso_program* p) {
    p->lip = 0.0f;
    p->slack = 0.0f;
    const auto& o = p->ops;
    const float* K = p->consts.data();
    for (float c : p->consts)
        if (!std::isfinite(c)) return;
    double scale = 1.0, mag = 2.0 * std::sqrt(3.0), lip = 0.0, vmag = 0.0;
    std::vector<std::pair<double, double>> saved;
    auto norm3 = [](const float* v) { return std::sqrt((double)v[0] * v[0] + (double)v[1] * v[1] + (double)v[2] * v[2]); };
    for (size_t pc = 0; pc < o.size(); ++pc) {
        const uint32_t op = o[pc] & 0xFFu;
        const float* k = K + (o[pc] >> 8);
        switch (op) {
        case OP_PT_DOMAIN: {
            const double s = std::max({std::fabs((double)k[0]), std::fabs((double)k[1]), std::fabs((double)k[2])});
            saved.push_back({scale, mag});
            scale *= s;
            mag = s * mag + norm3(k + 3);
            break;
        }
        case OP_PT_TRANSLATE:
            saved.push_back({scale, mag});
            mag += norm3(k);
            break;
        case OP_PT_RIGID: {
            double g = 0.0;  // Gershgorin bound on the largest eigenvalue of M^T M
            for (int i = 0; i < 3; ++i) {
                double row = 0.0;
                for (int j = 0; j < 3; ++j) {
                    double a = 0.0;
                    for (int r = 0; r < 3; ++r) a += (double)k[3 + 3 * r + i] * (double)k[3 + 3 * r + j];
                    row += std::fabs(a);
                }
                g = std::max(g, row);
            }
            const double n = std::sqrt(g) * (1.0 + 1e-6);
            saved.push_back({scale, mag});
            scale *= n;
            mag = n * (mag + norm3(k));
            break;
        }
        case OP_PT_POP:
            if (saved.empty()) return;
            scale = saved.back().first;
            mag = saved.back().second;
            saved.pop_back();
            break;
        case OP_SPHERE: case OP_BOX: case OP_CYLINDER: case OP_TORUS: {
            const int na = op == OP_SPHERE ? 1 : (op == OP_BOX ? 3 : 2);
            double a = 0.0;
            for (int j = 0; j < na; ++j) a += std::fabs((double)k[j]);
            lip = std::max(lip, scale);
            vmag = std::max(vmag, mag + a);
            break;
        }
        case OP_SPHERE_SET: {
            const uint32_t n = (uint32_t)k[0];
            double cmax = 0.0;
            for (uint32_t i = 0; i < n; ++i) cmax = std::max(cmax, norm3(k + 3 + 4 * i) + std::fabs((double)k[6 + 4 * i]));
            lip = std::max(lip, scale);
            vmag = std::max(vmag, mag + cmax + std::fabs((double)k[2]));
            break;
        }
        case OP_SMOOTH_UNION:
            vmag += std::fabs((double)k[0]);
            break;
        default:
            break;  // min, max, negation and the CD markers
        }
    }
    const double m = std::max(vmag, mag);
    if (!(lip > 0.0) || !(lip < 1e30) || !(m < 1e30)) return;
    p->lip = (float)(lip * (1.0 + 1e-6));
    p->slack = (float)(m * std::ldexp(1.0, -13));
}

}  // namespace

namespace iso {

iso_status sample_lattice(iso_ctx* ctx, const iso_program* prog, uint32_t size, Lattice* L) {
    const uint32_t nx = size, ny = size, nz = size + 1;
    const uint64_t pitch = default_pitch(nx);
    const uint32_t W = words_per_row(nx);
    iso_status s;
    if ((s = ensure(ctx, ctx->field, 4ull * pitch * ny * nz)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->bits, 4ull * W * ny * nz)) != ISO_OK) return s;
    const float inv = 1.0f / (float)(size - 1);
    // marching cubes reads values only at the ends of crossing edges: the
    // sampler may skip the values far from the surface
    if ((s = launch_sample_grid(ctx, prog, nx, ny, nz, inv, (float*)ctx->field.p, pitch, (uint32_t*)ctx->bits.p,
                                true)) != ISO_OK)
        return s;
    *L = Lattice{nx, ny, nz, pitch, (const float*)ctx->field.p, (const uint32_t*)ctx->bits.p, W, inv, nullptr};
    return ISO_OK;
}

iso_status sample_lattice_slab(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t zlo, uint32_t nz,
                               Lattice* L) {
    const uint32_t nx = size, ny = size;
    const uint64_t pitch = default_pitch(nx);
    const uint32_t W = words_per_row(nx);
    iso_status s;
    if ((s = ensure(ctx, ctx->field, 4ull * pitch * ny * nz)) != ISO_OK) return s;
    if ((s = ensure(ctx, ctx->bits, 4ull * W * ny * nz)) != ISO_OK) return s;
    const float inv = 1.0f / (float)(size - 1);
    if ((s = launch_sample_grid(ctx, prog, nx, ny, nz, inv, (float*)ctx->field.p, pitch, (uint32_t*)ctx->bits.p,
                                true, zlo)) != ISO_OK)
        return s;
    *L = Lattice{nx, ny, nz, pitch, (const float*)ctx->field.p, (const uint32_t*)ctx->bits.p, W, inv, nullptr, zlo};
    return ISO_OK;
}

}  // namespace iso

namespace {

// Contexts alive in this process: a program destroyed after its context
// (a caller's order, or a garbage collector's) frees its block directly.
std::mutex g_ctx_mutex;
std::unordered_set<const iso_ctx*> g_live_ctx;

constexpr size_t POOL_BLOCKS = 32;  // free program blocks a context keeps

// A device block of at least `bytes` for a program: the smallest free one
// of the context that is not more than twice too large, else a new one.
cudaError_t program_block(iso_ctx* ctx, size_t bytes, void** block, size_t* cap) {
    {
        std::lock_guard<std::mutex> lock(g_ctx_mutex);
        auto& fb = ctx->free_blocks;
        size_t best = fb.size();
        for (size_t i = 0; i < fb.size(); ++i)
            if (fb[i].first >= bytes && fb[i].first <= 2 * bytes + 4096 &&
                (best == fb.size() || fb[i].first < fb[best].first))
                best = i;
        if (best < fb.size()) {
            *cap = fb[best].first;
            *block = fb[best].second;
            fb.erase(fb.begin() + (ptrdiff_t)best);
            return cudaSuccess;
        }
    }
    *cap = (bytes + 255) & ~(size_t)255;
    return cudaMalloc(block, *cap);
}

}  // namespace

extern "C" {

const char* iso_status_str(iso_status s) {
    switch (s) {
    case ISO_OK: return "ISO_OK";
    case ISO_ERR_INVALID_ARG: return "ISO_ERR_INVALID_ARG";
    case ISO_ERR_CAPACITY: return "ISO_ERR_CAPACITY";
    case ISO_ERR_CUDA: return "ISO_ERR_CUDA";
    case ISO_ERR_TIMEOUT: return "ISO_ERR_TIMEOUT";
    case ISO_ERR_BAD_PROGRAM: return "ISO_ERR_BAD_PROGRAM";
    case ISO_ERR_NO_DEVICE: return "ISO_ERR_NO_DEVICE";
    case ISO_ERR_OUT_OF_MEMORY: return "ISO_ERR_OUT_OF_MEMORY";
    case ISO_ERR_TOO_LARGE: return "ISO_ERR_TOO_LARGE";
    case ISO_ERR_UNSUPPORTED: return "ISO_ERR_UNSUPPORTED";
    default: return "ISO_ERR_UNKNOWN";
    }
}

const char* iso_ctx_last_error(const iso_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

iso_status iso_ctx_create(int device, iso_ctx** out) {
    if (!out) return ISO_ERR_INVALID_ARG;
    *out = nullptr;
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        return ISO_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) return ISO_ERR_NO_DEVICE;
    iso_ctx* ctx = new (std::nothrow) iso_ctx();
    if (!ctx) return ISO_ERR_OUT_OF_MEMORY;
    ctx->device = device;
    cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
    if (ctx->sms < 1) ctx->sms = 1;
    iso_status s = set_device(ctx);
    cudaError_t e = cudaSuccess;
    if (s == ISO_OK) e = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking);
    if (s == ISO_OK && e == cudaSuccess) e = cudaMallocHost(&ctx->h_pinned, 4096);
    if (s == ISO_OK && e == cudaSuccess) e = cudaMalloc(&ctx->d_err, 256);
    if (s == ISO_OK && e == cudaSuccess) e = cudaMemset(ctx->d_err, 0, 256);
    if (s != ISO_OK || e != cudaSuccess) {
        iso_status r = s != ISO_OK ? s : cuda_fail(ctx, e, "context setup");
        iso_ctx_destroy(ctx);
        return r;
    }
    ctx->stream = ctx->own_stream;
    {
        std::lock_guard<std::mutex> lock(g_ctx_mutex);
        g_live_ctx.insert(ctx);
    }
    *out = ctx;
    return ISO_OK;
}

iso_status iso_ctx_destroy(iso_ctx* ctx) {
    if (!ctx) return ISO_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    {
        std::lock_guard<std::mutex> lock(g_ctx_mutex);
        g_live_ctx.erase(ctx);
        for (auto& b : ctx->free_blocks) cudaFree(b.second);
        ctx->free_blocks.clear();
    }
    DevBuf* bufs[] = {&ctx->field, &ctx->bits, &ctx->rowtri, &ctx->rowvert, &ctx->scan, &ctx->aux,
                      &ctx->aux2, &ctx->aux3, &ctx->tiles, &ctx->edges, &ctx->mesh_v, &ctx->mesh_i, &ctx->mesh_k};
    for (DevBuf* b : bufs)
        if (b->p) cudaFree(b->p);
    if (ctx->d_err) cudaFree(ctx->d_err);
    if (ctx->h_pinned) cudaFreeHost(ctx->h_pinned);
    for (auto& p : ctx->pending) {
        cudaEventDestroy(p.a);
        cudaEventDestroy(p.b);
    }
    for (cudaEvent_t ev : ctx->event_pool) cudaEventDestroy(ev);
    mc_plan_release(ctx);
    lhmc_plan_release(ctx);
    if (ctx->side) {
        cudaStreamSynchronize(ctx->side);
        cudaStreamDestroy(ctx->side);
    }
    if (ctx->side_fork) cudaEventDestroy(ctx->side_fork);
    if (ctx->side_join) cudaEventDestroy(ctx->side_join);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return ISO_OK;
}

iso_status iso_ctx_get_stream(iso_ctx* ctx, void** stream) {
    if (!ctx || !stream) return ISO_ERR_INVALID_ARG;
    *stream = (void*)ctx->stream;
    return ISO_OK;
}

iso_status iso_ctx_set_stream(iso_ctx* ctx, void* stream) {
    if (!ctx) return ISO_ERR_INVALID_ARG;
    // program uploads are ordered on the context's stream: let them land
    // before work moves to another one
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return ISO_OK;
}

uint64_t iso_ctx_kernel_launches(const iso_ctx* ctx) { return ctx ? ctx->launches : 0; }

iso_status iso_debug_fail_allocation(iso_ctx* ctx, int64_t after) {
    if (!ctx) return ISO_ERR_INVALID_ARG;
    ctx->fail_alloc_after = after < 0 ? -1 : after;
    return ISO_OK;
}

iso_status iso_ctx_enable_stage_timing(iso_ctx* ctx, int enable) {
    if (!ctx) return ISO_ERR_INVALID_ARG;
    ctx->timing = enable != 0;
    return ISO_OK;
}

iso_status iso_ctx_stage_times(iso_ctx* ctx, double* ms, uint64_t* launches) {
    if (!ctx) return ISO_ERR_INVALID_ARG;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "stage times");
    for (auto& p : ctx->pending) {
        float t = 0.0f;
        if (cudaEventElapsedTime(&t, p.a, p.b) == cudaSuccess) ctx->stage_ms[p.stage] += t;
        else cudaGetLastError();
        ctx->event_pool.push_back(p.a);
        ctx->event_pool.push_back(p.b);
    }
    ctx->pending.clear();
    for (int i = 0; i < ISO_STAGE_COUNT; ++i) {
        if (ms) ms[i] = ctx->stage_ms[i];
        if (launches) launches[i] = ctx->stage_launches[i];
        ctx->stage_ms[i] = 0.0;
        ctx->stage_launches[i] = 0;
    }
    return ISO_OK;
}

}  // extern "C"

namespace iso {
// The host side of a program from its bytes: header checks, ops and
// constants, validation, fast-path forms and culling bounds (no device work).
iso_status parse_program(const uint8_t* bytes, size_t len, iso_program* p, std::string* err) {
    if (len < 16) return *err = "program shorter than its header", ISO_ERR_BAD_PROGRAM;
    uint32_t h[4];
    std::memcpy(h, bytes, 16);
    if (h[0] != 0x314F5349u) return *err = "bad magic", ISO_ERR_BAD_PROGRAM;
    if ((uint64_t)16 + 4ull * h[1] + 4ull * h[2] != len)
        return *err = "length does not match header", ISO_ERR_BAD_PROGRAM;
    if (h[1] == 0) return *err = "empty program", ISO_ERR_BAD_PROGRAM;
    p->ops.resize(h[1]);
    p->consts.resize(h[2]);
    std::memcpy(p->ops.data(), bytes + 16, 4ull * h[1]);
    if (h[2]) std::memcpy(p->consts.data(), bytes + 16 + 4ull * h[1], 4ull * h[2]);
    if (!validate(p, err)) return ISO_ERR_BAD_PROGRAM;
    classify(p);
    cull_bounds(p);
    uint64_t hash = 0xCBF29CE484222325ull;  // FNV-1a 64
    for (size_t i = 0; i < len; ++i) hash = (hash ^ bytes[i]) * 0x100000001B3ull;
    p->content_hash = hash;
    return ISO_OK;
}
}  // namespace iso

extern "C" {

iso_status iso_program_create(iso_ctx* ctx, const uint8_t* bytes, size_t len, iso_program** out) {
    if (!ctx || !bytes || !out) return ISO_ERR_INVALID_ARG;
    *out = nullptr;
    iso_program* p = new (std::nothrow) iso_program();
    if (!p) return ISO_ERR_OUT_OF_MEMORY;
    p->ctx = ctx;
    p->device = ctx->device;
    static std::atomic<uint64_t> next_uid{1};
    p->uid = next_uid.fetch_add(1);
    std::string err;
    iso_status s = parse_program(bytes, len, p, &err);
    if (s != ISO_OK) {
        delete p;
        return fail(ctx, s, err);
    }
    s = set_device(ctx);
    if (s != ISO_OK) {
        delete p;
        return s;
    }
    // one device block holds every array (16-byte aligned pieces, so the
    // sphere data of the fast path takes float4 loads), from the context's
    // pool of blocks that destroyed programs left (else a new allocation),
    // filled by one copy ordered on the context's stream: after the work
    // that used the block before, before the work that uses it now
    const size_t nk = p->consts.size() + 4;
    auto at16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
    const size_t o_ops = 0, o_consts = at16(o_ops + 4 * p->ops.size()), o_jump = at16(o_consts + 4 * nk);
    const size_t o_set = at16(o_jump + 4 * p->jump.size());
    const size_t set_bytes = p->kind == PK_SPHERE_SET_HARD ? 16ull * p->set_n : 0;
    const size_t o_prims = at16(o_set + set_bytes), total = at16(o_prims + 4 * p->prims.size());
    std::vector<unsigned char> staged(total, 0);
    std::memcpy(staged.data() + o_ops, p->ops.data(), 4 * p->ops.size());
    if (!p->consts.empty()) std::memcpy(staged.data() + o_consts, p->consts.data(), 4 * p->consts.size());
    if (!p->jump.empty()) std::memcpy(staged.data() + o_jump, p->jump.data(), 4 * p->jump.size());
    if (set_bytes) std::memcpy(staged.data() + o_set, p->consts.data() + p->set_at + 3, set_bytes);
    if (!p->prims.empty()) std::memcpy(staged.data() + o_prims, p->prims.data(), 4 * p->prims.size());
    unsigned char* block = nullptr;
    cudaError_t e = program_block(ctx, total, (void**)&block, &p->block_bytes);
    if (e == cudaSuccess) {
        p->d_block = block;
        p->d_ops = (uint32_t*)(block + o_ops);
        p->d_consts = (float*)(block + o_consts);
        p->d_jump = (int32_t*)(block + o_jump);
        if (set_bytes) p->d_set = (float*)(block + o_set);
        if (!p->prims.empty()) p->d_prims = (float4*)(block + o_prims);
        // from pageable memory: returns once the bytes are staged
        e = cudaMemcpyAsync(block, staged.data(), total, cudaMemcpyHostToDevice, ctx->stream);
    }
    if (e != cudaSuccess) {
        iso_status r = cuda_fail(ctx, e, "program upload");
        iso_program_destroy(p);
        return r;
    }
    *out = p;
    return ISO_OK;
}

iso_status iso_program_destroy(iso_program* p) {
    if (!p) return ISO_ERR_INVALID_ARG;
    if (p->d_block) {
        bool pooled = false;
        {
            std::lock_guard<std::mutex> lock(g_ctx_mutex);
            if (p->ctx && g_live_ctx.count(p->ctx) && p->ctx->free_blocks.size() < POOL_BLOCKS) {
                // kept for the context's next upload, which its stream orders
                // after every kernel queued so far that reads this block
                p->ctx->free_blocks.push_back({p->block_bytes, p->d_block});
                pooled = true;
            }
        }
        if (!pooled) {
            // the context may be gone: the program keeps its own device
            int cur = 0;
            const bool moved = cudaGetDevice(&cur) == cudaSuccess && cur != p->device &&
                               cudaSetDevice(p->device) == cudaSuccess;
            cudaFree(p->d_block);
            if (moved) cudaSetDevice(cur);
            cudaGetLastError();
        }
    }
    delete p;
    return ISO_OK;
}

iso_status iso_mesh_download(iso_ctx* ctx, float* vertices, uint64_t vertex_floats_cap, uint32_t* indices,
                             uint64_t index_cap, uint64_t* keys, uint64_t key_cap) {
    if (!ctx) return ISO_ERR_INVALID_ARG;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    const uint64_t nvf = ctx->last.num_vertices * (uint64_t)ctx->last_vertex_floats;
    const uint64_t ni = 3 * ctx->last.num_triangles;
    if ((vertices && vertex_floats_cap < nvf) || (indices && index_cap < ni))
        return fail(ctx, ISO_ERR_CAPACITY, "host buffers too small for the mesh");
    if (keys) {
        if (!(ctx->last_flags & ISO_FLAG_KEYS)) return fail(ctx, ISO_ERR_INVALID_ARG, "mesh was extracted without keys");
        if (key_cap < 2 * ctx->last.num_vertices) return fail(ctx, ISO_ERR_CAPACITY, "key buffer too small");
    }
    cudaError_t e = cudaSuccess;
    if (vertices && nvf) e = cudaMemcpyAsync(vertices, ctx->mesh_v.p, 4 * nvf, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && indices && ni)
        e = cudaMemcpyAsync(indices, ctx->mesh_i.p, 4 * ni, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && keys && ctx->last.num_vertices)
        e = cudaMemcpyAsync(keys, ctx->mesh_k.p, 16 * ctx->last.num_vertices, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, "mesh download");
}

iso_status iso_mesh_device(iso_ctx* ctx, const float** vertices, const uint32_t** indices, const uint64_t** keys,
                           iso_mesh_info* info) {
    if (!ctx) return ISO_ERR_INVALID_ARG;
    if (vertices) *vertices = (const float*)ctx->mesh_v.p;
    if (indices) *indices = (const uint32_t*)ctx->mesh_i.p;
    if (keys) *keys = (ctx->last_flags & ISO_FLAG_KEYS) ? (const uint64_t*)ctx->mesh_k.p : nullptr;
    if (info) *info = ctx->last;
    return ISO_OK;
}


static iso_status check_size(iso_ctx* ctx, const iso_program* prog, uint32_t size) {
    if (!ctx || !prog) return ISO_ERR_INVALID_ARG;
    if (prog->ctx != ctx) return fail(ctx, ISO_ERR_INVALID_ARG, "program belongs to another context");
    if (size == 0) return fail(ctx, ISO_ERR_INVALID_ARG, "size must be at least 1");
    if (size > 65536) return fail(ctx, ISO_ERR_INVALID_ARG, "size above 65536");
    return set_device(ctx);
}

iso_status iso_sample_grid(iso_ctx* ctx, const iso_program* prog, uint32_t size, float* field, uint64_t pitch) {
    iso::NvtxRange nvtx_range("iso_sample_grid");
    iso_status s = check_size(ctx, prog, size);
    if (s != ISO_OK) return s;
    if (!field || pitch < size) return fail(ctx, ISO_ERR_INVALID_ARG, "field null or pitch < size");
    const uint32_t W = words_per_row(size);
    if ((s = ensure(ctx, ctx->bits, 4ull * W * size * (size + 1))) != ISO_OK) return s;
    const float inv = size > 1 ? 1.0f / (float)(size - 1) : 0.0f;
    if ((s = launch_sample_grid(ctx, prog, size, size, size + 1, inv, field, pitch, (uint32_t*)ctx->bits.p)) != ISO_OK)
        return s;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, "sample grid");
}

iso_status iso_sample_grid_near(iso_ctx* ctx, const iso_program* prog, uint32_t size, float* field, uint64_t pitch,
                                uint32_t* bits) {
    iso::NvtxRange nvtx_range("iso_sample_grid_near");
    iso_status s = check_size(ctx, prog, size);
    if (s != ISO_OK) return s;
    if (!field || !bits || pitch < size) return fail(ctx, ISO_ERR_INVALID_ARG, "field or bits null or pitch < size");
    const float inv = size > 1 ? 1.0f / (float)(size - 1) : 0.0f;
    if ((s = launch_sample_grid(ctx, prog, size, size, size + 1, inv, field, pitch, bits, true)) != ISO_OK) return s;
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, "sample grid near");
}

iso_status iso_program_lipschitz(const iso_program* prog, float* lip) {
    if (!prog || !lip) return ISO_ERR_INVALID_ARG;
    *lip = prog->lip;
    return ISO_OK;
}

iso_status iso_mc_extract(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t flags, iso_mesh_info* info) {
    iso::NvtxRange nvtx_range("iso_mc_extract");
    iso_status s = check_size(ctx, prog, size);
    if (s != ISO_OK) return s;
    if (flags & ~(uint32_t)(ISO_FLAG_KEYS | ISO_FLAG_NORMALS)) return fail(ctx, ISO_ERR_INVALID_ARG, "unknown flags");
    if (size == 1) {
        ctx->last = iso_mesh_info{};
        ctx->last_flags = flags;
        ctx->last_vertex_floats = (flags & ISO_FLAG_NORMALS) ? 6 : 3;
        if (info) *info = ctx->last;
        return ISO_OK;
    }
    if ((s = mc_extract_program(ctx, prog, size, flags & ~(uint32_t)ISO_FLAG_NORMALS, info)) != ISO_OK) return s;
    return (flags & ISO_FLAG_NORMALS) ? attach_normals(ctx, prog) : ISO_OK;
}


// the device-side address of page-locked host memory (null: pageable,
// device memory or unknown)
static void* pinned_device_view(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

iso_status iso_host_register(void* p, uint64_t bytes) {
    if (!p || !bytes) return ISO_ERR_INVALID_ARG;
    const cudaError_t e = cudaHostRegister(p, bytes, cudaHostRegisterMapped | cudaHostRegisterPortable);
    if (e == cudaSuccess) return ISO_OK;
    cudaGetLastError();
    return e == cudaErrorHostMemoryAlreadyRegistered ? ISO_ERR_INVALID_ARG : ISO_ERR_CUDA;
}

iso_status iso_host_unregister(void* p) {
    if (!p) return ISO_ERR_INVALID_ARG;
    const cudaError_t e = cudaHostUnregister(p);
    if (e == cudaSuccess) return ISO_OK;
    cudaGetLastError();
    return e == cudaErrorHostMemoryNotRegistered ? ISO_ERR_INVALID_ARG : ISO_ERR_CUDA;
}

iso_status iso_mc_extract_host(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t flags, float* vertices,
                               uint64_t vertex_floats, uint32_t* indices, uint64_t index_count, iso_mesh_info* info) {
    iso::NvtxRange nvtx_range("iso_mc_extract_host");
    if (!ctx) return ISO_ERR_INVALID_ARG;
    if ((!vertices && vertex_floats) || (!indices && index_count))
        return fail(ctx, ISO_ERR_INVALID_ARG, "null host buffer with nonzero room");
    iso_status s = check_size(ctx, prog, size);
    if (s != ISO_OK) return s;
    if (flags & ~(uint32_t)(ISO_FLAG_KEYS | ISO_FLAG_NORMALS | ISO_FLAG_HOST_COPY))
        return fail(ctx, ISO_ERR_INVALID_ARG, "unknown flags");
    void* dv = flags == 0 && size > 1 ? pinned_device_view(vertices) : nullptr;
    void* di = dv ? pinned_device_view(indices) : nullptr;
    const bool direct = dv && di && ((uintptr_t)di & 15) == 0;
    iso_mesh_info mi{};
    if (direct) {
        ctx->host_out = iso_ctx::HostOut{(float*)dv, (uint32_t*)di, vertex_floats / 3, index_count / 3, false};
        s = mc_extract_program(ctx, prog, size, 0, &mi);
        const bool delivered = ctx->host_out.armed;
        ctx->host_out = iso_ctx::HostOut{};
        if (s != ISO_OK) return s;
        if (info) *info = mi;
        if (3 * mi.num_vertices > vertex_floats || 3 * mi.num_triangles > index_count)
            return fail(ctx, ISO_ERR_CAPACITY, "host buffers too small for the mesh (its size is in info)");
        if (delivered) return ISO_OK;
        // the lattice went through the block emit, which writes only the device mesh
        return iso_mesh_download(ctx, vertices, vertex_floats, indices, index_count, nullptr, 0);
    }
    flags &= ~(uint32_t)ISO_FLAG_HOST_COPY;
    if ((s = iso_mc_extract(ctx, prog, size, flags, &mi)) != ISO_OK) return s;
    if (info) *info = mi;
    const uint64_t vf = (flags & ISO_FLAG_NORMALS) ? 6 : 3;
    if (vf * mi.num_vertices > vertex_floats || 3 * mi.num_triangles > index_count)
        return fail(ctx, ISO_ERR_CAPACITY, "host buffers too small for the mesh (its size is in info)");
    return iso_mesh_download(ctx, vertices, vertex_floats, indices, index_count, nullptr, 0);
}

iso_status iso_mc_extract_field(iso_ctx* ctx, const float* field, uint32_t nx, uint32_t ny, uint32_t nz, uint64_t pitch,
                                uint32_t flags, iso_mesh_info* info) {
    iso::NvtxRange nvtx_range("iso_mc_extract_field");
    if (!ctx || !field) return ISO_ERR_INVALID_ARG;
    if (nx != ny || nx < 2 || nz < 2 || pitch < nx || nx > 65536 || nz > 65537)
        return fail(ctx, ISO_ERR_INVALID_ARG, "need nx == ny >= 2, nz >= 2, pitch >= nx");
    if (flags & ~(uint32_t)ISO_FLAG_KEYS) return fail(ctx, ISO_ERR_INVALID_ARG, "unknown flags");
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    const uint32_t W = words_per_row(nx);
    if ((s = ensure(ctx, ctx->bits, 4ull * W * ny * nz)) != ISO_OK) return s;
    if ((s = launch_sign_bits(ctx, field, nx, ny, nz, pitch, (uint32_t*)ctx->bits.p)) != ISO_OK) return s;
    Lattice L{nx, ny, nz, pitch, field, (const uint32_t*)ctx->bits.p, W, 1.0f / (float)(nx - 1), nullptr};
    return mc_extract_lattice(ctx, L, flags, info);
}

iso_status iso_mc_extract_slab(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t z_begin,
                               uint32_t z_end, uint32_t flags, iso_mesh_info* info, uint64_t* halo_vertices,
                               uint64_t* halo_triangles) {
    iso::NvtxRange nvtx_range("iso_mc_extract_slab");
    iso_status s = check_size(ctx, prog, size);
    if (s != ISO_OK) return s;
    if (size < 2 || !(z_begin < z_end) || z_end > size)
        return fail(ctx, ISO_ERR_INVALID_ARG, "need size >= 2 and 0 <= z_begin < z_end <= size");
    if (flags & ~(uint32_t)ISO_FLAG_KEYS) return fail(ctx, ISO_ERR_INVALID_ARG, "unknown flags");
    return mc_extract_slab(ctx, prog, size, z_begin, z_end, flags, info, halo_vertices, halo_triangles);
}

iso_status iso_mc_cases(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint8_t* cases_host) {
    iso_status s = check_size(ctx, prog, size);
    if (s != ISO_OK) return s;
    if (!cases_host) return fail(ctx, ISO_ERR_INVALID_ARG, "null output");
    if (size < 2) return ISO_OK;
    Lattice L;
    if ((s = sample_lattice(ctx, prog, size, &L)) != ISO_OK) return s;
    const uint64_t ncells = (uint64_t)(size - 1) * (size - 1) * size;
    if ((s = ensure(ctx, ctx->aux, ncells)) != ISO_OK) return s;
    if ((s = mc_cases_lattice(ctx, L, (uint8_t*)ctx->aux.p)) != ISO_OK) return s;
    cudaError_t e = cudaMemcpyAsync(cases_host, ctx->aux.p, ncells, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, "mc cases");
}

iso_status iso_sample_points(iso_ctx* ctx, const iso_program* prog, const float* points, uint64_t n, float* values,
                             float* normals) {
    if (!ctx || !prog || (!points && n) || (!values && n)) return ISO_ERR_INVALID_ARG;
    iso_status s = set_device(ctx);
    if (s != ISO_OK) return s;
    if (n == 0) return ISO_OK;
    if ((s = ensure(ctx, ctx->aux, 28 * n)) != ISO_OK) return s;
    float* d_pts = (float*)ctx->aux.p;
    float* d_vals = d_pts + 3 * n;
    float* d_nrm = d_vals + n;
    cudaError_t e = cudaMemcpyAsync(d_pts, points, 12 * n, cudaMemcpyHostToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "upload points");
    if ((s = launch_sample_points(ctx, prog, d_pts, n, d_vals, normals ? d_nrm : nullptr)) != ISO_OK) return s;
    e = cudaMemcpyAsync(values, d_vals, 4 * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess && normals) e = cudaMemcpyAsync(normals, d_nrm, 12 * n, cudaMemcpyDeviceToHost, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    return e == cudaSuccess ? ISO_OK : cuda_fail(ctx, e, "sample points");
}

iso_status iso_point_cloud_extract(iso_ctx* ctx, const iso_program* prog, uint32_t size, uint32_t flags,
                                   iso_mesh_info* info) {
    iso::NvtxRange nvtx_range("iso_point_cloud_extract");
    iso_status s = check_size(ctx, prog, size);
    if (s != ISO_OK) return s;
    if (flags & ~(uint32_t)ISO_FLAG_NORMALS) return fail(ctx, ISO_ERR_INVALID_ARG, "unsupported flags");
    if (size == 1) {  // no cell
        ctx->last = iso_mesh_info{};
        ctx->last_flags = 0;
        ctx->last_vertex_floats = 3;
    } else {
        Lattice L;
        if ((s = sample_lattice(ctx, prog, size, &L)) != ISO_OK) return s;
        if ((s = point_cloud_lattice(ctx, L, nullptr)) != ISO_OK) return s;
    }
    if ((flags & ISO_FLAG_NORMALS) && (s = attach_normals(ctx, prog)) != ISO_OK) return s;
    if (info) *info = ctx->last;
    return ISO_OK;
}

}  // extern "C"
