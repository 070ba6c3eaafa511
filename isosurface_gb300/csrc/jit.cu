// Per-program compiled evaluators for the culled sampler and the full field.
//
// The interpreter (vm.cuh) spends most of its instructions on dispatch and
// on its value and point stacks in local memory.  For a general program (no
// sphere set) the library instead writes the program out as straight-line
// CUDA C -- the same primitive functions (vm_math.cuh) and the same f32
// operations in the same order, constants as exact bit patterns -- around
// the samplers' device code (bricks_core.cuh), compiles it with NVRTC at run
// time (--fmad=false, so nothing is contracted: values stay bit-identical to
// the interpreter's), and launches the kernels from the loaded module: the
// culled sampler's two (not for a flat union of translated primitives,
// whose interpreted form prunes the primitives per sub-brick), the full
// field's one and, when the program's normals are written out too (no
// central difference), DualContouring's placement pass (dc_core.cuh).  Modules are cached
// per program contents for the life of the process.  NVRTC is loaded with
// dlopen on first use; without it, or when a compilation fails, the
// interpreter runs instead.
#include <cuda_runtime.h>
#include <dlfcn.h>
#include <nvrtc.h>

#include <atomic>
#include <cinttypes>
#include <cstdio>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "bricks.cuh"
#include "internal.h"
#include "qef.cuh"
#include "vm.cuh"
#include "dc_core.cuh"

// the texts of vm_math.cuh, bricks_core.cuh, qef_planes.cuh and dc_core.cuh
// (written by the build)
#include "jit_sources.inc"

namespace iso {
namespace {

// ----------------------------------------------------------------- NVRTC ---
struct Nvrtc {
    bool ok = false;
    std::string why;
    decltype(&nvrtcCreateProgram) create = nullptr;
    decltype(&nvrtcCompileProgram) compile = nullptr;
    decltype(&nvrtcGetCUBINSize) cubin_size = nullptr;
    decltype(&nvrtcGetCUBIN) cubin = nullptr;
    decltype(&nvrtcGetProgramLogSize) log_size = nullptr;
    decltype(&nvrtcGetProgramLog) log = nullptr;
    decltype(&nvrtcDestroyProgram) destroy = nullptr;
};

const Nvrtc& nvrtc() {
    static Nvrtc n;
    static std::once_flag once;
    std::call_once(once, [] {
        const char* names[] = {"libnvrtc.so.13", "libnvrtc.so", "/usr/local/cuda/lib64/libnvrtc.so.13",
                               "/usr/local/cuda/lib64/libnvrtc.so"};
        void* h = nullptr;
        for (const char* name : names)
            if ((h = dlopen(name, RTLD_NOW | RTLD_LOCAL)) != nullptr) break;
        if (!h) {
            n.why = "libnvrtc not found";
            return;
        }
        n.create = (decltype(n.create))dlsym(h, "nvrtcCreateProgram");
        n.compile = (decltype(n.compile))dlsym(h, "nvrtcCompileProgram");
        n.cubin_size = (decltype(n.cubin_size))dlsym(h, "nvrtcGetCUBINSize");
        n.cubin = (decltype(n.cubin))dlsym(h, "nvrtcGetCUBIN");
        n.log_size = (decltype(n.log_size))dlsym(h, "nvrtcGetProgramLogSize");
        n.log = (decltype(n.log))dlsym(h, "nvrtcGetProgramLog");
        n.destroy = (decltype(n.destroy))dlsym(h, "nvrtcDestroyProgram");
        n.ok = n.create && n.compile && n.cubin_size && n.cubin && n.log_size && n.log && n.destroy;
        if (!n.ok) n.why = "libnvrtc lacks an entry point";
    });
    return n;
}

// ------------------------------------------------------- code generation ---
std::string flit(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    char buf[48];
    std::snprintf(buf, sizeof(buf), "__int_as_float(0x%08" PRIx32 ")", u);
    return buf;
}

// The program's value at p as straight-line code, or false for a program
// the generator does not cover (sphere sets, which the interpreter loops).
bool emit_value(const iso_program* p, std::string* out) {
    std::string& s = *out;
    std::vector<std::string> points{"p"}, values;
    std::string q = "p";
    int np = 0, nv = 0;
    const float* K = p->consts.data();
    auto point = [&](const std::string& expr) {
        const std::string name = "pt" + std::to_string(++np);
        s += "        const V3 " + name + " = " + expr + ";\n";
        points.push_back(q);
        q = name;
    };
    auto value = [&](const std::string& expr) {
        const std::string name = "val" + std::to_string(++nv);
        s += "        const float " + name + " = " + expr + ";\n";
        values.push_back(name);
    };
    for (uint32_t w : p->ops) {
        const uint32_t op = w & 0xFFu;
        const float* k = K + (w >> 8);
        switch (op) {
        case OP_PT_DOMAIN:  // pt_apply: p * scale + offset per axis
            point("v3(" + q + ".x * " + flit(k[0]) + " + " + flit(k[3]) + ", " + q + ".y * " + flit(k[1]) + " + " +
                  flit(k[4]) + ", " + q + ".z * " + flit(k[2]) + " + " + flit(k[5]) + ")");
            break;
        case OP_PT_TRANSLATE:
            point("v3(" + q + ".x - " + flit(k[0]) + ", " + q + ".y - " + flit(k[1]) + ", " + q + ".z - " +
                  flit(k[2]) + ")");
            break;
        case OP_PT_RIGID: {  // pt_apply: d = p - t, then M d row by row, ((m0 dx + m1 dy) + m2 dz)
            const std::string d = "dif" + std::to_string(np + 1);
            s += "        const V3 " + d + " = v3(" + q + ".x - " + flit(k[0]) + ", " + q + ".y - " + flit(k[1]) +
                 ", " + q + ".z - " + flit(k[2]) + ");\n";
            const float* m = k + 3;
            auto row = [&](int r) {
                return "(" + flit(m[3 * r]) + " * " + d + ".x + " + flit(m[3 * r + 1]) + " * " + d + ".y) + " +
                       flit(m[3 * r + 2]) + " * " + d + ".z";
            };
            point("v3(" + row(0) + ", " + row(1) + ", " + row(2) + ")");
            break;
        }
        case OP_PT_POP:
            if (points.size() < 2) return false;
            q = points.back();
            points.pop_back();
            break;
        case OP_SPHERE: value("sd_sphere(" + q + ", " + flit(k[0]) + ")"); break;
        case OP_BOX: value("sd_box(" + q + ", " + flit(k[0]) + ", " + flit(k[1]) + ", " + flit(k[2]) + ")"); break;
        case OP_CYLINDER: value("sd_cylinder(" + q + ", " + flit(k[0]) + ", " + flit(k[1]) + ")"); break;
        case OP_TORUS: value("sd_torus(" + q + ", " + flit(k[0]) + ", " + flit(k[1]) + ")"); break;
        case OP_UNION: case OP_INTERSECTION: case OP_DIFFERENCE: case OP_SMOOTH_UNION: {
            // a = the entry below the top, b = the top (eval_range)
            if (values.size() < 2) return false;
            const std::string b = values.back();
            values.pop_back();
            const std::string a = values.back();
            values.pop_back();
            if (op == OP_UNION) value("fminf(" + a + ", " + b + ")");
            else if (op == OP_INTERSECTION) value("fmaxf(" + a + ", " + b + ")");
            else if (op == OP_DIFFERENCE) value("fmaxf(" + b + ", -" + a + ")");
            else value("smooth_min(" + a + ", " + b + ", " + flit(k[0]) + ")");
            break;
        }
        case OP_CD_BEGIN: case OP_CD_END: break;  // markers for values
        default: return false;                    // sphere sets and anything new
        }
    }
    if (values.size() != 1) return false;
    s += "        return " + values.back() + ";\n";
    return true;
}

// The program's normal at p (the Hermite evaluation of vm.cuh's
// eval_hermite: the same values, the same normal selections and rigid-map
// rotations, in the same order) as straight-line code, or false for a
// program the generator does not cover (sphere sets, central differences).
bool emit_hermite(const iso_program* p, std::string* out) {
    std::string& s = *out;
    struct Pt {
        std::string name;
        uint32_t op;
        const float* k;
    };
    std::vector<Pt> points{{"p", 0u, nullptr}};
    std::vector<std::pair<std::string, std::string>> vals;  // (value, normal)
    int np = 0, nv = 0;
    const float* K = p->consts.data();
    auto point = [&](const std::string& expr, uint32_t op, const float* k) {
        const std::string name = "hpt" + std::to_string(++np);
        s += "        const V3 " + name + " = " + expr + ";\n";
        points.push_back({name, op, k});
    };
    auto push = [&](const std::string& value, const std::string& normal) {
        const std::string id = std::to_string(++nv);
        s += "        const float hval" + id + " = " + value + ";\n";
        s += "        const V3 hnrm" + id + " = " + normal + ";\n";
        vals.push_back({"hval" + id, "hnrm" + id});
    };
    for (uint32_t w : p->ops) {
        const uint32_t op = w & 0xFFu;
        const float* k = K + (w >> 8);
        const std::string q = points.back().name;
        switch (op) {
        case OP_PT_DOMAIN:
            point("v3(" + q + ".x * " + flit(k[0]) + " + " + flit(k[3]) + ", " + q + ".y * " + flit(k[1]) + " + " +
                      flit(k[4]) + ", " + q + ".z * " + flit(k[2]) + " + " + flit(k[5]) + ")",
                  op, k);
            break;
        case OP_PT_TRANSLATE:
            point("v3(" + q + ".x - " + flit(k[0]) + ", " + q + ".y - " + flit(k[1]) + ", " + q + ".z - " +
                      flit(k[2]) + ")",
                  op, k);
            break;
        case OP_PT_RIGID: {
            const std::string d = "hdif" + std::to_string(np + 1);
            s += "        const V3 " + d + " = v3(" + q + ".x - " + flit(k[0]) + ", " + q + ".y - " + flit(k[1]) +
                 ", " + q + ".z - " + flit(k[2]) + ");\n";
            const float* m = k + 3;
            auto row = [&](int r) {
                return "(" + flit(m[3 * r]) + " * " + d + ".x + " + flit(m[3 * r + 1]) + " * " + d + ".y) + " +
                       flit(m[3 * r + 2]) + " * " + d + ".z";
            };
            point("v3(" + row(0) + ", " + row(1) + ", " + row(2) + ")", op, k);
            break;
        }
        case OP_PT_POP: {
            if (points.size() < 2) return false;
            const Pt top = points.back();
            points.pop_back();
            if (top.op == OP_PT_RIGID) {  // the normal rotated back: M^T n, column by column
                if (vals.empty()) return false;
                const float* m = top.k + 3;
                const std::string n = vals.back().second, r = "hrot" + std::to_string(++np);
                auto col = [&](int c) {
                    return "(" + flit(m[c]) + " * " + n + ".x + " + flit(m[c + 3]) + " * " + n + ".y) + " +
                           flit(m[c + 6]) + " * " + n + ".z";
                };
                s += "        const V3 " + r + " = v3(" + col(0) + ", " + col(1) + ", " + col(2) + ");\n";
                vals.back().second = r;
            }
            break;
        }
        case OP_SPHERE: push("sd_sphere(" + q + ", " + flit(k[0]) + ")", q); break;
        case OP_BOX:
            push("sd_box(" + q + ", " + flit(k[0]) + ", " + flit(k[1]) + ", " + flit(k[2]) + ")", "n_box(" + q + ")");
            break;
        case OP_CYLINDER:
            push("sd_cylinder(" + q + ", " + flit(k[0]) + ", " + flit(k[1]) + ")",
                 "n_cylinder(" + q + ", " + flit(k[0]) + ", " + flit(k[1]) + ")");
            break;
        case OP_TORUS:
            push("sd_torus(" + q + ", " + flit(k[0]) + ", " + flit(k[1]) + ")", "n_torus(" + q + ", " + flit(k[0]) + ")");
            break;
        case OP_UNION: case OP_INTERSECTION: case OP_DIFFERENCE: case OP_SMOOTH_UNION: {
            if (vals.size() < 2) return false;
            const auto b = vals.back();
            vals.pop_back();
            const auto a = vals.back();
            vals.pop_back();
            const std::string& va = a.first; const std::string& na = a.second;
            const std::string& vb = b.first; const std::string& nb = b.second;
            if (op == OP_UNION)
                push("fminf(" + va + ", " + vb + ")", "vmin(" + na + ", " + nb + ")");
            else if (op == OP_INTERSECTION)
                push("fmaxf(" + va + ", " + vb + ")", "(!(" + va + " >= " + vb + ")) ? " + nb + " : " + na);
            else if (op == OP_DIFFERENCE)
                push("fmaxf(" + vb + ", -" + va + ")",
                     "(" + vb + " >= -" + va + ") ? " + nb + " : v3(-" + na + ".x, -" + na + ".y, -" + na + ".z)");
            else
                push("smooth_min(" + va + ", " + vb + ", " + flit(k[0]) + ")",
                     "(!(" + va + " <= " + vb + ")) ? " + nb + " : " + na);
            break;
        }
        default: return false;  // sphere sets, central differences and anything new
        }
    }
    if (vals.size() != 1) return false;
    s += "        return " + vals.back().second + ";\n";
    return true;
}

std::string module_source(const std::string& value_body, const std::string& hermite_body) {
    std::string s;
    s += "typedef unsigned char uint8_t;\ntypedef unsigned int uint32_t;\ntypedef unsigned long long uint64_t;\n";
    s += kJitVmMath;
    s += kJitBricksCore;
    if (!hermite_body.empty()) {
        s += kJitQefPlanes;
        s += kJitDcCore;
    }
    s += "namespace iso {\nstruct JitEval {\n"
         "    __device__ __forceinline__ float value(V3 p) const {\n";
    s += value_body;
    s += "    }\n"
         "    __device__ __forceinline__ bool prunable() const { return false; }\n"
         "    __device__ __forceinline__ uint32_t nprims() const { return 0; }\n"
         "    __device__ __forceinline__ V3 point(V3 p) const { return p; }\n"
         "    __device__ __forceinline__ float prim(uint32_t, V3) const { return 0.0f; }\n"
         "    __device__ __forceinline__ float value_kept(uint64_t, V3 p) const { return value(p); }\n"
         "};\n}  // namespace iso\n"
         "extern \"C\" __global__ void __launch_bounds__(256) iso_jit_classify(iso::GridTiles tiles, "
         "iso::BrickTask* list, uint32_t* count, uint32_t cap, uint32_t* err) {\n"
         "    iso::brick_classify_body(iso::JitEval{}, tiles, list, count, cap, err);\n}\n"
         "extern \"C\" __global__ void __launch_bounds__(256) iso_jit_rows(iso::GridTiles tiles, "
         "const iso::BrickTask* list, const uint32_t* count, uint32_t cap) {\n"
         "    iso::brick_rows_body(iso::JitEval{}, tiles, list, count, cap);\n}\n"
         "extern \"C\" __global__ void __launch_bounds__(256) iso_jit_field(iso::BrickLattice g) {\n"
         "    iso::field_warp(iso::JitEval{}, g, (uint64_t)blockIdx.x * 8 + (threadIdx.x >> 5));\n}\n";
    if (!hermite_body.empty()) {
        s += "namespace iso {\nstruct JitHermite {\n"
             "    __device__ __forceinline__ V3 normal(V3 p) const {\n";
        s += hermite_body;
        s += "    }\n};\n}  // namespace iso\n"
             "extern \"C\" __global__ void __launch_bounds__(128) iso_jit_dc_place(iso::DcCells cells) {\n"
             "    iso::dc_place_body(iso::JitHermite{}, cells);\n}\n";
    }
    return s;
}

// ------------------------------------------------------------------ cache ---
struct Module {
    std::vector<uint32_t> ops;
    std::vector<float> consts;
    bool ok = false;
    cudaLibrary_t lib = nullptr;
    cudaKernel_t classify = nullptr, rows = nullptr, field = nullptr;
    cudaKernel_t dc_place = nullptr;  // only for a program whose normals are compiled too
    std::atomic<int> rows_per_sm{0};
};

std::mutex g_jit_mutex;
std::unordered_multimap<uint64_t, std::unique_ptr<Module>> g_modules;
std::atomic<int> g_jit_enabled{1};
std::atomic<uint64_t> g_jit_compiles{0};

Module* compile_module(const iso_program* p, std::string* why) {
    std::string body;
    if (!emit_value(p, &body)) {
        *why = "program form not compiled";
        return nullptr;
    }
    const Nvrtc& n = nvrtc();
    if (!n.ok) {
        *why = n.why;
        return nullptr;
    }
    std::string hermite;
    if (!emit_hermite(p, &hermite)) hermite.clear();
    const std::string src = module_source(body, hermite);
    nvrtcProgram prog = nullptr;
    if (n.create(&prog, src.c_str(), "iso_program.cu", 0, nullptr, nullptr) != NVRTC_SUCCESS) {
        *why = "nvrtcCreateProgram failed";
        return nullptr;
    }
    int major = 0, minor = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    const std::string arch = "--gpu-architecture=sm_" + std::to_string(major) + std::to_string(minor) + "a";
    const char* opts[] = {arch.c_str(), "--fmad=false", "--std=c++17", "-default-device"};
    const nvrtcResult cr = n.compile(prog, 4, opts);
    std::vector<char> cubin;
    if (cr == NVRTC_SUCCESS) {
        size_t bytes = 0;
        if (n.cubin_size(prog, &bytes) == NVRTC_SUCCESS && bytes) {
            cubin.resize(bytes);
            if (n.cubin(prog, cubin.data()) != NVRTC_SUCCESS) cubin.clear();
        }
    } else {
        size_t bytes = 0;
        n.log_size(prog, &bytes);
        std::string log(bytes, '\0');
        if (bytes) n.log(prog, &log[0]);
        *why = "nvrtc: " + log.substr(0, 400);
    }
    n.destroy(&prog);
    if (cubin.empty()) {
        if (why->empty()) *why = "no cubin";
        return nullptr;
    }
    std::unique_ptr<Module> m(new Module());
    cudaError_t e = cudaLibraryLoadData(&m->lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&m->classify, m->lib, "iso_jit_classify");
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&m->rows, m->lib, "iso_jit_rows");
    if (e == cudaSuccess) e = cudaLibraryGetKernel(&m->field, m->lib, "iso_jit_field");
    if (e == cudaSuccess && !hermite.empty()) e = cudaLibraryGetKernel(&m->dc_place, m->lib, "iso_jit_dc_place");
    if (e != cudaSuccess) {
        cudaGetLastError();
        if (m->lib) cudaLibraryUnload(m->lib);
        *why = std::string("module load: ") + cudaGetErrorString(e);
        return nullptr;
    }
    m->ok = true;
    g_jit_compiles.fetch_add(1);
    return m.release();
}

// The compiled module of a program (compiled on first use), or null.
Module* module_for(const iso_program* p) {
    if (!g_jit_enabled.load() || p->kind != PK_GENERIC) return nullptr;
    std::lock_guard<std::mutex> lock(g_jit_mutex);
    auto range = g_modules.equal_range(p->content_hash);
    for (auto it = range.first; it != range.second; ++it) {
        Module* m = it->second.get();
        if (m->ops == p->ops && m->consts.size() == p->consts.size() &&
            std::memcmp(m->consts.data(), p->consts.data(), 4 * p->consts.size()) == 0)
            return m->ok ? m : nullptr;
    }
    std::string why;
    Module* m = compile_module(p, &why);
    if (!m) m = new Module();  // remembered as not compiled
    m->ops = p->ops;
    m->consts = p->consts;
    g_modules.emplace(p->content_hash, std::unique_ptr<Module>(m));
    return m->ok ? m : nullptr;
}

}  // namespace

// The culled sampler with the program's compiled evaluator: false (nothing
// launched) when the program has none, so the caller runs the interpreter.
bool jit_sample_bricks(iso_ctx* ctx, const iso_program* prog, const GridTiles& tiles, uint32_t ntiles,
                       BrickTask* list, uint32_t* count, uint32_t cap, cudaError_t* err) {
    // a flat union of translated primitives stays with the interpreter,
    // which prunes the primitives per sub-brick
    if (!prog->prims.empty()) return false;
    Module* m = module_for(prog);
    if (!m) return false;
    static_assert(sizeof(GridTiles) % 8 == 0, "kernel argument layout");
    GridTiles t = tiles;
    uint32_t c = cap;
    uint32_t* derr = ctx->d_err;
    void* a1[] = {&t, &list, &count, &c, &derr};
    cudaError_t e = cudaLaunchKernel((const void*)m->classify, dim3(ntiles), dim3(256), a1, 0, ctx->stream);
    if (e == cudaSuccess) {
        const BrickTask* clist = list;
        const uint32_t* ccount = count;
        void* a2[] = {&t, &clist, &ccount, &c};
        const unsigned blocks = persistent_blocks((const void*)m->rows, m->rows_per_sm, ctx->sms);
        e = cudaLaunchKernel((const void*)m->rows, dim3(blocks), dim3(256), a2, 0, ctx->stream);
    }
    *err = e;
    return true;
}

bool jit_dc_place(iso_ctx* ctx, const iso_program* prog, const DcCells& cells, uint64_t blocks, cudaError_t* err) {
    Module* m = module_for(prog);
    if (!m || !m->dc_place) return false;
    DcCells a = cells;
    void* args[] = {&a};
    *err = cudaLaunchKernel((const void*)m->dc_place, dim3((unsigned)blocks), dim3(128), args, 0, ctx->stream);
    return true;
}

bool jit_sample_field(iso_ctx* ctx, const iso_program* prog, const BrickLattice& g, uint64_t blocks,
                      cudaError_t* err) {
    Module* m = module_for(prog);
    if (!m) return false;
    static_assert(sizeof(BrickLattice) % 8 == 0, "kernel argument layout");
    BrickLattice a = g;
    void* args[] = {&a};
    *err = cudaLaunchKernel((const void*)m->field, dim3((unsigned)blocks), dim3(256), args, 0, ctx->stream);
    return true;
}

}  // namespace iso

namespace iso {
// bumped whenever compilation is switched on or off: recorded extractions
// hold the kernels of the setting they were recorded with
std::atomic<uint64_t> g_jit_generation{0};
uint64_t jit_generation() { return g_jit_generation.load(); }
}  // namespace iso

extern "C" iso_status iso_jit_enable(int enable) {
    if (iso::g_jit_enabled.exchange(enable ? 1 : 0) != (enable ? 1 : 0)) iso::g_jit_generation.fetch_add(1);
    return ISO_OK;
}

extern "C" iso_status iso_program_source(const uint8_t* bytes, size_t len, char* out, size_t cap, size_t* needed) {
    if (!bytes || !needed) return ISO_ERR_INVALID_ARG;
    *needed = 0;
    iso_program p;
    std::string err;
    iso_status s = iso::parse_program(bytes, len, &p, &err);
    if (s != ISO_OK) return s;
    std::string body;
    if (p.kind != iso::PK_GENERIC || !iso::emit_value(&p, &body)) return ISO_ERR_UNSUPPORTED;
    std::string hermite;
    if (!iso::emit_hermite(&p, &hermite)) hermite.clear();
    const std::string src = iso::module_source(body, hermite);
    *needed = src.size() + 1;
    if (!out) return ISO_OK;
    if (cap < src.size() + 1) return ISO_ERR_CAPACITY;
    std::memcpy(out, src.c_str(), src.size() + 1);
    return ISO_OK;
}

extern "C" iso_status iso_program_compiled(const iso_program* prog, int* compiled) {
    if (!prog || !compiled) return ISO_ERR_INVALID_ARG;
    // the extractors' sampler of a flat union of primitives is the
    // interpreter's pruned one, compiled module or not
    *compiled = prog->prims.empty() && iso::module_for(prog) != nullptr ? 1 : 0;
    return ISO_OK;
}
