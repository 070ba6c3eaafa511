// Device evaluator of source programs (format: include/isosurface_gpu.h).
//
// The arithmetic restates the reference's f32 operation order exactly
// (src/math/vector.rs len_sq = (x*x + y*y) + z*z, src/implicit/*.rs), and the
// translation units that include this header are built with -fmad=false so
// that no a*b+c is fused: corner values are bit-identical to the reference's,
// which keeps cube classification bit-exact.
#pragma once
#include <cuda_runtime.h>
#include <string.h>

#include "internal.h"
#include "vm_math.cuh"

namespace iso {

enum : uint32_t {
    OP_PT_DOMAIN = 0x01, OP_PT_TRANSLATE = 0x02, OP_PT_RIGID = 0x03, OP_PT_POP = 0x04,
    OP_SPHERE = 0x10, OP_BOX = 0x11, OP_CYLINDER = 0x12, OP_TORUS = 0x13,
    OP_UNION = 0x20, OP_INTERSECTION = 0x21, OP_DIFFERENCE = 0x22, OP_SMOOTH_UNION = 0x23,
    OP_SPHERE_SET = 0x30, OP_CD_BEGIN = 0x40, OP_CD_END = 0x41,
};

// Read-only loads: through the non-coherent cache on the device, plain on
// the host (the evaluator also compiles for host code that checks it).
template <class T>
__host__ __device__ __forceinline__ T ld_ro(const T* p) {
#ifdef __CUDA_ARCH__
    return __ldg(p);
#else
    return *p;
#endif
}
__host__ __device__ __forceinline__ uint32_t float_bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    uint32_t u;
    memcpy(&u, &f, sizeof(u));
    return u;
#endif
}

__host__ __device__ __forceinline__ V3 pt_apply(uint32_t op, const float* k, V3 p) {
    if (op == OP_PT_DOMAIN) return v3(p.x * k[0] + k[3], p.y * k[1] + k[4], p.z * k[2] + k[5]);
    if (op == OP_PT_TRANSLATE) return v3(p.x - k[0], p.y - k[1], p.z - k[2]);
    V3 d = v3(p.x - k[0], p.y - k[1], p.z - k[2]);
    const float* m = k + 3;
    return v3((m[0] * d.x + m[1] * d.y) + m[2] * d.z, (m[3] * d.x + m[4] * d.y) + m[5] * d.z,
              (m[6] * d.x + m[7] * d.y) + m[8] * d.z);
}

// Scalar evaluation of ops[begin, end) at p (one value left on the stack).
// The top value and the current point live in registers; only the entries
// below them are kept in (local-memory) stacks, so a primitive, a binary
// operator and a point op each touch memory at most once.
static __host__ __device__ __noinline__ float eval_range(const ProgView& pv, uint32_t begin, uint32_t end, V3 p) {
    float vs[VSTACK];  // values below the top: vs[0 .. vsp-2]
    V3 ps[PSTACK];     // points below the current one: ps[0 .. psp-1]
    float tos = 0.0f;  // top value (vsp > 0)
    V3 q = p;          // current point
    int vsp = 0, psp = 0;
    auto push = [&](float x) {
        if (vsp > 0) vs[vsp - 1] = tos;
        tos = x;
        ++vsp;
    };
    for (uint32_t pc = begin; pc < end; ++pc) {
        const uint32_t w = ld_ro(pv.ops + pc);
        const uint32_t op = w & 0xFFu;
        const float* k = pv.k + (w >> 8);
        switch (op) {
        case OP_PT_DOMAIN: case OP_PT_TRANSLATE: case OP_PT_RIGID:
            ps[psp++] = q;
            q = pt_apply(op, k, q);
            break;
        case OP_PT_POP: q = ps[--psp]; break;
        case OP_SPHERE: push(sd_sphere(q, k[0])); break;
        case OP_BOX: push(sd_box(q, k[0], k[1], k[2])); break;
        case OP_CYLINDER: push(sd_cylinder(q, k[0], k[1])); break;
        case OP_TORUS: push(sd_torus(q, k[0], k[1])); break;
        // binary operators: a = the entry below the top, b = the top
        case OP_UNION: tos = fminf(vs[vsp - 2], tos); --vsp; break;
        case OP_INTERSECTION: tos = fmaxf(vs[vsp - 2], tos); --vsp; break;
        case OP_DIFFERENCE: tos = fmaxf(tos, -vs[vsp - 2]); --vsp; break;
        case OP_SMOOTH_UNION: tos = smooth_min(vs[vsp - 2], tos, k[0]); --vsp; break;
        case OP_SPHERE_SET: {
            uint32_t n = (uint32_t)k[0];
            bool smooth = k[1] != 0.0f;
            float kk = k[2];
            float v = 0.0f;
            for (uint32_t i = 0; i < n; ++i) {
                const float* c = k + 3 + 4 * i;
                float d = vlen(v3(q.x - c[0], q.y - c[1], q.z - c[2])) - c[3];
                v = (i == 0) ? d : (smooth ? smooth_min(v, d, kk) : fminf(v, d));
            }
            push(v);
            break;
        }
        default: break;  // CD_BEGIN / CD_END are markers in scalar mode
        }
    }
    return tos;
}

// Primitive i of ProgView::prims at q (a point after the leading domain map):
// the translate and primitive operations of its ops.
__host__ __device__ __forceinline__ float prim_at(const ProgView& pv, uint32_t i, V3 q) {
    const float4 c = ld_ro(pv.prims + 2 * i), a = ld_ro(pv.prims + 2 * i + 1);
    const V3 t = v3(q.x - c.x, q.y - c.y, q.z - c.z);
    const uint32_t type = float_bits(c.w);
    if (type == OP_SPHERE) return sd_sphere(t, a.x);
    if (type == OP_BOX) return sd_box(t, a.x, a.y, a.z);
    if (type == OP_CYLINDER) return sd_cylinder(t, a.x, a.y);
    return sd_torus(t, a.x, a.y);
}

__host__ __device__ __forceinline__ V3 prims_point(const ProgView& pv, V3 p) {
    return pv.dom_at >= 0 ? pt_apply(OP_PT_DOMAIN, pv.k + pv.dom_at, p) : p;
}

// A hard union of translated primitives (ProgView::prims): the same
// translate, primitive and fminf operations as the ops, in the same order.
static __host__ __device__ __noinline__ float eval_prims(const ProgView& pv, V3 p) {
    const V3 q = prims_point(pv, p);
    float v = 0.0f;
    for (uint32_t i = 0; i < pv.nprims; ++i) {
        const float d = prim_at(pv, i, q);
        v = (i == 0) ? d : fminf(v, d);
    }
    return v;
}

// The same union over the primitives whose bits are set in `keep` (nonzero;
// at most 64 primitives), in the same order.  Equal to eval_prims wherever
// every dropped primitive's value exceeds some kept one's: fminf returns one
// of its operands, so the minimum over a subset that holds the minimiser is
// the minimum over all.
__host__ __device__ __forceinline__ uint32_t lowest_bit(uint64_t m) {
#ifdef __CUDA_ARCH__
    return (uint32_t)(__ffsll((long long)m) - 1);
#else
    return (uint32_t)__builtin_ctzll(m);
#endif
}
static __host__ __device__ __noinline__ float eval_prims_kept(const ProgView& pv, uint64_t keep, V3 p) {
    const V3 q = prims_point(pv, p);
    float v = prim_at(pv, lowest_bit(keep), q);
    for (keep &= keep - 1; keep; keep &= keep - 1) v = fminf(v, prim_at(pv, lowest_bit(keep), q));
    return v;
}

__host__ __device__ __forceinline__ float eval_scalar(const ProgView& pv, V3 p) {
    return pv.prims ? eval_prims(pv, p) : eval_range(pv, 0, pv.n_ops, p);
}

// Value and (unnormalised) normal: HermiteSource::sample_normal semantics.
static __host__ __device__ __noinline__ float eval_hermite(const ProgView& pv, V3 p, V3* normal) {
    float vs[VSTACK];
    V3 ns[VSTACK];
    V3 ps[PSTACK];
    uint32_t pop_op[PSTACK];
    const float* pop_k[PSTACK];
    int vsp = 0, psp = 0;
    ps[0] = p;
    for (uint32_t pc = 0; pc < pv.n_ops; ++pc) {
        uint32_t w = pv.ops[pc];
        uint32_t op = w & 0xFFu;
        const float* k = pv.k + (w >> 8);
        V3 q = ps[psp];
        switch (op) {
        case OP_PT_DOMAIN: case OP_PT_TRANSLATE: case OP_PT_RIGID:
            ps[++psp] = pt_apply(op, k, q);
            pop_op[psp] = op;
            pop_k[psp] = k;
            break;
        case OP_PT_POP:
            if (pop_op[psp] == OP_PT_RIGID) {
                const float* m = pop_k[psp] + 3;
                V3 n = ns[vsp - 1];
                ns[vsp - 1] = v3((m[0] * n.x + m[3] * n.y) + m[6] * n.z, (m[1] * n.x + m[4] * n.y) + m[7] * n.z,
                                 (m[2] * n.x + m[5] * n.y) + m[8] * n.z);
            }
            --psp;
            break;
        case OP_SPHERE: vs[vsp] = sd_sphere(q, k[0]); ns[vsp++] = q; break;
        case OP_BOX: vs[vsp] = sd_box(q, k[0], k[1], k[2]); ns[vsp++] = n_box(q); break;
        case OP_CYLINDER: vs[vsp] = sd_cylinder(q, k[0], k[1]); ns[vsp++] = n_cylinder(q, k[0], k[1]); break;
        case OP_TORUS: vs[vsp] = sd_torus(q, k[0], k[1]); ns[vsp++] = n_torus(q, k[0]); break;
        case OP_UNION:
            --vsp;
            vs[vsp - 1] = fminf(vs[vsp - 1], vs[vsp]);
            ns[vsp - 1] = vmin(ns[vsp - 1], ns[vsp]);
            break;
        case OP_INTERSECTION: {
            --vsp;
            float a = vs[vsp - 1], b = vs[vsp];
            vs[vsp - 1] = fmaxf(a, b);
            if (!(a >= b)) ns[vsp - 1] = ns[vsp];
            break;
        }
        case OP_DIFFERENCE: {
            --vsp;
            float a = vs[vsp - 1], b = vs[vsp];
            vs[vsp - 1] = fmaxf(b, -a);
            V3 na = ns[vsp - 1];
            ns[vsp - 1] = (b >= -a) ? ns[vsp] : v3(-na.x, -na.y, -na.z);
            break;
        }
        case OP_SMOOTH_UNION: {
            --vsp;
            float a = vs[vsp - 1], b = vs[vsp];
            vs[vsp - 1] = smooth_min(a, b, k[0]);
            if (!(a <= b)) ns[vsp - 1] = ns[vsp];
            break;
        }
        case OP_SPHERE_SET: {
            uint32_t n = (uint32_t)k[0];
            bool smooth = k[1] != 0.0f;
            float kk = k[2];
            float v = 0.0f;
            V3 nn = v3(0.0f, 0.0f, 0.0f);
            for (uint32_t i = 0; i < n; ++i) {
                V3 c = v3(k[3 + 4 * i], k[4 + 4 * i], k[5 + 4 * i]);
                V3 d3 = q - c;
                float d = vlen(d3) - k[6 + 4 * i];
                if (i == 0) {
                    v = d;
                    nn = d3;
                } else if (smooth) {
                    if (!(v <= d)) nn = d3;
                    v = smooth_min(v, d, kk);
                } else {
                    v = fminf(v, d);
                    nn = vmin(nn, d3);
                }
            }
            vs[vsp] = v;
            ns[vsp++] = nn;
            break;
        }
        case OP_CD_BEGIN: {
            // source.rs:52-95: (f(q+e) - f(q-e)) / (2 eps) per axis
            uint32_t end = (uint32_t)pv.jump[pc];
            float eps = k[0];
            float v = eval_range(pv, pc + 1, end, q);
            float vx = eval_range(pv, pc + 1, end, v3(q.x + eps, q.y + 0.0f, q.z + 0.0f)) -
                       eval_range(pv, pc + 1, end, v3(q.x - eps, q.y - 0.0f, q.z - 0.0f));
            float vy = eval_range(pv, pc + 1, end, v3(q.x + 0.0f, q.y + eps, q.z + 0.0f)) -
                       eval_range(pv, pc + 1, end, v3(q.x - 0.0f, q.y - eps, q.z - 0.0f));
            float vz = eval_range(pv, pc + 1, end, v3(q.x + 0.0f, q.y + 0.0f, q.z + eps)) -
                       eval_range(pv, pc + 1, end, v3(q.x - 0.0f, q.y - 0.0f, q.z - eps));
            float e2 = 2.0f * eps;
            vs[vsp] = v;
            ns[vsp++] = v3(vx / e2, vy / e2, vz / e2);
            pc = end;  // loop increment skips the CD_END
            break;
        }
        default: break;
        }
    }
    *normal = ns[0];
    return vs[0];
}

}  // namespace iso
