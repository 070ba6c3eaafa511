// The f32 half of feature placement (src/feature/mod.rs, particle_minimisation.rs):
// the vector helpers, TangentPlanes::new over the 8 cell corners
// (mod.rs:91-148) and ParticleBasedMinimisation (particle_minimisation.rs:25-72).
// No includes, so that the kernels the library compiles at run time for one
// program (jit.cu) take it as is; qef.cuh adds the f64 SVD of MinimiseQEF.
// Every translation unit that uses it is built with -fmad=false.
#pragma once

namespace iso {
namespace qef {

struct F3 {
    float x, y, z;
};
__host__ __device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__host__ __device__ __forceinline__ F3 add(F3 a, F3 b) { return f3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ F3 sub(F3 a, F3 b) { return f3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ F3 mul(F3 a, float f) { return f3(a.x * f, a.y * f, a.z * f); }
__host__ __device__ __forceinline__ F3 mulf(float f, F3 a) { return f3(f * a.x, f * a.y, f * a.z); }
// dot == (a*b).component_sum() == (x + y) + z
__host__ __device__ __forceinline__ float dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__host__ __device__ __forceinline__ F3 cross(F3 a, F3 r) {
    return f3(a.y * r.z - a.z * r.y, a.z * r.x - a.x * r.z, a.x * r.y - a.y * r.x);
}
__host__ __device__ __forceinline__ F3 normalised_or_zero(F3 v) {
    const float l = sqrtf((v.x * v.x + v.y * v.y) + v.z * v.z);
    if (fabsf(l) < 1.1920929e-07f) return f3(0.0f, 0.0f, 0.0f);
    return f3(v.x / l, v.y / l, v.z / l);
}

constexpr float FEATURE_ANGLE = 0.8660254037844387f;  // cos(30 degrees), feature/mod.rs:22
enum Topology { PLANAR = 0, EDGE = 1, CORNER = 2 };

struct Planes {
    F3 normal[8];
    float d[8];
    F3 com;
    int feature;
};

__host__ __device__ inline void tangent_planes(const F3* vtx, const F3* nrm, Planes* t) {
    F3 com = f3(0.0f, 0.0f, 0.0f), axis = f3(0.0f, 0.0f, 0.0f);
    float min_angle = 3.40282347e+38f;
    float count = 0.0f;
    for (int i = 0; i < 8; ++i) {
        for (int j = 0; j < 8; ++j) {
            const float angle = dot(nrm[i], nrm[j]);
            if (angle < min_angle) {
                axis = cross(nrm[i], nrm[j]);
                min_angle = angle;
            }
        }
        com = add(com, vtx[i]);
        count += 1.0f;
    }
    com = f3(com.x / count, com.y / count, com.z / count);
    int feature;
    if (min_angle > FEATURE_ANGLE) {
        feature = PLANAR;
    } else {
        axis = normalised_or_zero(axis);
        float min_c = 1.0f, max_c = -1.0f;
        for (int i = 0; i < 8; ++i) {
            const float c = dot(axis, nrm[i]);
            min_c = fminf(min_c, c);
            max_c = fmaxf(max_c, c);
        }
        float c = fmaxf(fabsf(min_c), fabsf(max_c));
        c = sqrtf(1.0f - c * c);
        feature = (c > FEATURE_ANGLE) ? EDGE : CORNER;
    }
    for (int i = 0; i < 8; ++i) {
        t->normal[i] = nrm[i];
        t->d[i] = dot(sub(vtx[i], com), nrm[i]);
    }
    t->com = com;
    t->feature = feature;
}

__host__ __device__ inline F3 trilinear(const F3* c, const F3* f, F3 p) {
    const F3 den = sub(f3(c[1].x, c[3].y, c[4].z), c[0]);
    const F3 num = sub(p, c[0]);
    const F3 g = f3(num.x / den.x, num.y / den.y, num.z / den.z);
    const F3 c00 = add(mulf(1.0f - g.x, f[0]), mulf(g.x, f[1]));
    const F3 c01 = add(mulf(1.0f - g.x, f[4]), mulf(g.x, f[5]));
    const F3 c10 = add(mulf(1.0f - g.x, f[3]), mulf(g.x, f[2]));
    const F3 c11 = add(mulf(1.0f - g.x, f[7]), mulf(g.x, f[6]));
    const F3 c0 = add(mulf(1.0f - g.y, c00), mulf(g.y, c10));
    const F3 c1 = add(mulf(1.0f - g.y, c01), mulf(g.y, c11));
    return add(mulf(1.0f - g.z, c0), mulf(g.z, c1));
}

__host__ __device__ inline F3 particle_placement(const F3* corners, const F3* normals) {
    const float STEP_SIZE = 0.05f, THRESHOLD = 0.02f;
    Planes t;
    tangent_planes(corners, normals, &t);
    const float max_feature_size = corners[6].x - corners[0].x;
    F3 particle = t.com;
    F3 forces[8];
    for (int i = 0; i < 8; ++i) {
        F3 acc = f3(0.0f, 0.0f, 0.0f);
        for (int j = 0; j < 8; ++j) {
            const float dist = dot(t.normal[j], corners[i]) - t.d[j];   // Plane::distance
            const F3 closest = sub(corners[i], mul(t.normal[j], dist));  // point_closest_to
            acc = add(acc, sub(corners[i], closest));
        }
        forces[i] = acc;
    }
    for (int it = 0; it < 100; ++it) {
        const F3 force = mul(mul(trilinear(corners, forces, particle), STEP_SIZE), max_feature_size);
        particle = add(particle, force);
        if ((force.x * force.x + force.y * force.y) + force.z * force.z < THRESHOLD * max_feature_size) break;
    }
    return particle;
}

}  // namespace qef
}  // namespace iso
