// The f32 arithmetic of the source primitives and operators, shared by the
// library's evaluator (vm.cuh) and by the kernels the library compiles at
// run time for one program (jit.cu): no includes, so that it compiles as is
// under NVRTC.
//
// The operation order restates the reference's exactly
// (src/math/vector.rs len_sq = (x*x + y*y) + z*z, src/implicit/*.rs); every
// translation unit that uses it is built with -fmad=false (no a*b+c fusion),
// so values are bit-identical to the reference's f32 evaluation.
#pragma once

namespace iso {

struct V3 {
    float x, y, z;
};

__host__ __device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__host__ __device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ V3 operator*(V3 a, float f) { return v3(a.x * f, a.y * f, a.z * f); }
__host__ __device__ __forceinline__ float len_sq(V3 a) { return (a.x * a.x + a.y * a.y) + a.z * a.z; }
__host__ __device__ __forceinline__ float vlen(V3 a) { return sqrtf(len_sq(a)); }
__host__ __device__ __forceinline__ V3 vmin(V3 a, V3 b) { return v3(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z)); }

// primitives: sphere.rs:35-63, rectangular_prism.rs:36-80, cylinder.rs:41-85, torus.rs:40-108
__host__ __device__ __forceinline__ float sd_sphere(V3 q, float r) { return vlen(q) - r; }
__host__ __device__ __forceinline__ float sd_box(V3 q, float hx, float hy, float hz) {
    float ax = fabsf(q.x) - hx, ay = fabsf(q.y) - hy, az = fabsf(q.z) - hz;
    float l = vlen(v3(fmaxf(ax, 0.0f), fmaxf(ay, 0.0f), fmaxf(az, 0.0f)));
    return l + fminf(fmaxf(ax, fmaxf(ay, az)), 0.0f);
}
__host__ __device__ __forceinline__ float sd_cylinder(V3 q, float r, float hl) {
    float qx = fabsf(sqrtf(q.x * q.x + q.y * q.y)) - r;
    float qz = fabsf(q.z) - hl;
    float dx = fmaxf(qx, 0.0f), dz = fmaxf(qz, 0.0f);
    float l = sqrtf((dx * dx + dz * dz) + 0.0f * 0.0f);
    return fminf(fmaxf(qx, qz), 0.0f) + l;
}
__host__ __device__ __forceinline__ float sd_torus(V3 q, float R, float r) {
    float qx = fabsf(sqrtf(q.x * q.x + q.y * q.y)) - R;
    float l = sqrtf(qx * qx + q.z * q.z);
    return l - r;
}
// the primitives' analytic normals, unnormalised (sample_normal:
// rectangular_prism.rs:77 with vector.rs:612-621, cylinder.rs:75, torus.rs:99;
// a sphere's is the point itself, sphere.rs:60)
__host__ __device__ __forceinline__ V3 n_box(V3 p) {  // vector.rs:612-621
    float ax = fabsf(p.x), ay = fabsf(p.y), az = fabsf(p.z);
    if (ax > ay && ax > az) return v3(p.x, 0.0f, 0.0f);
    if (ay > az) return v3(0.0f, p.y, 0.0f);
    return v3(0.0f, 0.0f, p.z);
}
__host__ __device__ __forceinline__ V3 n_cylinder(V3 p, float r, float hl) {
    float z = fabsf(p.z) / hl;
    float rr = sqrtf(p.x * p.x + p.y * p.y) / r;
    if (z > rr) return v3(0.0f, 0.0f, p.z);
    return v3(p.x, p.y, 0.0f);
}
__host__ __device__ __forceinline__ V3 n_torus(V3 p, float R) {
    float l = sqrtf((p.x * p.x + p.y * p.y) + 0.0f * 0.0f);
    V3 ring;
    if (fabsf(l) < 1.1920929e-07f) ring = v3(1.0f, 0.0f, 0.0f);
    else ring = v3(p.x / l, p.y / l, 0.0f / l);
    return p - ring * R;
}

// Polynomial smooth minimum (Quilez 2013)
__host__ __device__ __forceinline__ float smooth_min(float a, float b, float k) {
    const float gap = k - fabsf(a - b);
    // with k > 0 and no overlap, h is +0 and the formula gives min(a, b) - 0
    // exactly (also for -0 and NaN operands): skip the division
    if (k > 0.0f && !(gap > 0.0f)) return fminf(a, b);
    float h = fmaxf(gap, 0.0f) / k;
    return fminf(a, b) - ((h * h) * k) * 0.25f;
}

}  // namespace iso
