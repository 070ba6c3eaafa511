// DualContouring's placement of one dual vertex per active primal cell
// (src/dual_contouring.rs:78-87 with src/feature/*.rs), the f32 part: the
// cell's corners and normalised normals (sample_normals_at_corners,
// marching_cubes_impl.rs:58-69), TangentPlanes, the centre of mass of a
// planar cell and ParticleBasedMinimisation; MinimiseQEF of the non-planar
// cells (its f64 SVD) is listed for a kernel of its own.  Written so that it
// also compiles on its own under NVRTC (no includes: the library includes it
// after vm_math.cuh and qef_planes.cuh, the run-time compiler after the same
// texts).  The evaluator `Ev` provides normal(p), the program's unnormalised
// normal at p.
#pragma once

namespace iso {

struct alignas(16) DcPos {
    float x, y, z, w;
};

struct DcCells {
    uint32_t n;             // primal size: n x n x (n+1) samples
    uint32_t zoff;          // primal cell layer of dual layer 0 (a slab of the whole lattice)
    float inv;
    const uint32_t* list;   // active primal cells (linear dual index)
    const uint32_t* count;
    DcPos* dpos;            // placed positions, by dual index
    int placer;             // 0 MinimiseQEF, 1 ParticleBasedMinimisation
    uint32_t* features;     // MinimiseQEF: the non-planar cells, for the f64 QEF
    uint32_t* nfeatures;
    qef::F3* fnormals;      // the first fcap listed cells' 8 normalised normals, in list order
    uint32_t fcap;
};

// the corners of dual vertex `id`'s primal cell and their normalised normals
template <class Ev>
__device__ __forceinline__ void dc_cell_normals(const Ev& ev, const DcCells& A, uint32_t id, qef::F3* corners,
                                                qef::F3* normals) {
    const uint32_t m = A.n - 1;
    const uint32_t x = id % m, r = id / m;
    const uint32_t y = r % m, z = r / m;
    const uint8_t cornr[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
    for (int k = 0; k < 8; ++k) {
        const float px = (float)(x + cornr[k][0]) * A.inv, py = (float)(y + cornr[k][1]) * A.inv,
                    pz = (float)(z + A.zoff + cornr[k][2]) * A.inv;
        corners[k] = qef::f3(px, py, pz);
        const V3 nn = ev.normal(v3(px, py, pz));
        normals[k] = qef::normalised_or_zero(qef::f3(nn.x, nn.y, nn.z));
    }
}

// dual vertex `id`: placed here, or (a non-planar cell under MinimiseQEF)
// listed for the QEF kernel
template <class Ev>
__device__ __forceinline__ void dc_place_one(const Ev& ev, const DcCells& A, uint32_t id) {
    qef::F3 corners[8], normals[8];
    dc_cell_normals(ev, A, id, corners, normals);
    qef::F3 p;
    if (A.placer == 0) {
        qef::Planes t;
        qef::tangent_planes(corners, normals, &t);
        if (t.feature != qef::PLANAR) {
            const uint32_t j = atomicAdd(A.nfeatures, 1u);
            A.features[j] = id;
            if (j < A.fcap)  // kept for the QEF kernel, which then need not evaluate them
                for (int k = 0; k < 8; ++k) A.fnormals[8 * (uint64_t)j + k] = normals[k];
            return;
        }
        p = t.com;  // MinimiseQEF of a planar cell
    } else {
        p = qef::particle_placement(corners, normals);
    }
    A.dpos[id] = DcPos{p.x, p.y, p.z, 0.0f};
}

// one thread per active cell, grid-stride over the list
template <class Ev>
__device__ __forceinline__ void dc_place_body(const Ev& ev, const DcCells& A) {
    const uint32_t count = *A.count;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x)
        dc_place_one(ev, A, A.list[i]);
}

}  // namespace iso
