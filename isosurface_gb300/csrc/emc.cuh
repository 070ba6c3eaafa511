// ExtendedMarchingCubes (src/extended_marching_cubes.rs) over the Directed
// metric (src/distance.rs:72-104): the work of one lattice point or one cell,
// as functions that compile for the device (emc.cu launches them, one thread
// per item) and for the host (so that a host build of the same code can be
// checked item by item).  The including unit defines ISO_TABLE and includes
// mc_tables.h and emc_tables.h first.
//
// Passes, all over the PrimalGrid lattice of size n (n x n x (n+1) points,
// (n-1) x (n-1) x n cells in (z, y, x) order, primal_grid.rs:39-89):
//   sample     Directed value (sample_vector) of every lattice point;
//   count      per cell: case from Directed::is_positive, the edge crossings
//              along each edge's own axis, normals there, tangent planes
//              (TangentPlanes::from_edge_crossings) and the feature decision;
//              vertices the cell adds (owned crossing edges, plus the feature
//              point) and triangles (marching-cubes triangles, or one fan
//              triangle per edge-loop segment);
//   (an exclusive scan of each count gives each cell's output offsets)
//   vertices   the feature point (MinimiseQEF::place_feature_with_tangents)
//              first, then the owned edge vertices in the cell's order of
//              first use; the edge map records each owned edge's vertex id;
//   triangles  in the reference's order: march_cube's triangles for planar
//              cells, (e0, e1, centre) per loop segment for feature cells;
//   flips      flip_feature_edges: a loop segment shared by exactly two fan
//              triangles is rotated (MeshTopology::rotate_edge) to join
//              their centres.
//
// Ownership: IndexCache hands a lattice edge's vertex to the first cell in
// traversal order that uses it; every cell around a crossing edge uses it,
// so the first is a function of position: the cell owns its edge when, on
// each of the edge's two other axes, the edge lies on the cell's far side or
// the cell is on the lattice's low boundary.
//
// Flips: an edge joining two edge vertices with a feature vertex opposite on
// both of its two faces is a segment of two fans, either of two feature
// cells sharing the cube face the segment lies on, or of two loops of one
// cell (a segment across the cell's interior).  Edges at a fan centre have
// edge vertices opposite and marching-cubes triangles have no feature
// vertex, so each fan triangle is rotated at most once and the result does
// not depend on the order the reference's HashSet yields.  The earlier of the
// two faces (the lower triangle index) is rotate_edge's first face.
#pragma once
#include <cuda_runtime.h>

#include "qef.cuh"
#include "vm.cuh"

namespace iso {
namespace emc {

constexpr float F32_MAX = 3.40282347e+38f;

__host__ __device__ __forceinline__ void set_err(uint32_t* err, uint32_t bit) {
#ifdef __CUDA_ARCH__
    atomicOr(err, bit);
#else
    *err |= bit;
#endif
}

__host__ __device__ __forceinline__ int popc(uint32_t v) {
#ifdef __CUDA_ARCH__
    return __popc(v);
#else
    return __builtin_popcount(v);
#endif
}

__host__ __device__ __forceinline__ V3 vmax3(V3 a, V3 b) { return v3(fmaxf(a.x, b.x), fmaxf(a.y, b.y), fmaxf(a.z, b.z)); }
__host__ __device__ __forceinline__ V3 vabs(V3 a) { return v3(fabsf(a.x), fabsf(a.y), fabsf(a.z)); }

// ---------------------------------------------------------------------------
// VectorSource::sample_vector of the primitives: per axis, the signed
// distance from the point to the surface along that axis, F32_MAX where the
// axis line through the point misses the surface.
// ---------------------------------------------------------------------------

// sphere.rs:41-57
__host__ __device__ __forceinline__ V3 dir_sphere(V3 p, float r) {
    const V3 a = vabs(p);
    const float r2 = r * r;
    const float l_yz = r2 - (a.y * a.y + a.z * a.z);
    const float l_xz = r2 - (a.x * a.x + a.z * a.z);
    const float l_xy = r2 - (a.x * a.x + a.y * a.y);
    return v3(l_yz < 0.0f ? F32_MAX : a.x - sqrtf(l_yz), l_xz < 0.0f ? F32_MAX : a.y - sqrtf(l_xz),
              l_xy < 0.0f ? F32_MAX : a.z - sqrtf(l_xy));
}

// rectangular_prism.rs:43-70: outside the slab of the other two axes the
// axis line misses the box (+MAX); otherwise the distance to the clamp point
__host__ __device__ __forceinline__ V3 dir_box(V3 p, float hx, float hy, float hz) {
    const V3 a = vabs(p);
    const V3 mask = v3(((a.y - hy > 0.0f || a.z - hz > 0.0f) ? 1.0f : -1.0f) * F32_MAX,
                       ((a.x - hx > 0.0f || a.z - hz > 0.0f) ? 1.0f : -1.0f) * F32_MAX,
                       ((a.x - hx > 0.0f || a.y - hy > 0.0f) ? 1.0f : -1.0f) * F32_MAX);
    const bool inside = a.x < hx && a.y < hy && a.z < hz;
    const V3 h = v3(hx, hy, hz);
    const V3 closest = inside ? vmax3(a, h) : vmin(a, h);
    return vmax3(a - closest, mask);
}

// cylinder.rs:50-71
__host__ __device__ __forceinline__ V3 dir_cylinder(V3 p, float r, float hl) {
    const V3 a = vabs(p);
    const float r2 = r * r;
    return v3((a.z > hl || a.y > r) ? F32_MAX : a.x - sqrtf(r2 - a.y * a.y),
              (a.z > hl || a.x > r) ? F32_MAX : a.y - sqrtf(r2 - a.x * a.x),
              (a.x * a.x + a.y * a.y > r2) ? F32_MAX : a.z - hl);
}

// torus.rs:48-100; square roots of negative numbers give NaN, which fmaxf
// (f32::max) drops in favour of the other operand
__host__ __device__ __forceinline__ V3 dir_torus(V3 p, float R, float t) {
    const V3 a = vabs(p);
    const float l = sqrtf(a.x * a.x + a.y * a.y);
    const float l_xy = l - R;
    const float trz = sqrtf(t * t - a.z * a.z);
    const float rx = R + trz, ry = R - trz;
    float x, y;
    if (a.z > t || a.y > R + trz) x = F32_MAX;
    else if (a.x == 0.0f) x = fabsf(a.y - R) - t;
    else x = fmaxf(a.x - sqrtf(rx * rx - a.y * a.y), sqrtf(ry * ry - a.y * a.y) - a.x);
    if (a.z > t || a.x > R + trz) y = F32_MAX;
    else if (a.y == 0.0f) y = fabsf(a.x - R) - t;
    else y = fmaxf(a.y - sqrtf(rx * rx - a.x * a.x), sqrtf(ry * ry - a.x * a.x) - a.y);
    const float z = fabsf(l_xy) > t ? F32_MAX : a.z - sqrtf(t * t - l_xy * l_xy);
    return v3(x, y, z);
}

// sample_vector of a program: the point ops move the point (translate and
// domain map, as in scalar mode), Union / Intersection / Difference take the
// component-wise min, max and max(b, -a) (csg.rs:41-45, 74-78, 102-106), and
// CentralDifference passes the inner source's vector through (source.rs:76-80).
// The host accepts only programs made of these ops (directed_ops_only).
static __host__ __device__ __noinline__ V3 eval_vector(const ProgView& pv, V3 p) {
    V3 vs[VSTACK];
    V3 ps[PSTACK];
    int vsp = 0, psp = 0;
    V3 q = p;
    for (uint32_t pc = 0; pc < pv.n_ops; ++pc) {
        const uint32_t w = ld_ro(pv.ops + pc);
        const uint32_t op = w & 0xFFu;
        const float* k = pv.k + (w >> 8);
        switch (op) {
        case OP_PT_DOMAIN: case OP_PT_TRANSLATE:
            ps[psp++] = q;
            q = pt_apply(op, k, q);
            break;
        case OP_PT_POP: q = ps[--psp]; break;
        case OP_SPHERE: vs[vsp++] = dir_sphere(q, k[0]); break;
        case OP_BOX: vs[vsp++] = dir_box(q, k[0], k[1], k[2]); break;
        case OP_CYLINDER: vs[vsp++] = dir_cylinder(q, k[0], k[1]); break;
        case OP_TORUS: vs[vsp++] = dir_torus(q, k[0], k[1]); break;
        case OP_UNION: --vsp; vs[vsp - 1] = vmin(vs[vsp - 1], vs[vsp]); break;
        case OP_INTERSECTION: --vsp; vs[vsp - 1] = vmax3(vs[vsp - 1], vs[vsp]); break;
        case OP_DIFFERENCE: {
            --vsp;
            const V3 a = vs[vsp - 1], b = vs[vsp];
            vs[vsp - 1] = vmax3(b, v3(-a.x, -a.y, -a.z));
            break;
        }
        default: break;  // CD_BEGIN / CD_END: the vector is the inner source's
        }
    }
    return vs[0];
}

// ---------------------------------------------------------------------------
// Lattice and cells
// ---------------------------------------------------------------------------

struct Grid {
    uint32_t n;  // lattice points along x and y; z has n + 1 layers
    float inv;   // 1 / (n - 1), the reference's one_over_size
};

__host__ __device__ __forceinline__ uint64_t num_points(uint32_t n) { return (uint64_t)n * n * (n + 1); }
__host__ __device__ __forceinline__ uint64_t num_cells(uint32_t n) { return (uint64_t)(n - 1) * (n - 1) * n; }
__host__ __device__ __forceinline__ uint64_t point_index(uint32_t n, uint32_t x, uint32_t y, uint32_t z) {
    return ((uint64_t)z * n + y) * n + x;
}
__host__ __device__ __forceinline__ void cell_xyz(uint32_t n, uint64_t c, uint32_t* x, uint32_t* y, uint32_t* z) {
    const uint32_t m = n - 1;
    *x = (uint32_t)(c % m);
    const uint64_t r = c / m;
    *y = (uint32_t)(r % m);
    *z = (uint32_t)(r / m);
}

// lattice point position, `x as f32 * one_over_size` (primal_grid.rs:50-70)
__host__ __device__ __forceinline__ V3 point_pos(const Grid& g, uint32_t x, uint32_t y, uint32_t z) {
    return v3((float)x * g.inv, (float)y * g.inv, (float)z * g.inv);
}

// lattice edge id: 3 x (its lower end point) + axis
__host__ __device__ __forceinline__ uint32_t edge_key(uint32_t n, uint32_t x, uint32_t y, uint32_t z, int e) {
    const uint32_t lo = iso_emc_edge_lo[e];
    return (uint32_t)(3 * point_index(n, x + (lo & 1), y + ((lo >> 1) & 1), z + (lo >> 2)) + iso_emc_edge_axis[e]);
}

// the first cell in traversal order to use the edge: see the file comment
__host__ __device__ __forceinline__ bool owns_edge(uint32_t x, uint32_t y, uint32_t z, int e) {
    const uint32_t lo = iso_emc_edge_lo[e], axis = iso_emc_edge_axis[e];
    const uint32_t c[3] = {x, y, z};
    for (uint32_t b = 0; b < 3; ++b)
        if (b != axis && !((lo >> b) & 1) && c[b] != 0) return false;
    return true;
}

// Directed::is_positive (distance.rs:87-90): outside when any component is
// positive; classify_corners sets bit i when corner i is not outside
__host__ __device__ __forceinline__ int classify_directed(const V3* v) {
    int cube = 0;
    for (int i = 0; i < 8; ++i)
        if (!(v[i].x > 0.0f || v[i].y > 0.0f || v[i].z > 0.0f)) cube |= 1 << i;
    return cube;
}

__host__ __device__ __forceinline__ float comp(V3 v, int axis) { return axis == 0 ? v.x : axis == 1 ? v.y : v.z; }

// Directed::find_crossing_point (distance.rs:94-103): interpolate on the
// component of the edge's axis (Vec3::max_component_index of |pa - pb|)
__host__ __device__ __forceinline__ V3 crossing_directed(V3 a, V3 b, V3 pa, V3 pb) {
    const V3 d = vabs(pa - pb);
    const int axis = (d.x > d.y && d.x > d.z) ? 0 : (d.y > d.z) ? 1 : 2;
    const float delta = comp(b, axis) - comp(a, axis);
    const float t = (delta == 0.0f) ? 0.5f : -comp(a, axis) / delta;
    return pa * (1.0f - t) + pb * t;
}

// the cell's corner positions and Directed values, in CORNERS order
__host__ __device__ __forceinline__ void load_cell(const float4* field, const Grid& g, uint32_t x, uint32_t y, uint32_t z,
                                                   V3* corners, V3* values) {
    for (int i = 0; i < 8; ++i) {
        const uint32_t px = x + iso_corners[i][0], py = y + iso_corners[i][1], pz = z + iso_corners[i][2];
        const float4 f = ld_ro(field + point_index(g.n, px, py, pz));
        corners[i] = point_pos(g, px, py, pz);
        values[i] = v3(f.x, f.y, f.z);
    }
}

// find_edge_crossings (marching_cubes_impl.rs:39-56) over the Directed values
__host__ __device__ __forceinline__ void edge_crossings(int cube, const V3* corners, const V3* values, V3* vtx) {
    const uint32_t mask = iso_edge_mask[cube];
    for (int i = 0; i < 12; ++i)
        if (mask & (1u << i)) {
            const int u = iso_edge_connection[i][0], v = iso_edge_connection[i][1];
            vtx[i] = crossing_directed(values[u], values[v], corners[u], corners[v]);
        }
}

// ---------------------------------------------------------------------------
// TangentPlanes::from_edge_crossings and MinimiseQEF over 3..12 crossings
// (feature/mod.rs:76-148, feature/qef.rs:36-68): the steps of the 8-point
// versions in qef.cuh, for n points.
// ---------------------------------------------------------------------------
struct PlanesN {
    qef::F3 normal[12];
    float d[12];
    int n;
    qef::F3 com;
    int feature;
};

__host__ __device__ inline void tangent_planes_n(const qef::F3* vtx, const qef::F3* nrm, int n, PlanesN* t) {
    using namespace qef;
    F3 com = f3(0.0f, 0.0f, 0.0f), axis = f3(0.0f, 0.0f, 0.0f);
    float min_angle = 3.40282347e+38f;
    float count = 0.0f;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
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
        for (int i = 0; i < n; ++i) {
            const float c = dot(axis, nrm[i]);
            min_c = fminf(min_c, c);
            max_c = fmaxf(max_c, c);
        }
        float c = fmaxf(fabsf(min_c), fabsf(max_c));
        c = sqrtf(1.0f - c * c);
        feature = (c > FEATURE_ANGLE) ? EDGE : CORNER;
    }
    for (int i = 0; i < n; ++i) {
        t->normal[i] = nrm[i];
        t->d[i] = dot(sub(vtx[i], com), nrm[i]);
    }
    t->n = n;
    t->com = com;
    t->feature = feature;
}

// *ok = false if the QR sweep bound was reached
__host__ __device__ inline qef::F3 minimise_qef_n(const PlanesN& t, bool* ok) {
    using namespace qef;
    *ok = true;
    if (t.feature == PLANAR) return t.com;
    double u[12][3], v[3][3], d[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < t.n; ++i) {
        u[i][0] = (double)t.normal[i].x;
        u[i][1] = (double)t.normal[i].y;
        u[i][2] = (double)t.normal[i].z;
    }
    double tau_v[2] = {0.0, 0.0};
    bidiagonalise<12>(u, d, tau_v, t.n);
    unpack(u, v, d, tau_v, t.n);
    *ok = diagonalise<12>(u, v, d, tau_v, t.n);
    singularise(u, v, d, t.n);
    if (t.feature == EDGE) {
        double s_min = 1.7976931348623157e308;
        int id = 0;
        for (int i = 0; i < 3; ++i)
            if (d[i] < s_min) {
                s_min = d[i];
                id = i;
            }
        d[id] = 0.0;
    }
    if (d[2] < 0.1) d[2] = 0.0;
    if (d[1] < 0.1) d[1] = 0.0;
    if (d[0] < 0.1) d[0] = 0.0;
    double w[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < t.n; ++i) {
        const double b = (double)t.d[i];
        if (b != 0.0)
            for (int j = 0; j < 3; ++j) w[j] += b * u[i][j];
    }
    for (int i = 0; i < 3; ++i)
        if (d[i] != 0.0) w[i] /= d[i];
    double x[3];
    for (int i = 0; i < 3; ++i) {
        double s = 0.0;
        for (int j = 0; j < 3; ++j) s += w[j] * v[i][j];
        x[i] = s;
    }
    return add(t.com, f3((float)x[0], (float)x[1], (float)x[2]));
}

// The tangent planes of an active cell: the normal (sample_normal,
// normalised or zero) at each edge crossing, in edge order
// (sample_normals_at_edge_crossings, marching_cubes_impl.rs:71-89).
__host__ __device__ inline void cell_planes(const ProgView& pv, int cube, const V3* vtx, PlanesN* t) {
    qef::F3 pv3[12], pn[12];
    const uint32_t mask = iso_edge_mask[cube];
    int n = 0;
    for (int i = 0; i < 12; ++i)
        if (mask & (1u << i)) {
            V3 nrm;
            eval_hermite(pv, vtx[i], &nrm);
            pv3[n] = qef::f3(vtx[i].x, vtx[i].y, vtx[i].z);
            pn[n] = qef::normalised_or_zero(qef::f3(nrm.x, nrm.y, nrm.z));
            ++n;
        }
    tangent_planes_n(pv3, pn, n, t);
}

// ---------------------------------------------------------------------------
// Per-item work
// ---------------------------------------------------------------------------
struct Args {
    ProgView prog;
    Grid g;
    float4* field;       // Directed value per lattice point (w unused)
    uint16_t* cell;      // per cell: case | feature << 8
    uint32_t* voff;      // per cell: vertices it adds; after the scan, its first vertex id
    uint32_t* toff;      // per cell: triangles it adds; after the scan, its first triangle
    uint32_t* edge_map;  // vertex id per lattice edge (3 per point), written by owners
    float* vertices;     // xyz per vertex
    uint32_t* indices;   // 3 per triangle
    uint64_t cap_v, cap_t;
    uint32_t* err;       // DERR_* bits
};

// the Directed value of lattice point `i`
__host__ __device__ inline void sample_item(const Args& A, uint64_t i) {
    const uint32_t n = A.g.n;
    const uint32_t x = (uint32_t)(i % n);
    const uint64_t r = i / n;
    const uint32_t y = (uint32_t)(r % n), z = (uint32_t)(r / n);
    const V3 v = eval_vector(A.prog, point_pos(A.g, x, y, z));
    A.field[i] = make_float4(v.x, v.y, v.z, 0.0f);
}

// case, feature decision and counts of cell `c`
__host__ __device__ inline void count_item(const Args& A, uint64_t c) {
    uint32_t x, y, z;
    cell_xyz(A.g.n, c, &x, &y, &z);
    V3 corners[8], values[8], vtx[12];
    load_cell(A.field, A.g, x, y, z, corners, values);
    const int cube = classify_directed(values);
    uint32_t feature = 0, nv = 0, nt = 0;
    if (cube != 0 && cube != 255) {
        edge_crossings(cube, corners, values, vtx);
        PlanesN t;
        cell_planes(A.prog, cube, vtx, &t);
        feature = t.feature != qef::PLANAR;
        const uint32_t mask = iso_edge_mask[cube];
        for (int e = 0; e < 12; ++e)
            if ((mask & (1u << e)) && owns_edge(x, y, z, e)) ++nv;
        nv += feature;
        nt = feature ? iso_emc_fan_count[cube] : iso_tri_count[cube];
    }
    A.cell[c] = (uint16_t)(cube | (feature << 8));
    A.voff[c] = nv;
    A.toff[c] = nt;
}

// the feature point of a feature cell (case `cube`, edge crossings `vtx`)
// as vertex `id`: MinimiseQEF over the cell's tangent planes
__host__ __device__ inline void put_feature(const Args& A, int cube, const V3* vtx, uint32_t id) {
    PlanesN t;
    cell_planes(A.prog, cube, vtx, &t);
    bool ok;
    const qef::F3 p = minimise_qef_n(t, &ok);
    if (!ok) set_err(A.err, DERR_SVD_ITER);
    if (id < A.cap_v) {
        A.vertices[3 * (uint64_t)id] = p.x;
        A.vertices[3 * (uint64_t)id + 1] = p.y;
        A.vertices[3 * (uint64_t)id + 2] = p.z;
    }
}

// the vertices cell `c` adds (offsets already scanned); with
// feature_point = false a feature cell's first vertex (its feature point) is
// left to feature_item
__host__ __device__ inline void vertex_item(const Args& A, uint64_t c, bool feature_point = true) {
    const uint32_t info = A.cell[c];
    const int cube = (int)(info & 0xFF);
    if (cube == 0 || cube == 255) return;
    const bool feature = (info >> 8) & 1;
    uint32_t x, y, z;
    cell_xyz(A.g.n, c, &x, &y, &z);
    V3 corners[8], values[8], vtx[12];
    load_cell(A.field, A.g, x, y, z, corners, values);
    edge_crossings(cube, corners, values, vtx);
    uint32_t id = A.voff[c];
    if (feature) {
        if (feature_point) put_feature(A, cube, vtx, id);
        ++id;
    }
    const uint64_t order = feature ? iso_emc_fan_order[cube] : iso_edge_order[cube];
    const int count = popc(iso_edge_mask[cube]);
    for (int k = 0; k < count; ++k) {
        const int e = (int)((order >> (4 * k)) & 15);
        if (!owns_edge(x, y, z, e)) continue;
        if (id < A.cap_v) {
            A.vertices[3 * (uint64_t)id] = vtx[e].x;
            A.vertices[3 * (uint64_t)id + 1] = vtx[e].y;
            A.vertices[3 * (uint64_t)id + 2] = vtx[e].z;
        }
        A.edge_map[edge_key(A.g.n, x, y, z, e)] = id;
        ++id;
    }
}

// the feature point of feature cell `c` (its first vertex)
__host__ __device__ inline void feature_item(const Args& A, uint64_t c) {
    const int cube = (int)(A.cell[c] & 0xFF);
    uint32_t x, y, z;
    cell_xyz(A.g.n, c, &x, &y, &z);
    V3 corners[8], values[8], vtx[12];
    load_cell(A.field, A.g, x, y, z, corners, values);
    edge_crossings(cube, corners, values, vtx);
    put_feature(A, cube, vtx, A.voff[c]);
}

// the triangles of cell `c`, after every vertex_item
__host__ __device__ inline void triangle_item(const Args& A, uint64_t c) {
    const uint32_t info = A.cell[c];
    const int cube = (int)(info & 0xFF);
    if (cube == 0 || cube == 255) return;
    const bool feature = (info >> 8) & 1;
    uint32_t x, y, z;
    cell_xyz(A.g.n, c, &x, &y, &z);
    const uint32_t n = A.g.n;
    uint64_t t = A.toff[c];
    auto put = [&](uint32_t a, uint32_t b, uint32_t d) {
        if (t < A.cap_t) {
            A.indices[3 * t] = a;
            A.indices[3 * t + 1] = b;
            A.indices[3 * t + 2] = d;
        }
        ++t;
    };
    if (!feature) {
        const uint64_t tri = iso_tri_edges[cube];
        for (int k = 0; k < iso_tri_count[cube]; ++k) {
            const int a = (int)((tri >> (12 * k)) & 15), b = (int)((tri >> (12 * k + 4)) & 15),
                      d = (int)((tri >> (12 * k + 8)) & 15);
            put(A.edge_map[edge_key(n, x, y, z, a)], A.edge_map[edge_key(n, x, y, z, b)],
                A.edge_map[edge_key(n, x, y, z, d)]);
        }
        return;
    }
    const uint32_t centre = A.voff[c];
    const int8_t* row = iso_emc_loops[cube];
    int at = 1 + row[0];
    for (int l = 0; l < row[0]; ++l) {
        const int k = row[1 + l];
        for (int i = 0; i < k; ++i) {
            const int e0 = row[at + i], e1 = row[at + (i + 1) % k];
            put(A.edge_map[edge_key(n, x, y, z, e0)], A.edge_map[edge_key(n, x, y, z, e1)], centre);
        }
        at += k;
    }
}

// the cube face two edges share: axis * 2 + side, or -1
__host__ __device__ __forceinline__ int shared_face(int e0, int e1) {
    const uint32_t a0 = iso_emc_edge_axis[e0], a1 = iso_emc_edge_axis[e1];
    const uint32_t l0 = iso_emc_edge_lo[e0], l1 = iso_emc_edge_lo[e1];
    for (uint32_t b = 0; b < 3; ++b)
        if (b != a0 && b != a1 && ((l0 >> b) & 1) == ((l1 >> b) & 1)) return (int)(2 * b + ((l0 >> b) & 1));
    return -1;
}

// the edge of the neighbour across the far face on axis b that is edge e here
__host__ __device__ __forceinline__ int edge_across(int e, uint32_t b) {
    return iso_emc_edge_at[iso_emc_edge_axis[e]][iso_emc_edge_lo[e] & ~(1u << b)];
}

// fan segments of a case joining edges {e0, e1} in either direction: their
// number, and the fan index of the first
__host__ __device__ inline int find_segment(int cube, int e0, int e1, int* first) {
    const int8_t* row = iso_emc_loops[cube];
    int at = 1 + row[0], j = 0, found = 0;
    *first = -1;
    for (int l = 0; l < row[0]; ++l) {
        const int k = row[1 + l];
        for (int i = 0; i < k; ++i, ++j) {
            const int a = row[at + i], b = row[at + (i + 1) % k];
            if ((a == e0 && b == e1) || (a == e1 && b == e0)) {
                if (found == 0) *first = j;
                ++found;
            }
        }
        at += k;
    }
    return found;
}

// rotate_edge (mesh.rs:138-172) on faces ta = (va, vb, c) and tb, the
// segment's other face with centre d: ta becomes (c, d, vb), tb (c, va, d)
__host__ __device__ __forceinline__ void rotate(const Args& A, uint64_t ta, uint64_t tb, uint32_t c, uint32_t d) {
    if (ta >= A.cap_t || tb >= A.cap_t) return;
    const uint32_t va = A.indices[3 * ta], vb = A.indices[3 * ta + 1];
    A.indices[3 * ta] = c;
    A.indices[3 * ta + 1] = d;
    A.indices[3 * ta + 2] = vb;
    A.indices[3 * tb] = c;
    A.indices[3 * tb + 1] = va;
    A.indices[3 * tb + 2] = d;
}

// the flips whose first face is a fan triangle of cell `c`, after every
// triangle_item; returns how many it made
__host__ __device__ inline uint32_t flip_item(const Args& A, uint64_t c) {
    const uint32_t info = A.cell[c];
    if (!((info >> 8) & 1)) return 0;
    const int cube = (int)(info & 0xFF);
    const uint32_t n = A.g.n;
    uint32_t x, y, z;
    cell_xyz(n, c, &x, &y, &z);
    const uint32_t cxyz[3] = {x, y, z};
    const uint32_t lim[3] = {n - 2, n - 2, n - 1};  // largest cell coordinate per axis
    const uint64_t stride[3] = {1, (uint64_t)(n - 1), (uint64_t)(n - 1) * (n - 1)};
    const uint64_t t0 = A.toff[c];
    const uint32_t centre = A.voff[c];
    const int8_t* row = iso_emc_loops[cube];
    int at = 1 + row[0], j = 0;
    uint32_t flips = 0;
    for (int l = 0; l < row[0]; ++l) {
        const int k = row[1 + l];
        for (int i = 0; i < k; ++i, ++j) {
            const int e0 = row[at + i], e1 = row[at + (i + 1) % k];
            const int face = shared_face(e0, e1);
            int first;
            const int here = find_segment(cube, e0, e1, &first);
            if (face < 0) {
                // a segment across the interior: two loops of this cell
                if (here != 2 || first != j) continue;
                int second = -1;
                const int8_t* r2 = row;
                int at2 = 1 + r2[0], j2 = 0;
                for (int l2 = 0; l2 < r2[0] && second < 0; ++l2) {
                    const int k2 = r2[1 + l2];
                    for (int i2 = 0; i2 < k2; ++i2, ++j2) {
                        const int a = r2[at2 + i2], b = r2[at2 + (i2 + 1) % k2];
                        if (j2 > j && ((a == e0 && b == e1) || (a == e1 && b == e0))) {
                            second = j2;
                            break;
                        }
                    }
                    at2 += k2;
                }
                if (second < 0) continue;
                rotate(A, t0 + j, t0 + second, centre, centre);
                ++flips;
                continue;
            }
            const uint32_t b = (uint32_t)(face >> 1);
            if (!(face & 1) || cxyz[b] >= lim[b]) continue;  // the earlier cell, or none, holds the first face
            const uint64_t nb = c + stride[b];
            const uint32_t ninfo = A.cell[nb];
            if (!((ninfo >> 8) & 1) || here != 1) continue;
            int jb;
            if (find_segment((int)(ninfo & 0xFF), edge_across(e0, b), edge_across(e1, b), &jb) != 1) continue;
            rotate(A, t0 + j, A.toff[nb] + (uint64_t)jb, centre, A.voff[nb]);
            ++flips;
        }
        at += k;
    }
    return flips;
}

}  // namespace emc
}  // namespace iso
