// CPU restatement of swiftcoder/isosurface's extraction path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the oracle: the checker that the
// GPU library's results are compared against (by tests/, by
// __graft_entry__.smoke() and by bench.py's cpu_baseline leg and reference
// arm).  The product never links, loads or calls it.
//
// The reference is pure Rust and no Rust toolchain exists on either machine,
// so it cannot be built and run here; every function below restates the cited
// reference code in C++ with the same f32/f64 operation order (built with
// -ffp-contract=off, no fast-math).
//
// Parity pin: the Source layer is pinned against the reference's own
// known-answer tests (tests/golden/kats.json, read from the reference's
// src/implicit/*.rs tests: values, normals and Directed vectors).  The
// reference has no test of any extractor, so the extraction stages (MC, DC,
// LHMC, EMC) are "parity unpinned" by reference tests; tests/ cross-checks
// them by mesh invariants and against independent plain-Python restatements
// of the same reference code (tests/test_mc_independent.py,
// tests/test_svd_independent.py).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <deque>
#include <map>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "program.h"
#include "ref_tables.h"

using namespace oracle;
using namespace ref_tables;

namespace {

// ===========================================================================
// Mesh assembly: src/mesh.rs + src/index_cache.rs + src/extractor.rs
// ===========================================================================

struct Key2 {  // ordered key pair; GridKey or MortonKey (index_cache.rs:17-73)
    uint64_t a, b;
    bool operator==(const Key2& o) const { return a == o.a && b == o.b; }
};
struct Key2Hash {
    size_t operator()(const Key2& k) const {
        uint64_t h = k.a * 0x9E3779B97F4A7C15ull ^ (k.b + 0x632BE59BD9B4E019ull + (k.a << 6) + (k.a >> 2));
        h ^= h >> 31;
        return (size_t)h;
    }
};
struct EdgeHash {
    size_t operator()(const std::pair<uint32_t, uint32_t>& e) const {
        return (size_t)(((uint64_t)e.first << 32 | e.second) * 0x9E3779B97F4A7C15ull >> 7);
    }
};

// The IndexedVertices extractor (extractor.rs:72-93), optionally with the
// normal of IndexedInterleavedNormals (extractor.rs:97-127).
struct Mesh {
    std::vector<float> vertices;   // xyz per vertex
    std::vector<float> normals;    // xyz per vertex when requested
    std::vector<uint32_t> indices;
    std::vector<uint64_t> keys;    // the dedup key of each vertex (2 words)
    uint64_t stale_corners = 0;    // LHMC only (implicit_octree.rs:84-95)
    uint64_t cells = 0;
};

// MeshTopologyBuilder (mesh.rs:225-260) with MeshTopology's face list and its
// edge bookkeeping (mesh.rs:44-100).  The edge set and edge-to-face map are
// only read by ExtendedMarchingCubes, but the reference maintains them for
// every face, so the CPU baseline keeps that cost.
struct MeshBuilder {
    Mesh* mesh;
    const Source* normal_source;  // non-null: IndexedInterleavedNormals
    bool keep_edge_maps;
    std::unordered_map<Key2, uint32_t, Key2Hash> cache;
    std::vector<uint32_t> faces;
    std::unordered_set<std::pair<uint32_t, uint32_t>, EdgeHash> edges;
    std::unordered_map<std::pair<uint32_t, uint32_t>, std::vector<uint32_t>, EdgeHash> edge_to_face;
    uint32_t next_vertex = 0;

    MeshBuilder(Mesh* m, const Source* ns, bool maps) : mesh(m), normal_source(ns), keep_edge_maps(maps) {}

    uint32_t add_vertex(const Key2& key, const Vec3& v) {
        auto it = cache.find(key);
        if (it != cache.end()) return it->second;
        uint32_t idx = next_vertex++;
        cache.emplace(key, idx);
        mesh->vertices.push_back(v.x);
        mesh->vertices.push_back(v.y);
        mesh->vertices.push_back(v.z);
        mesh->keys.push_back(key.a);
        mesh->keys.push_back(key.b);
        if (normal_source) {
            Vec3 n = normal_source->normal(v);
            mesh->normals.push_back(n.x);
            mesh->normals.push_back(n.y);
            mesh->normals.push_back(n.z);
        }
        return idx;
    }
    // add_vertex(None, v): a vertex no key refers to (the feature points of
    // ExtendedMarchingCubes); its dedup key reads as all ones
    uint32_t add_unkeyed(const Vec3& v) {
        uint32_t idx = next_vertex++;
        mesh->vertices.push_back(v.x);
        mesh->vertices.push_back(v.y);
        mesh->vertices.push_back(v.z);
        mesh->keys.push_back(~0ull);
        mesh->keys.push_back(~0ull);
        if (normal_source) {
            Vec3 n = normal_source->normal(v);
            mesh->normals.push_back(n.x);
            mesh->normals.push_back(n.y);
            mesh->normals.push_back(n.z);
        }
        return idx;
    }
    void edge(uint32_t u, uint32_t v, uint32_t face) {
        std::pair<uint32_t, uint32_t> e = u > v ? std::make_pair(v, u) : std::make_pair(u, v);
        edges.insert(e);
        edge_to_face[e].push_back(face);
    }
    void add_face(uint32_t a, uint32_t b, uint32_t c) {
        uint32_t face = (uint32_t)(faces.size() / 3);
        faces.push_back(a);
        faces.push_back(b);
        faces.push_back(c);
        if (keep_edge_maps) {
            edge(a, b, face);
            edge(b, c, face);
            edge(c, a, face);
        }
    }
    void finish() { mesh->indices = faces; }  // extract_indices, mesh.rs:91-100
};

// ===========================================================================
// Marching-cubes cell kernels: src/marching_cubes_impl.rs
// ===========================================================================

// classify_corners (:26-37): bit i set iff !(v_i > 0)
inline int classify_corners(const float* values) {
    int cube = 0;
    for (int i = 0; i < 8; ++i)
        if (!(values[i] > 0.0f)) cube |= 1 << i;
    return cube;
}

// Signed::find_crossing_point (distance.rs:64-69)
inline Vec3 find_crossing_point(float a, float b, const Vec3& pa, const Vec3& pb) {
    float delta = b - a;
    float t = (delta == 0.0f) ? 0.5f : -a / delta;
    return pa * (1.0f - t) + pb * t;
}

// find_edge_crossings (:39-56)
inline void find_edge_crossings(int cube, const Vec3* corners, const float* values, Vec3* vertices) {
    uint32_t edges = EDGE_CROSSING_MASK[cube];
    for (int i = 0; i < 12; ++i) {
        if (edges & (1u << i)) {
            int u = EDGE_CONNECTION[i][0], v = EDGE_CONNECTION[i][1];
            vertices[i] = find_crossing_point(values[u], values[v], corners[u], corners[v]);
        }
    }
}

// march_cube (:102-117)
template <class F>
inline void march_cube(int cube, F&& f) {
    for (int i = 0; i < 5; ++i) {
        if (TRIANGLE_CONNECTION[cube][3 * i] < 0) break;
        f(TRIANGLE_CONNECTION[cube][3 * i], TRIANGLE_CONNECTION[cube][3 * i + 1], TRIANGLE_CONNECTION[cube][3 * i + 2]);
    }
}

// sample_normals_at_corners (:58-69)
inline void sample_normals_at_corners(const Source& s, const Vec3* corners, Vec3* normals) {
    for (int i = 0; i < 8; ++i) normals[i] = s.normal(corners[i]).normalised_or_zero();
}

// GridKey::new (index_cache.rs:48-61) encoded as a lattice-edge id: the
// smaller lattice point (tuples compare x first, which for two neighbours
// picks the lower one) and the axis along which they differ.
struct LatticeKeys {
    uint64_t nx, ny;
    uint64_t point(uint64_t x, uint64_t y, uint64_t z) const { return (z * ny + y) * nx + x; }
};
inline Key2 grid_key(const LatticeKeys& lk, const uint32_t (*keys)[3], int edge) {
    const uint32_t* a = keys[EDGE_CONNECTION[edge][0]];
    const uint32_t* b = keys[EDGE_CONNECTION[edge][1]];
    bool a_gt = (a[0] != b[0]) ? a[0] > b[0] : (a[1] != b[1]) ? a[1] > b[1] : a[2] > b[2];
    const uint32_t* lo = a_gt ? b : a;
    const uint32_t* hi = a_gt ? a : b;
    uint64_t axis = hi[0] != lo[0] ? 0 : hi[1] != lo[1] ? 1 : 2;
    return Key2{lk.point(lo[0], lo[1], lo[2]) * 3 + axis, 0};
}

// ===========================================================================
// PrimalGrid::traverse (src/traversal/primal_grid.rs:39-89), restricted to
// the cell layers [z_begin, z_end) so that a bounded slab can be timed.  The
// full traversal is z_begin = 0, z_end = size.
// ===========================================================================
// `V` is the distance type (f32 for Signed, Vec3 for Directed) and `sample`
// the Sample<D> of the source.
template <class V, class S, class C>
void primal_grid(uint32_t size, uint32_t z_begin, uint32_t z_end, S&& sample, C&& callback) {
    const uint32_t n = size;
    const float one_over_size = 1.0f / (float)(size - 1);
    std::vector<Vec3> pos[2] = {std::vector<Vec3>((size_t)n * n), std::vector<Vec3>((size_t)n * n)};
    std::vector<V> val[2] = {std::vector<V>((size_t)n * n), std::vector<V>((size_t)n * n)};
    // layer z_begin (layer 0 in the reference)
    for (uint32_t y = 0; y < n; ++y)
        for (uint32_t x = 0; x < n; ++x) {
            Vec3 c((float)x * one_over_size, (float)y * one_over_size,
                   z_begin == 0 ? 0.0f : (float)z_begin * one_over_size);
            pos[0][(size_t)y * n + x] = c;
            val[0][(size_t)y * n + x] = sample(c);
        }
    uint32_t keys[8][3];
    Vec3 corners[8];
    V values[8];
    int cur = 0;
    for (uint32_t z = z_begin; z < z_end; ++z) {
        int nxt = cur ^ 1;
        for (uint32_t y = 0; y < n; ++y)
            for (uint32_t x = 0; x < n; ++x) {
                Vec3 c((float)x * one_over_size, (float)y * one_over_size, (float)(z + 1) * one_over_size);
                pos[nxt][(size_t)y * n + x] = c;
                val[nxt][(size_t)y * n + x] = sample(c);
            }
        for (uint32_t y = 0; y + 1 < n; ++y)
            for (uint32_t x = 0; x + 1 < n; ++x) {
                for (int i = 0; i < 8; ++i) {
                    keys[i][0] = x + CORNERS[i][0];
                    keys[i][1] = y + CORNERS[i][1];
                    keys[i][2] = z + CORNERS[i][2];
                    int layer = CORNERS[i][2] ? nxt : cur;
                    size_t at = (size_t)(y + CORNERS[i][1]) * n + x + CORNERS[i][0];
                    corners[i] = pos[layer][at];
                    values[i] = val[layer][at];
                }
                callback(x, y, z, keys, corners, values);
            }
        cur = nxt;
    }
}

template <class C>
void primal_traverse(const Source& src, uint32_t size, uint32_t z_begin, uint32_t z_end, C&& callback) {
    primal_grid<float>(size, z_begin, z_end, [&](const Vec3& c) { return src.scalar(c); }, callback);
}

// MarchingCubes::extract (src/marching_cubes.rs:59-82)
void marching_cubes(const Source& src, uint32_t size, uint32_t z0, uint32_t z1, Mesh* mesh,
                    const Source* normal_source, bool edge_maps) {
    MeshBuilder mb(mesh, normal_source, edge_maps);
    LatticeKeys lk{size, size};
    primal_traverse(src, size, z0, z1, [&](uint32_t, uint32_t, uint32_t, const uint32_t (*keys)[3],
                                           const Vec3* corners, const float* values) {
        int cube = classify_corners(values);
        Vec3 vertices[12];
        find_edge_crossings(cube, corners, values, vertices);
        march_cube(cube, [&](int a, int b, int c) {
            uint32_t ia = mb.add_vertex(grid_key(lk, keys, a), vertices[a]);
            uint32_t ib = mb.add_vertex(grid_key(lk, keys, b), vertices[b]);
            uint32_t ic = mb.add_vertex(grid_key(lk, keys, c), vertices[c]);
            mb.add_face(ia, ib, ic);
        });
        mesh->cells++;
    });
    mb.finish();
}

// PointCloud::extract (src/point_cloud.rs:50-63)
void point_cloud(const Source& src, uint32_t size, Mesh* mesh) {
    primal_traverse(src, size, 0, size, [&](uint32_t, uint32_t, uint32_t, const uint32_t (*)[3],
                                            const Vec3* corners, const float* values) {
        int cube = classify_corners(values);
        if (cube != 0 && cube != 255) {
            Vec3 p = corners[0].lerp(corners[6], 0.5f);
            mesh->vertices.push_back(p.x);
            mesh->vertices.push_back(p.y);
            mesh->vertices.push_back(p.z);
        }
        mesh->cells++;
    });
}

// ===========================================================================
// 3-column SVD in f64: src/math/svd.rs (Householder bidiagonalisation, then
// implicit-shift QR with Givens rotations, then sign/order normalisation).
// The steps and their operation order follow the reference function by
// function; rows <= 12.
// ===========================================================================
namespace svd {

// factorize_hh (svd.rs:254-292): Householder vector of x[0..n), in place
double householder(double** x, int n) {
    double tau = 0.0;
    if (n > 1) {
        double xnorm;
        if (n == 2) {
            xnorm = std::fabs(*x[1]);
        } else {
            double scl = 0.0, ssq = 1.0;
            for (int i = 1; i < n; ++i) {
                double v = std::fabs(*x[i]);
                if (v != 0.0) {
                    if (scl < v) {
                        ssq = 1.0 + ssq * (scl / v) * (scl / v);
                        scl = v;
                    } else {
                        ssq += v / scl * (v / scl);
                    }
                }
            }
            xnorm = scl * std::sqrt(ssq);
        }
        if (xnorm != 0.0) {
            double alpha = *x[0];
            double beta = std::sqrt(alpha * alpha + xnorm * xnorm);
            if (alpha >= 0.0) beta = -beta;
            tau = (beta - alpha) / beta;
            double s = 1.0 / (alpha - beta);
            *x[0] = beta;
            for (int i = 1; i < n; ++i) *x[i] *= s;
        }
    }
    return tau;
}

// factorize (svd.rs:149-251): A = U B V^T with B upper bidiagonal
void bidiagonalise(double (*m)[3], double* tau_u, double* tau_v, int rows) {
    for (int i = 0; i < 3; ++i) {
        double* col[12];
        int n = rows - i;
        for (int q = 0; q < n; ++q) col[q] = &m[q + i][i];
        double tau = householder(col, n);
        tau_u[i] = tau;
        if (i + 1 < 3) {
            if (tau != 0.0) {
                for (int x = i + 1; x < 3; ++x) {
                    double wx = m[i][x];
                    for (int y = i + 1; y < rows; ++y) wx += m[y][x] * *col[y - i];
                    double tau_wx = tau * wx;
                    m[i][x] -= tau_wx;
                    for (int y = i + 1; y < rows; ++y) m[y][x] -= tau_wx * *col[y - i];
                }
            }
            double* row[2];
            row[0] = &m[i][i + 1];
            int nr = 1;
            if (i == 0) {
                row[1] = &m[i][i + 2];
                nr = 2;
            }
            tau = householder(row, nr);
            tau_v[i] = tau;
            if (tau != 0.0) {
                for (int y = i + 1; y < rows; ++y) {
                    double wy = m[y][i + 1];
                    if (i == 0) wy += m[y][i + 2] * *row[1];
                    double tau_wy = tau * wy;
                    m[y][i + 1] -= tau_wy;
                    if (i == 0) m[y][i + 2] -= tau_wy * *row[1];
                }
            }
        }
    }
}

// unpack (svd.rs:295-410): accumulate U and V from the reflectors
void unpack(double (*u)[3], double (*v)[3], double* tau_u, double* tau_v, int rows) {
    v[0][0] = v[1][1] = v[2][2] = 1.0;
    v[0][1] = v[0][2] = v[1][0] = v[1][2] = v[2][0] = v[2][1] = 0.0;
    for (int i = 1; i >= 0; --i) {
        double tau = tau_v[i];
        if (tau != 0.0) {
            for (int x = i + 1; x < 3; ++x) {
                double wx = v[i + 1][x];
                for (int y = i + 2; y < 3; ++y) wx += v[y][x] * u[i][y];
                double tau_wx = tau * wx;
                v[i + 1][x] -= tau_wx;
                for (int y = i + 2; y < 3; ++y) v[y][x] -= tau_wx * u[i][y];
            }
        }
    }
    for (int i = 0; i < 2; ++i) tau_v[i] = u[i][i + 1];
    for (int i = 2; i >= 0; --i) {
        double tau = tau_u[i];
        tau_u[i] = u[i][i];
        if (tau == 0.0) {
            u[i][i] = 1.0;
            if (i < 2) {
                u[i][2] = 0.0;
                if (i < 1) u[i][1] = 0.0;
            }
            for (int y = i + 1; y < rows; ++y) u[y][i] = 0.0;
        } else {
            for (int x = i + 1; x < 3; ++x) {
                double wx = 0.0;
                for (int y = i + 1; y < rows; ++y) wx += u[y][x] * u[y][i];
                double tau_wx = tau * wx;
                u[i][x] = -tau_wx;
                for (int y = i + 1; y < rows; ++y) u[y][x] -= tau_wx * u[y][i];
            }
            for (int y = i + 1; y < rows; ++y) u[y][i] = u[y][i] * -tau;
            u[i][i] = 1.0 - tau;
        }
    }
}

// chop (svd.rs:480-493)
void chop(double* a, double* b, int n) {
    double ai = a[0];
    for (int i = 0; i < n - 1; ++i) {
        double bi = b[i];
        double ai1 = a[i + 1];
        if (std::fabs(bi) < 1e-5 * (std::fabs(ai) + std::fabs(ai1))) b[i] = 0.0;
        ai = ai1;
    }
}

// computeGivens (svd.rs:850-866)
void givens(double a, double b, double* c, double* s) {
    if (b == 0.0) {
        *c = 1.0;
        *s = 0.0;
    } else if (std::fabs(b) > std::fabs(a)) {
        double t = -a / b;
        double s1 = 1.0 / std::sqrt(1.0 + t * t);
        *s = s1;
        *c = s1 * t;
    } else {
        double t = -b / a;
        double c1 = 1.0 / std::sqrt(1.0 + t * t);
        *c = c1;
        *s = c1 * t;
    }
}

// computeSchur (svd.rs:868-890)
void schur(double a1, double a2, double a3, double* c, double* s) {
    double apq = a1 * a2 * 2.0;
    if (apq == 0.0) {
        *c = 1.0;
        *s = 0.0;
    } else {
        double t;
        double tau = (a2 * a2 + (a3 + a1) * (a3 - a1)) / apq;
        if (tau >= 0.0) t = 1.0 / (tau + std::sqrt(1.0 + tau * tau));
        else t = -1.0 / (std::sqrt(1.0 + tau * tau) - tau);
        *c = 1.0 / std::sqrt(1.0 + t * t);
        *s = t * *c;
    }
}

inline void rot_cols(double (*m)[3], int rows, int p, int q, double c, double s) {
    for (int i = 0; i < rows; ++i) {
        double mp = m[i][p], mq = m[i][q];
        m[i][p] = mp * c - mq * s;
        m[i][q] = mp * s + mq * c;
    }
}

// qrstep_middle (svd.rs:604-637)
void qr_middle(double (*u)[3], double* tau_u, double* tau_v, int rows, int cols, int col) {
    double x = tau_v[col];
    double y = tau_u[col + 1];
    for (int j = col; j < cols - 1; ++j) {
        double c, s;
        givens(y, -x, &c, &s);
        for (int i = 0; i < rows; ++i) {
            double up = u[i][col], uq = u[i][j + 1];
            u[i][col] = up * c - uq * s;
            u[i][j + 1] = up * s + uq * c;
        }
        tau_u[j + 1] = x * s + y * c;
        if (j == col) tau_v[j] = x * c - y * s;
        if (j < cols - 2) {
            double z = tau_v[j + 1];
            tau_v[j + 1] *= c;
            x = z * -s;
            y = tau_u[j + 2];
        }
    }
}

// qrstep_end (svd.rs:639-666)
void qr_end(double (*v)[3], double* tau_u, double* tau_v) {
    double x = tau_u[1];
    double y = tau_v[1];
    for (int k = 1; k >= 0; --k) {
        double c, s;
        givens(x, y, &c, &s);
        rot_cols(v, 3, k, 2, c, s);
        tau_u[k] = x * c - y * s;
        if (k == 1) tau_v[k] = x * s + y * c;
        if (k > 0) {
            double z = tau_v[k - 1];
            tau_v[k - 1] *= c;
            x = tau_u[k - 1];
            y = z * s;
        }
    }
}

// qrstep_eigenvalue (svd.rs:668-683): Wilkinson shift
double shift(const double* tau_u, const double* tau_v) {
    double ta = tau_u[1] * tau_u[1] + tau_v[0] * tau_v[0];
    double tb = tau_u[2] * tau_u[2] + tau_v[1] * tau_v[1];
    double tab = tau_u[1] * tau_v[1];
    double dt = (ta - tb) / 2.0;
    if (dt >= 0.0) return tb - tab * tab / (dt + std::sqrt(dt * dt + tab * tab));
    return tb + tab * tab / (std::sqrt(dt * dt + tab * tab) - dt);
}

// qrstep_cols2 (svd.rs:685-847)
void qr_cols2(double (*u)[3], double (*v)[3], double* tau_u, double* tau_v, int rows) {
    if (tau_u[0] == 0.0) {
        double c, s;
        givens(tau_v[0], tau_u[1], &c, &s);
        tau_u[0] = tau_v[0] * c - tau_u[1] * s;
        tau_v[0] = tau_v[0] * s + tau_u[1] * c;
        tau_u[1] = 0.0;
        rot_cols(u, rows, 0, 1, c, s);
        for (int i = 0; i < 3; ++i) std::swap(v[i][0], v[i][1]);
    } else if (tau_u[1] == 0.0) {
        double c, s;
        givens(tau_u[0], tau_v[0], &c, &s);
        tau_u[0] = tau_u[0] * c - tau_v[0] * s;
        tau_v[0] = 0.0;
        rot_cols(v, 3, 0, 1, c, s);
    } else {
        double c, s;
        schur(tau_u[0], tau_v[0], tau_u[1], &c, &s);
        double a11 = tau_u[0] * c - tau_v[0] * s;
        double a21 = -tau_u[1] * s;
        double a12 = tau_u[0] * s + tau_v[0] * c;
        double a22 = tau_u[1] * c;
        rot_cols(v, 3, 0, 1, c, s);
        if (a11 * a11 + a21 * a21 < a12 * a12 + a22 * a22) {
            std::swap(a11, a12);
            std::swap(a21, a22);
            for (int i = 0; i < 3; ++i) std::swap(v[i][0], v[i][1]);
        }
        givens(a11, a21, &c, &s);
        tau_u[0] = a11 * c - a21 * s;
        tau_v[0] = a12 * c - a22 * s;
        tau_u[1] = a12 * s + a22 * c;
        rot_cols(u, rows, 0, 1, c, s);
    }
}

// qrstep (svd.rs:495-602)
void qr_step(double (*u)[3], double (*v)[3], double* tau_u, double* tau_v, int rows, int cols) {
    if (cols == 2) {
        qr_cols2(u, v, tau_u, tau_v, rows);
        return;
    }
    for (int i = 0; i < cols - 1; ++i) {
        if (tau_u[i] == 0.0) {
            qr_middle(u, tau_u, tau_v, rows, cols, i);
            return;
        }
    }
    if (tau_u[cols - 1] == 0.0) {
        qr_end(v, tau_u, tau_v);
        return;
    }
    double mu = shift(tau_u, tau_v);
    double y = tau_u[0] * tau_u[0] - mu;
    double z = tau_u[0] * tau_v[0];
    double ak = 0.0, bk = 0.0, zk;
    double ap = tau_u[0], bp = tau_v[0], aq = tau_u[1];
    for (int k = 0; k < cols - 1; ++k) {
        double c, s;
        givens(y, z, &c, &s);
        rot_cols(v, 3, k, k + 1, c, s);
        double bk1 = bk * c - z * s;
        double ap1 = ap * c - bp * s;
        double bp1 = ap * s + bp * c;
        double zp1 = aq * -s;
        double aq1 = aq * c;
        if (k > 0) tau_v[k - 1] = bk1;
        ak = ap1;
        bk = bp1;
        zk = zp1;
        ap = aq1;
        bp = (k < cols - 2) ? tau_v[k + 1] : 0.0;
        y = ak;
        z = zk;
        givens(y, z, &c, &s);
        rot_cols(u, rows, k, k + 1, c, s);
        double ak1 = ak * c - zk * s;
        bk1 = bk * c - ap * s;
        double zk1 = bp * -s;
        ap1 = bk * s + ap * c;
        bp1 = bp * c;
        tau_u[k] = ak1;
        ak = ak1;
        bk = bk1;
        zk = zk1;
        ap = ap1;
        bp = bp1;
        aq = (k < cols - 2) ? tau_u[k + 2] : 0.0;
        y = bk;
        z = zk;
    }
    tau_v[cols - 2] = bk;
    tau_u[cols - 1] = ap;
}

// diagonalize (svd.rs:413-478).  The reference loops until convergence with
// no bound; this restatement stops after 10000 sweeps (never reached on
// finite input in the tests) so that a NaN cannot hang the checker.
void diagonalise(double (*u)[3], double (*v)[3], double* tau_u, double* tau_v, int rows) {
    chop(tau_u, tau_v, 3);
    int b = 2;
    int guard = 0;
    while (b > 0 && guard++ < 10000) {
        if (tau_v[b - 1] == 0.0) {
            b -= 1;
        } else {
            int a = b - 1;
            while (a > 0 && tau_v[a - 1] != 0.0) a -= 1;
            int n = b - a + 1;
            double u1[12][3] = {}, v1[3][3] = {};
            for (int j = a; j <= b; ++j) {
                for (int i = 0; i < rows; ++i) u1[i][j - a] = u[i][j];
                for (int i = 0; i < 3; ++i) v1[i][j - a] = v[i][j];
            }
            qr_step(u1, v1, tau_u + a, tau_v + a, rows, n);
            for (int j = a; j <= b; ++j) {
                for (int i = 0; i < rows; ++i) u[i][j] = u1[i][j - a];
                for (int i = 0; i < 3; ++i) v[i][j] = v1[i][j - a];
            }
            chop(tau_u + a, tau_v + a, n);
        }
    }
}

// singularize (svd.rs:892-925)
void singularise(double (*u)[3], double (*v)[3], double* d, int rows) {
    for (int j = 0; j < 3; ++j) {
        if (d[j] < 0.0) {
            for (int i = 0; i < 3; ++i) v[i][j] = -v[i][j];
            d[j] = -d[j];
        }
    }
    for (int i = 0; i < 3; ++i) {
        double d_max = d[i];
        int i_max = i;
        for (int j = i + 1; j < 3; ++j)
            if (d[j] > d_max) {
                d_max = d[j];
                i_max = j;
            }
        if (i_max != i) {
            std::swap(d[i], d[i_max]);
            for (int y = 0; y < rows; ++y) std::swap(u[y][i], u[y][i_max]);
            for (int y = 0; y < 3; ++y) std::swap(v[y][i], v[y][i_max]);
        }
    }
}

struct Svd {
    int rows;
    double u[12][3], v[3][3], d[3];
};

// computeSVD (svd.rs:130-146): tau_u aliases d
void compute(const double (*mat)[3], int rows, Svd* out) {
    out->rows = rows;
    std::memset(out->u, 0, sizeof(out->u));
    std::memset(out->v, 0, sizeof(out->v));
    std::memset(out->d, 0, sizeof(out->d));
    for (int i = 0; i < rows; ++i)
        for (int j = 0; j < 3; ++j) out->u[i][j] = mat[i][j];
    double tau_v[2] = {0.0, 0.0};
    bidiagonalise(out->u, out->d, tau_v, rows);
    unpack(out->u, out->v, out->d, tau_v, rows);
    diagonalise(out->u, out->v, out->d, tau_v, rows);
    singularise(out->u, out->v, out->d, rows);
}

// SVD::solve (svd.rs:55-84) + solveSVD (svd.rs:928-972)
void solve(Svd* s, const double* b, double* x) {
    if (s->d[2] < 0.1) s->d[2] = 0.0;
    if (s->d[1] < 0.1) s->d[1] = 0.0;
    if (s->d[0] < 0.1) s->d[0] = 0.0;
    double w[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < s->rows; ++i)
        if (b[i] != 0.0)
            for (int j = 0; j < 3; ++j) w[j] += b[i] * s->u[i][j];
    for (int i = 0; i < 3; ++i)
        if (s->d[i] != 0.0) w[i] /= s->d[i];
    for (int i = 0; i < 3; ++i) {
        double t = 0.0;
        for (int j = 0; j < 3; ++j) t += w[j] * s->v[i][j];
        x[i] = t;
    }
}

}  // namespace svd

// ===========================================================================
// Feature placement: src/feature/mod.rs, qef.rs, particle_minimisation.rs
// ===========================================================================
const float FEATURE_ANGLE = 0.8660254037844387f;  // feature/mod.rs:22
enum Topology { PLANAR, EDGE, CORNER };

struct Planes {
    Vec3 normal[12];
    float d[12];
    int n;
    Vec3 center_of_mass;
    Topology feature;
};

// TangentPlanes::new (feature/mod.rs:91-148) over n points: the 8 cell
// corners (from_corners, DualContouring) or a cell's 3-12 edge crossings
// (from_edge_crossings, ExtendedMarchingCubes)
void tangent_planes(const Vec3* vertices, const Vec3* normals, int n, Planes* t) {
    Vec3 com, axis;
    float min_angle = 3.40282347e+38f;
    float count = 0.0f;
    for (int i = 0; i < n; ++i) {
        for (int j = 0; j < n; ++j) {
            float angle = normals[i].dot(normals[j]);
            if (angle < min_angle) {
                axis = normals[i].cross(normals[j]);
                min_angle = angle;
            }
        }
        com = com + vertices[i];
        count += 1.0f;
    }
    com = com / count;
    Topology feature;
    if (min_angle > FEATURE_ANGLE) {
        feature = PLANAR;
    } else {
        axis = axis.normalised_or_zero();
        float min_c = 1.0f, max_c = -1.0f;
        for (int i = 0; i < n; ++i) {
            float c = axis.dot(normals[i]);
            min_c = std::fmin(min_c, c);
            max_c = std::fmax(max_c, c);
        }
        float c = std::fmax(std::fabs(min_c), std::fabs(max_c));
        c = std::sqrt(1.0f - c * c);
        feature = (c > FEATURE_ANGLE) ? EDGE : CORNER;
    }
    for (int i = 0; i < n; ++i) {
        t->normal[i] = normals[i];
        t->d[i] = (vertices[i] - com).dot(normals[i]);
    }
    t->n = n;
    t->center_of_mass = com;
    t->feature = feature;
}

// MinimiseQEF::place_feature_with_tangents (feature/qef.rs:36-68)
Vec3 minimise_qef(const Planes& t) {
    if (t.feature == PLANAR) return t.center_of_mass;
    double a[12][3];
    for (int i = 0; i < t.n; ++i) {
        a[i][0] = (double)t.normal[i].x;
        a[i][1] = (double)t.normal[i].y;
        a[i][2] = (double)t.normal[i].z;
    }
    svd::Svd s;
    svd::compute(a, t.n, &s);
    if (t.feature == EDGE) {
        double s_min = 1.7976931348623157e308;
        int id = 0;
        for (int i = 0; i < 3; ++i)
            if (s.d[i] < s_min) {
                s_min = s.d[i];
                id = i;
            }
        s.d[id] = 0.0;
    }
    double b[12];
    for (int i = 0; i < t.n; ++i) b[i] = (double)t.d[i];
    double x[3];
    svd::solve(&s, b, x);
    return t.center_of_mass + Vec3((float)x[0], (float)x[1], (float)x[2]);
}

// ParticleBasedMinimisation (feature/particle_minimisation.rs:25-72)
Vec3 trilinear(const Vec3* corners, const Vec3* forces, const Vec3& p) {
    Vec3 f = (p - corners[0]) / (Vec3(corners[1].x, corners[3].y, corners[4].z) - corners[0]);
    Vec3 c00 = (1.0f - f.x) * forces[0] + f.x * forces[1];
    Vec3 c01 = (1.0f - f.x) * forces[4] + f.x * forces[5];
    Vec3 c10 = (1.0f - f.x) * forces[3] + f.x * forces[2];
    Vec3 c11 = (1.0f - f.x) * forces[7] + f.x * forces[6];
    Vec3 c0 = (1.0f - f.y) * c00 + f.y * c10;
    Vec3 c1 = (1.0f - f.y) * c01 + f.y * c11;
    return (1.0f - f.z) * c0 + f.z * c1;
}

Vec3 particle_placement(const Vec3* corners, const Vec3* normals) {
    const float STEP_SIZE = 0.05f, THRESHOLD = 0.02f;
    Planes t;
    tangent_planes(corners, normals, 8, &t);
    float max_feature_size = corners[6].x - corners[0].x;
    Vec3 particle = t.center_of_mass;
    Vec3 forces[8];
    for (int i = 0; i < 8; ++i)
        for (int j = 0; j < 8; ++j) {
            float dist = t.normal[j].dot(corners[i]) - t.d[j];          // Plane::distance
            Vec3 closest = corners[i] - t.normal[j] * dist;             // point_closest_to
            forces[i] = forces[i] + (corners[i] - closest);
        }
    for (int it = 0; it < 100; ++it) {
        Vec3 force = trilinear(corners, forces, particle) * STEP_SIZE * max_feature_size;
        particle = particle + force;
        if (force.len_sq() < THRESHOLD * max_feature_size) break;
    }
    return particle;
}

// ===========================================================================
// DualGrid::traverse (src/traversal/dual_grid.rs:52-95) + DualContouring::extract
// (src/dual_contouring.rs:65-105).  placer: 0 = MinimiseQEF, 1 = particles.
// ===========================================================================
void dual_contouring(const Source& src, uint32_t size, int placer, Mesh* mesh, std::vector<float>* duals_out) {
    const uint32_t m = size - 1;  // dual lattice is (size-1) x (size-1) x size
    std::vector<Vec3> dpos[2] = {std::vector<Vec3>((size_t)m * m), std::vector<Vec3>((size_t)m * m)};
    std::vector<float> dval[2] = {std::vector<float>((size_t)m * m), std::vector<float>((size_t)m * m)};
    MeshBuilder mb(mesh, nullptr, true);
    LatticeKeys lk{m, m};
    uint32_t keys[8][3];
    Vec3 corners[8];
    float values[8];
    Vec3 normals[8];
    primal_traverse(src, size, 0, size, [&](uint32_t x, uint32_t y, uint32_t z, const uint32_t (*)[3],
                                            const Vec3* pc, const float* pv) {
        Vec3 vertex = pc[0].lerp(pc[6], 0.5f);
        int cube = classify_corners(pv);
        if (cube != 0 && cube != 255) {
            sample_normals_at_corners(src, pc, normals);
            if (placer == 0) {
                Planes t;
                tangent_planes(pc, normals, 8, &t);
                vertex = minimise_qef(t);
            } else {
                vertex = particle_placement(pc, normals);
            }
        }
        float value = (1.0f - 0.5f) * pv[0] + 0.5f * pv[6];  // Signed::lerp, distance.rs:56-58
        dpos[z % 2][(size_t)y * m + x] = vertex;
        dval[z % 2][(size_t)y * m + x] = value;
        if (duals_out) {
            duals_out->push_back(vertex.x);
            duals_out->push_back(vertex.y);
            duals_out->push_back(vertex.z);
            duals_out->push_back(value);
        }
        if (x > 0 && y > 0 && z > 0) {
            uint32_t bx = x - 1, by = y - 1, bz = z - 1;
            for (int i = 0; i < 8; ++i) {
                keys[i][0] = bx + CORNERS[i][0];
                keys[i][1] = by + CORNERS[i][1];
                keys[i][2] = bz + CORNERS[i][2];
                size_t at = (size_t)(by + CORNERS[i][1]) * m + bx + CORNERS[i][0];
                corners[i] = dpos[(bz + CORNERS[i][2]) % 2][at];
                values[i] = dval[(bz + CORNERS[i][2]) % 2][at];
            }
            int c2 = classify_corners(values);
            Vec3 vertices[12];
            find_edge_crossings(c2, corners, values, vertices);
            march_cube(c2, [&](int a, int b, int c) {
                uint32_t ia = mb.add_vertex(grid_key(lk, keys, a), vertices[a]);
                uint32_t ib = mb.add_vertex(grid_key(lk, keys, b), vertices[b]);
                uint32_t ic = mb.add_vertex(grid_key(lk, keys, c), vertices[c]);
                mb.add_face(ia, ib, ic);
            });
            mesh->cells++;
        }
    });
    mb.finish();
}

// ===========================================================================
// ExtendedMarchingCubes: src/extended_marching_cubes.rs over the Directed
// metric (src/distance.rs:72-104)
// ===========================================================================

// Directed::is_positive (distance.rs:87-90): outside when any component is
// positive; classify_corners (marching_cubes_impl.rs:26-37) sets bit i when
// corner i is not outside
inline int classify_directed(const Vec3* values) {
    int cube = 0;
    for (int i = 0; i < 8; ++i)
        if (!(values[i].x > 0.0f || values[i].y > 0.0f || values[i].z > 0.0f)) cube |= 1 << i;
    return cube;
}

// Vec3::max_component_index (vector.rs:255-263)
inline int max_component_index(const Vec3& v) {
    if (v.x > v.y && v.x > v.z) return 0;
    if (v.y > v.z) return 1;
    return 2;
}
inline float component(const Vec3& v, int axis) { return axis == 0 ? v.x : axis == 1 ? v.y : v.z; }

// Directed::find_crossing_point (distance.rs:94-103): interpolate on the
// component of the edge's own axis
inline Vec3 find_crossing_directed(const Vec3& a, const Vec3& b, const Vec3& pa, const Vec3& pb) {
    int axis = max_component_index((pa - pb).abs());
    float delta = component(b, axis) - component(a, axis);
    float t = (delta == 0.0f) ? 0.5f : -component(a, axis) / delta;
    return pa * (1.0f - t) + pb * t;
}

struct EmcStats {
    uint64_t features = 0;   // feature vertices spawned
    uint64_t flips = 0;      // edges rotated
    uint64_t conflicts = 0;  // flips that met a face an earlier flip rewrote
};

// Face::vertex_opposite (mesh.rs:190-199)
inline uint32_t vertex_opposite(const uint32_t* f, uint32_t e0, uint32_t e1) {
    for (int i = 0; i < 3; ++i)
        if (f[i] != e0 && f[i] != e1) return f[i];
    return f[0];  // unreachable for the faces extraction makes
}

// Face::matches_winding_direction (mesh.rs:201-213); false in *found when
// the edge is not on the face (the reference panics there)
inline bool matches_winding(const uint32_t* f, uint32_t e0, uint32_t e1, bool* found) {
    for (int i = 0; i < 3; ++i) {
        int j = (i + 1) % 3;
        if (e0 == f[i] && e1 == f[j]) { *found = true; return true; }
        if (e0 == f[j] && e1 == f[i]) { *found = true; return false; }
    }
    *found = false;
    return false;
}

// flip_feature_edges (extended_marching_cubes.rs:157-186) with
// MeshTopology::rotate_edge (mesh.rs:138-172).  The flips are chosen on the
// finished mesh, then applied.  The reference applies them in the order of
// its HashSet (random per run); when no face is rewritten by two flips the
// result is the same in every order, which `conflicts` == 0 states.  Here
// they are applied in ascending (start, end) order, or, with a non-zero
// `order_seed`, in a seeded random order (to check that claim).
void flip_feature_edges(MeshBuilder& mb, const std::vector<uint8_t>& feature, EmcStats* st, uint64_t order_seed) {
    typedef std::pair<uint32_t, uint32_t> Edge;
    std::vector<Edge> flips;
    for (const Edge& e : mb.edges) {
        if (feature[e.first] && feature[e.second]) continue;
        auto it = mb.edge_to_face.find(e);
        if (it == mb.edge_to_face.end() || it->second.size() != 2) continue;
        const uint32_t* fa = &mb.faces[3 * (size_t)it->second[0]];
        const uint32_t* fb = &mb.faces[3 * (size_t)it->second[1]];
        if (feature[vertex_opposite(fa, e.first, e.second)] && feature[vertex_opposite(fb, e.first, e.second)])
            flips.push_back(e);
    }
    std::sort(flips.begin(), flips.end());
    if (order_seed) {  // Fisher-Yates with SplitMix64
        uint64_t x = order_seed;
        for (size_t i = flips.size(); i > 1; --i) {
            x += 0x9E3779B97F4A7C15ull;
            uint64_t z = x;
            z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
            z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
            z ^= z >> 31;
            std::swap(flips[i - 1], flips[z % i]);
        }
    }
    std::vector<uint8_t> rewritten(mb.faces.size() / 3, 0);
    for (const Edge& e : flips) {
        auto it = mb.edge_to_face.find(e);
        if (it == mb.edge_to_face.end() || it->second.size() != 2) continue;
        uint32_t ha = it->second[0], hb = it->second[1];
        if (rewritten[ha] || rewritten[hb]) st->conflicts++;
        uint32_t fa[3], fb[3];
        std::memcpy(fa, &mb.faces[3 * (size_t)ha], sizeof(fa));
        std::memcpy(fb, &mb.faces[3 * (size_t)hb], sizeof(fb));
        uint32_t c = vertex_opposite(fa, e.first, e.second);
        uint32_t d = vertex_opposite(fb, e.first, e.second);
        bool found;
        bool m = matches_winding(fa, e.first, e.second, &found);
        if (!found) continue;
        uint32_t u = m ? e.second : e.first, v = m ? e.first : e.second;
        uint32_t na[3] = {c, d, u}, nb[3] = {c, v, d};
        std::memcpy(&mb.faces[3 * (size_t)ha], na, sizeof(na));
        std::memcpy(&mb.faces[3 * (size_t)hb], nb, sizeof(nb));
        rewritten[ha] = rewritten[hb] = 1;
        Edge ne = c > d ? Edge(d, c) : Edge(c, d);
        mb.edges.insert(ne);
        mb.edge_to_face[ne] = std::vector<uint32_t>{ha, hb};
        mb.edges.erase(e);
        mb.edge_to_face.erase(e);
        st->flips++;
    }
}

// ExtendedMarchingCubes::extract (extended_marching_cubes.rs:64-93) and
// march_cube_extended (:95-155): cells whose edge-crossing tangent planes
// are planar take the marching-cubes triangles; the others spawn a feature
// vertex placed by MinimiseQEF::place_feature_with_tangents and fan each of
// the case's edge loops (EDGE_LOOPS) around it.
void extended_marching_cubes(const Source& src, uint32_t size, Mesh* mesh, const Source* normal_source,
                             EmcStats* st, uint64_t flip_order_seed = 0) {
    MeshBuilder mb(mesh, normal_source, true);
    LatticeKeys lk{size, size};
    std::vector<uint8_t> feature;  // per vertex: 1 for a feature vertex
    primal_grid<Vec3>(size, 0, size, [&](const Vec3& c) { return src.vec(c); },
                      [&](uint32_t, uint32_t, uint32_t, const uint32_t (*keys)[3], const Vec3* corners,
                          const Vec3* values) {
        int cube = classify_directed(values);
        Vec3 vertices[12], normals[12];
        uint32_t edges = EDGE_CROSSING_MASK[cube];
        for (int i = 0; i < 12; ++i)  // find_edge_crossings (marching_cubes_impl.rs:39-56)
            if (edges & (1u << i)) {
                int u = EDGE_CONNECTION[i][0], v = EDGE_CONNECTION[i][1];
                vertices[i] = find_crossing_directed(values[u], values[v], corners[u], corners[v]);
            }
        for (int i = 0; i < 12; ++i)  // sample_normals_at_edge_crossings (:71-89)
            if (edges & (1u << i)) normals[i] = src.normal(vertices[i]).normalised_or_zero();
        // TangentPlanes::from_edge_crossings (feature/mod.rs:76-89)
        Vec3 pv[12], pn[12];
        int n = 0;
        for (int i = 0; i < 12; ++i)
            if (edges & (1u << i)) {
                pv[n] = vertices[i];
                pn[n] = normals[i];
                ++n;
            }
        Planes t;
        tangent_planes(pv, pn, n, &t);
        if (t.feature == PLANAR) {
            march_cube(cube, [&](int a, int b, int c) {
                uint32_t ia = mb.add_vertex(grid_key(lk, keys, a), vertices[a]);
                uint32_t ib = mb.add_vertex(grid_key(lk, keys, b), vertices[b]);
                uint32_t ic = mb.add_vertex(grid_key(lk, keys, c), vertices[c]);
                mb.add_face(ia, ib, ic);
            });
        } else {
            uint32_t centre = mb.add_unkeyed(minimise_qef(t));
            feature.resize((size_t)centre + 1, 0);
            feature[centre] = 1;
            st->features++;
            int loops = EDGE_LOOPS[cube][0];
            int at = 1 + loops;
            for (int l = 0; l < loops; ++l) {
                int k = EDGE_LOOPS[cube][1 + l];
                for (int i = 0; i < k; ++i) {
                    int e0 = EDGE_LOOPS[cube][at + i], e1 = EDGE_LOOPS[cube][at + (i + 1) % k];
                    uint32_t a = mb.add_vertex(grid_key(lk, keys, e0), vertices[e0]);
                    uint32_t b = mb.add_vertex(grid_key(lk, keys, e1), vertices[e1]);
                    mb.add_face(a, b, centre);
                }
                at += k;
            }
        }
        mesh->cells++;
    });
    feature.resize(mb.next_vertex, 0);
    flip_feature_edges(mb, feature, st, flip_order_seed);
    mb.finish();
}

// ===========================================================================
// Morton codes: src/morton.rs
// ===========================================================================
namespace morton {
const int THREE_2 = 9, THREE_1 = 3, THREE_0 = 1;
const uint64_t SHIFT_2A = 18, SHIFT_2B = 36, SHIFT_1A = 6, SHIFT_1B = 12, SHIFT_0A = 2, SHIFT_0B = 4;
const uint64_t DILATE_MASK_2 = 0x7FC0000FF80001FFull;
const uint64_t DILATE_MASK_1 = 0x01C0E070381C0E07ull;
const uint64_t DILATE_MASK_0 = 0x9249249249249249ull;
const uint64_t DILATE_TZ = 0x4924924924924924ull;
const uint64_t DILATE_TY = 0x2492492492492492ull;
const uint64_t DILATE_TX = 0x9249249249249249ull;
const uint64_t DILATE_T1 = 0xB6DB6DB6DB6DB6DBull;
const uint64_t DILATE_T2 = 0xDB6DB6DB6DB6DB6Dull;
const uint64_t DILATE_T3 = 0x6DB6DB6DB6DB6DB6ull;
const double LG2_3 = 0.48089834696;
const int MAX_LEVEL = (8 * 8 - 1) / 3;

// morton.rs:54-59: floor(ln(k) * 0.48089834696)
int level(uint64_t k) { return k == 0 ? 0 : (int)std::floor(std::log((double)k) * LG2_3); }
uint64_t parent(uint64_t k) { return std::max<uint64_t>(k >> 3, 1); }
uint64_t child(uint64_t k, uint64_t which) { return (k << 3) | which; }
float size(uint64_t k) { return 1.0f / (float)((uint64_t)2 << level(k)); }
uint64_t add(uint64_t a, uint64_t b) {  // morton.rs:147-157
    return (((a | DILATE_T1) + (b & DILATE_TZ)) & DILATE_TZ) | (((a | DILATE_T2) + (b & DILATE_TY)) & DILATE_TY) |
           (((a | DILATE_T3) + (b & DILATE_TX)) & DILATE_TX);
}
uint64_t sub(uint64_t a, uint64_t b) {  // morton.rs:159-169
    return (((a & DILATE_TZ) - (b & DILATE_TZ)) & DILATE_TZ) | (((a & DILATE_TY) - (b & DILATE_TY)) & DILATE_TY) |
           (((a & DILATE_TX) - (b & DILATE_TX)) & DILATE_TX);
}
Vec3 center(uint64_t k) {  // morton.rs:78-116
    uint64_t bz = (k >> 2) & DILATE_MASK_0, by = (k >> 1) & DILATE_MASK_0, bx = k & DILATE_MASK_0;
    int lv = level(k);
    if (lv > THREE_0) {
        bz = (bz | (bz >> SHIFT_0A) | (bz >> SHIFT_0B)) & DILATE_MASK_1;
        by = (by | (by >> SHIFT_0A) | (by >> SHIFT_0B)) & DILATE_MASK_1;
        bx = (bx | (bx >> SHIFT_0A) | (bx >> SHIFT_0B)) & DILATE_MASK_1;
        if (lv > THREE_1) {
            bz = (bz | (bz >> SHIFT_1A) | (bz >> SHIFT_1B)) & DILATE_MASK_2;
            by = (by | (by >> SHIFT_1A) | (by >> SHIFT_1B)) & DILATE_MASK_2;
            bx = (bx | (bx >> SHIFT_1A) | (bx >> SHIFT_1B)) & DILATE_MASK_2;
            if (lv > THREE_2) {
                bz = bz | (bz >> SHIFT_2A) | (bz >> SHIFT_2B);
                by = by | (by >> SHIFT_2A) | (by >> SHIFT_2B);
                bx = bx | (bx >> SHIFT_2A) | (bx >> SHIFT_2B);
            }
        }
    }
    uint64_t length_mask = ((uint64_t)1 << lv) - 1;
    bz &= length_mask;
    by &= length_mask;
    bx &= length_mask;
    float s = size(k);
    float s2 = s * 2.0f;
    return Vec3((float)bx * s2 + s, (float)by * s2 + s, (float)bz * s2 + s);
}
uint64_t primal_vertex(uint64_t self, int lv, uint64_t which) {  // morton.rs:120-136
    uint64_t k = (uint64_t)1 << (3 * lv);
    uint64_t k1 = k << 1;
    uint64_t vk = add(self, which);
    uint64_t dk = sub(vk, k);
    if (vk >= k1 || (dk & DILATE_TX) == 0 || (dk & DILATE_TY) == 0 || (dk & DILATE_TZ) == 0) return 0;
    return vk << (3 * (MAX_LEVEL - lv));
}
uint64_t dual_vertex(uint64_t self, int lv, uint64_t which) {  // morton.rs:140-144
    return sub(self >> (3 * (MAX_LEVEL - lv)), which);
}
}  // namespace morton

// ImplicitOctree::traverse (src/traversal/implicit_octree.rs:39-99) feeding
// LinearHashedMarchingCubes::extract (src/linear_hashed_marching_cubes.rs:62-84).
// The reference walks its primal-vertex HashMap in RandomState order; this
// restatement walks it in ascending key order (one of the orders the
// reference can take).
void lhmc(const Source& src, uint32_t max_depth, Mesh* mesh, std::vector<uint64_t>* nodes_out) {
    const float SQRT_OF_3 = 1.73205080757f;  // distance.rs:19
    // LinearHashedOctree::build (linear_hashed_octree.rs:30-51): BFS from the root
    std::unordered_map<uint64_t, float> nodes;
    std::vector<uint64_t> leaves;
    std::deque<uint64_t> queue;
    queue.push_back(1);
    while (!queue.empty()) {
        uint64_t key = queue.front();
        queue.pop_front();
        float d = src.scalar(morton::center(key));
        int lv = morton::level(key);
        float sz = morton::size(key);
        bool refine = lv < 2 || (lv < (int)max_depth && std::fabs(d) < sz * SQRT_OF_3);
        if (refine) {
            for (uint64_t i = 0; i < 8; ++i) queue.push_back(morton::child(key, i));
        } else {
            leaves.push_back(key);
        }
        nodes[key] = d;
        if (nodes_out) {
            nodes_out->push_back(key);
            uint32_t bits;
            std::memcpy(&bits, &d, 4);
            nodes_out->push_back(((uint64_t)(refine ? 1 : 0) << 32) | bits);
        }
    }
    std::map<uint64_t, int> primal;  // vertex -> deepest level
    for (uint64_t key : leaves) {
        int lv = morton::level(key);
        for (uint64_t i = 0; i < 8; ++i) {
            uint64_t v = morton::primal_vertex(key, lv, i);
            if (v != 0) {
                auto it = primal.find(v);
                if (it == primal.end()) primal[v] = lv;
                else if (lv > it->second) it->second = lv;
            }
        }
    }
    MeshBuilder mb(mesh, nullptr, true);
    uint64_t keys[8] = {1, 1, 1, 1, 1, 1, 1, 1};
    Vec3 corners[8];
    float values[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (auto& pv : primal) {
        for (int i = 0; i < 8; ++i) {
            uint64_t m = morton::dual_vertex(pv.first, pv.second, (uint64_t)REMAP_CUBE[i]);
            bool found = false;
            while (m > 1) {
                auto it = nodes.find(m);
                if (it != nodes.end()) {
                    keys[i] = m;
                    corners[i] = morton::center(m);
                    values[i] = it->second;
                    found = true;
                    break;
                }
                m = morton::parent(m);
            }
            if (!found) mesh->stale_corners++;
        }
        int cube = classify_corners(values);
        Vec3 vertices[12];
        find_edge_crossings(cube, corners, values, vertices);
        march_cube(cube, [&](int a, int b, int c) {
            auto mk = [&](int e) {
                uint64_t x = keys[EDGE_CONNECTION[e][0]], y = keys[EDGE_CONNECTION[e][1]];
                return x > y ? Key2{y, x} : Key2{x, y};
            };
            uint32_t ia = mb.add_vertex(mk(a), vertices[a]);
            uint32_t ib = mb.add_vertex(mk(b), vertices[b]);
            uint32_t ic = mb.add_vertex(mk(c), vertices[c]);
            mb.add_face(ia, ib, ic);
        });
        mesh->cells++;
    }
    mb.finish();
}

struct Program {
    SourcePtr src;
};

}  // namespace

// ===========================================================================
// C API used by the tests (ctypes) and by bench.py's CPU legs.
// ===========================================================================
extern "C" {

void* oracle_program_create(const uint8_t* bytes, size_t len, char* err, size_t errlen) {
    std::string e;
    SourcePtr s = parse_program(bytes, len, &e);
    if (!s) {
        if (err && errlen) std::snprintf(err, errlen, "%s", e.c_str());
        return nullptr;
    }
    Program* p = new Program();
    p->src = std::move(s);
    return p;
}

void oracle_program_destroy(void* p) { delete (Program*)p; }

int oracle_program_has_normal(void* p) { return ((Program*)p)->src->has_normal() ? 1 : 0; }

void oracle_sample_scalar(void* p, const float* pts, uint64_t n, float* out) {
    const Source& s = *((Program*)p)->src;
    for (uint64_t i = 0; i < n; ++i) out[i] = s.scalar(Vec3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
}

void oracle_sample_normal(void* p, const float* pts, uint64_t n, float* out) {
    const Source& s = *((Program*)p)->src;
    for (uint64_t i = 0; i < n; ++i) {
        Vec3 v = s.normal(Vec3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
        out[3 * i] = v.x;
        out[3 * i + 1] = v.y;
        out[3 * i + 2] = v.z;
    }
}

int oracle_program_has_vector(void* p) { return ((Program*)p)->src->has_vector() ? 1 : 0; }

// VectorSource::sample_vector (the Directed metric), 3 floats per point
void oracle_sample_vector(void* p, const float* pts, uint64_t n, float* out) {
    const Source& s = *((Program*)p)->src;
    for (uint64_t i = 0; i < n; ++i) {
        Vec3 v = s.vec(Vec3(pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]));
        out[3 * i] = v.x;
        out[3 * i + 1] = v.y;
        out[3 * i + 2] = v.z;
    }
}

// The sample grid of PrimalGrid: size x size x (size+1) values, x fastest.
void oracle_sample_grid(void* p, uint32_t size, float* out) {
    const Source& s = *((Program*)p)->src;
    const float inv = 1.0f / (float)(size - 1);
    size_t i = 0;
    for (uint32_t z = 0; z <= size; ++z)
        for (uint32_t y = 0; y < size; ++y)
            for (uint32_t x = 0; x < size; ++x)
                out[i++] = s.scalar(Vec3((float)x * inv, (float)y * inv, (float)z * inv));
}

// Case index of every cell visited by MarchingCubes::new(size), traversal order.
void oracle_mc_cases(void* p, uint32_t size, uint8_t* out) {
    size_t i = 0;
    primal_traverse(*((Program*)p)->src, size, 0, size,
                    [&](uint32_t, uint32_t, uint32_t, const uint32_t (*)[3], const Vec3*, const float* v) {
                        out[i++] = (uint8_t)classify_corners(v);
                    });
}

// flags bit 0: IndexedInterleavedNormals (per-vertex source normal)
void* oracle_mc(void* p, uint32_t size, uint32_t flags) {
    Mesh* m = new Mesh();
    const Source& s = *((Program*)p)->src;
    marching_cubes(s, size, 0, size, m, (flags & 1) ? &s : nullptr, true);
    return m;
}

// MarchingCubes::new(size) restricted to the cell layers [z0, z1): a bounded
// slab of the full traversal (its vertices are first seen inside the slab).
void* oracle_mc_slab(void* p, uint32_t size, uint32_t z0, uint32_t z1) {
    Mesh* m = new Mesh();
    marching_cubes(*((Program*)p)->src, size, z0, z1, m, nullptr, true);
    return m;
}

void* oracle_point_cloud(void* p, uint32_t size) {
    Mesh* m = new Mesh();
    point_cloud(*((Program*)p)->src, size, m);
    return m;
}

void* oracle_dc(void* p, uint32_t size, int placer, float* duals /* nullable, 4 per primal cell */) {
    Mesh* m = new Mesh();
    std::vector<float> d;
    dual_contouring(*((Program*)p)->src, size, placer, m, duals ? &d : nullptr);
    if (duals) std::memcpy(duals, d.data(), d.size() * sizeof(float));
    return m;
}

void* oracle_lhmc(void* p, uint32_t max_depth) {
    Mesh* m = new Mesh();
    lhmc(*((Program*)p)->src, max_depth, m, nullptr);
    return m;
}

// Octree node list in BFS order: (key, refine<<32 | value bits) pairs.
uint64_t oracle_lhmc_nodes(void* p, uint32_t max_depth, uint64_t* out, uint64_t cap) {
    Mesh m;
    std::vector<uint64_t> nodes;
    lhmc(*((Program*)p)->src, max_depth, &m, &nodes);
    uint64_t n = nodes.size() / 2;
    if (out) std::memcpy(out, nodes.data(), std::min<uint64_t>(n, cap) * 16);
    return n;
}

// TangentPlanes::from_edge_crossings + MinimiseQEF::place_feature_with_tangents
// over n (3..12) crossings with normalised normals: the topology (0 planar,
// 1 edge, 2 corner) and, for a feature, the placed point in out.
int oracle_emc_place(const float* vertices, const float* normals, int n, float* out) {
    Vec3 v[12], nn[12];
    for (int i = 0; i < n; ++i) {
        v[i] = Vec3(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2]);
        nn[i] = Vec3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
    }
    Planes t;
    tangent_planes(v, nn, n, &t);
    Vec3 p = minimise_qef(t);
    out[0] = p.x;
    out[1] = p.y;
    out[2] = p.z;
    return (int)t.feature;
}

// ExtendedMarchingCubes::new(size).extract; stats: features, flips, conflicts.
// flip_order_seed 0 applies the flips in ascending order, others in a seeded
// random order.
void* oracle_emc(void* p, uint32_t size, int normals, uint64_t* stats, uint64_t flip_order_seed) {
    const Source& s = *((Program*)p)->src;
    Mesh* m = new Mesh();
    EmcStats st;
    extended_marching_cubes(s, size, m, normals ? &s : nullptr, &st, flip_order_seed);
    if (stats) {
        stats[0] = st.features;
        stats[1] = st.flips;
        stats[2] = st.conflicts;
    }
    return m;
}

uint64_t oracle_mesh_vertices(void* m) { return ((Mesh*)m)->vertices.size() / 3; }
uint64_t oracle_mesh_indices(void* m) { return ((Mesh*)m)->indices.size(); }
uint64_t oracle_mesh_cells(void* m) { return ((Mesh*)m)->cells; }
uint64_t oracle_mesh_stale(void* m) { return ((Mesh*)m)->stale_corners; }
void oracle_mesh_copy(void* mp, float* vertices, uint32_t* indices, uint64_t* keys, float* normals) {
    Mesh* m = (Mesh*)mp;
    if (vertices && !m->vertices.empty()) std::memcpy(vertices, m->vertices.data(), m->vertices.size() * 4);
    if (indices && !m->indices.empty()) std::memcpy(indices, m->indices.data(), m->indices.size() * 4);
    if (keys && !m->keys.empty()) std::memcpy(keys, m->keys.data(), m->keys.size() * 8);
    if (normals && !m->normals.empty()) std::memcpy(normals, m->normals.data(), m->normals.size() * 4);
}
void oracle_mesh_destroy(void* m) { delete (Mesh*)m; }

// SVD + solve of a rows x 3 system (rows <= 12), for unit tests.
void oracle_svd_solve(const double* mat, int rows, const double* b, double* d_out, double* x_out) {
    double a[12][3];
    for (int i = 0; i < rows; ++i)
        for (int j = 0; j < 3; ++j) a[i][j] = mat[3 * i + j];
    svd::Svd s;
    svd::compute(a, rows, &s);
    for (int i = 0; i < 3; ++i) d_out[i] = s.d[i];
    svd::solve(&s, b, x_out);
}

// Feature placement of one cell (corners, normals already normalised).
void oracle_place_feature(const float* corners, const float* normals, int placer, float* out, int* topology) {
    Vec3 c[8], n[8];
    for (int i = 0; i < 8; ++i) {
        c[i] = Vec3(corners[3 * i], corners[3 * i + 1], corners[3 * i + 2]);
        n[i] = Vec3(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2]);
    }
    Planes t;
    tangent_planes(c, n, 8, &t);
    if (topology) *topology = (int)t.feature;
    Vec3 v = placer == 0 ? minimise_qef(t) : particle_placement(c, n);
    out[0] = v.x;
    out[1] = v.y;
    out[2] = v.z;
}

int oracle_morton_level(uint64_t k) { return morton::level(k); }
void oracle_morton_center(uint64_t k, float* out) {
    Vec3 c = morton::center(k);
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
}
uint64_t oracle_morton_primal_vertex(uint64_t k, int lv, uint64_t which) { return morton::primal_vertex(k, lv, which); }
uint64_t oracle_morton_dual_vertex(uint64_t k, int lv, uint64_t which) { return morton::dual_vertex(k, lv, which); }

// Checks the integer level rule used by the GPU, (floor(log2 k) / 3) less one
// at exact powers of 8 above 1, against morton.rs's ln-based formula for every
// k in [1, limit).  Returns the first k that differs, or 0.
uint64_t oracle_morton_level_rule_check(uint64_t limit) {
    for (uint64_t k = 1; k < limit; ++k) {
        int msb = 63 - __builtin_clzll(k);
        int lv = msb / 3;
        if (lv > 0 && k == ((uint64_t)1 << (3 * lv))) lv -= 1;
        if (lv != morton::level(k)) return k;
    }
    return 0;
}

// Timed MarchingCubes over the cell layers [z0, z1) of MarchingCubes::new(size),
// split into `threads` contiguous slabs each traversed by its own thread (one
// thread is the reference's own single-threaded path).  Returns seconds and
// the cells visited.
double oracle_mc_timed(void* p, uint32_t size, uint32_t z0, uint32_t z1, int threads, uint64_t* cells_out,
                       uint64_t* tris_out) {
    const Source& s = *((Program*)p)->src;
    if (threads < 1) threads = 1;
    std::vector<Mesh> meshes(threads);
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::thread> pool;
    uint32_t span = z1 - z0;
    for (int t = 0; t < threads; ++t) {
        uint32_t a = z0 + (uint32_t)((uint64_t)span * t / threads);
        uint32_t b = z0 + (uint32_t)((uint64_t)span * (t + 1) / threads);
        pool.emplace_back([&, a, b, t]() {
            if (b > a) marching_cubes(s, size, a, b, &meshes[t], nullptr, true);
        });
    }
    for (auto& th : pool) th.join();
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    uint64_t cells = 0, tris = 0;
    for (auto& m : meshes) {
        cells += m.cells;
        tris += m.indices.size() / 3;
    }
    if (cells_out) *cells_out = cells;
    if (tris_out) *tris_out = tris;
    return secs;
}

}  // extern "C"
