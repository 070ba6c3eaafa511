// Source-program parsing shared by the oracle's restatement: turns the byte
// program that callers hand to the GPU library (format documented in
// include/isosurface_gpu.h) into a tree of CPU source objects that follow the
// reference's Source types (src/source.rs, src/implicit/*.rs of
// swiftcoder/isosurface).
//
// TEST INFRASTRUCTURE ONLY: the oracle is the checker for the GPU library.
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

namespace oracle {

// ---------------------------------------------------------------------------
// Vec3 with the reference's f32 operation order (src/math/vector.rs).
// Built with -ffp-contract=off: Rust never fuses a*b+c.
// ---------------------------------------------------------------------------
struct Vec3 {
    float x, y, z;
    Vec3() : x(0), y(0), z(0) {}
    Vec3(float a, float b, float c) : x(a), y(b), z(c) {}
    Vec3 operator+(const Vec3& o) const { return Vec3(x + o.x, y + o.y, z + o.z); }
    Vec3 operator-(const Vec3& o) const { return Vec3(x - o.x, y - o.y, z - o.z); }
    Vec3 operator*(const Vec3& o) const { return Vec3(x * o.x, y * o.y, z * o.z); }
    Vec3 operator/(const Vec3& o) const { return Vec3(x / o.x, y / o.y, z / o.z); }
    Vec3 operator*(float f) const { return Vec3(x * f, y * f, z * f); }
    Vec3 operator/(float f) const { return Vec3(x / f, y / f, z / f); }
    Vec3 operator-() const { return Vec3(-x, -y, -z); }
    // vector.rs:458-466: fold!(+, x*x, y*y, z*z) == (x*x + y*y) + z*z
    float len_sq() const { return (x * x + y * y) + z * z; }
    float len() const { return std::sqrt(len_sq()); }
    // vector.rs:468-478: None when |len| < f32::EPSILON
    bool normalised(Vec3* out) const {
        float l = len();
        if (std::fabs(l) < 1.1920929e-07f) return false;
        *out = Vec3(x / l, y / l, z / l);
        return true;
    }
    Vec3 normalised_or_zero() const {
        Vec3 r;
        return normalised(&r) ? r : Vec3();
    }
    Vec3 abs() const { return Vec3(std::fabs(x), std::fabs(y), std::fabs(z)); }
    float component_sum() const { return x + y + z; }      // vector.rs:574-576
    float max_component() const { return std::fmax(x, std::fmax(y, z)); }  // :579-581
    float dot(const Vec3& o) const { return (*this * o).component_sum(); }  // :624-626
    Vec3 cross(const Vec3& r) const {                      // :629-635
        return Vec3(y * r.z - z * r.y, z * r.x - x * r.z, x * r.y - y * r.x);
    }
    Vec3 vmin(const Vec3& o) const { return Vec3(std::fmin(x, o.x), std::fmin(y, o.y), std::fmin(z, o.z)); }
    Vec3 vmax(const Vec3& o) const { return Vec3(std::fmax(x, o.x), std::fmax(y, o.y), std::fmax(z, o.z)); }
    // vector.rs:659-667: of = 1 - f; of*self + f*other per component
    Vec3 lerp(const Vec3& o, float f) const {
        float of = 1.0f - f;
        return Vec3(of * x + f * o.x, of * y + f * o.y, of * z + f * o.z);
    }
    // vector.rs:612-621
    Vec3 clamp_to_cardinal_axis() const {
        Vec3 p = abs();
        if (p.x > p.y && p.x > p.z) return Vec3(x, 0.0f, 0.0f);
        if (p.y > p.z) return Vec3(0.0f, y, 0.0f);
        return Vec3(0.0f, 0.0f, z);
    }
};
inline Vec3 operator*(float f, const Vec3& v) { return Vec3(f * v.x, f * v.y, f * v.z); }

// ---------------------------------------------------------------------------
// Sources (src/source.rs:21-48). `scalar` is ScalarSource::sample_scalar,
// `normal` HermiteSource::sample_normal (unnormalised), `vec`
// VectorSource::sample_vector (the Directed metric: per axis, the signed
// distance to the surface along that axis, f32::MAX where the axis line
// misses it), defined where has_vector() holds.
// ---------------------------------------------------------------------------
const float F32_MAX = 3.40282347e+38f;

struct Source {
    virtual ~Source() {}
    virtual float scalar(const Vec3& p) const = 0;
    virtual bool has_normal() const { return true; }
    virtual Vec3 normal(const Vec3& p) const = 0;
    virtual bool has_vector() const { return false; }
    virtual Vec3 vec(const Vec3&) const { return Vec3(); }
};
typedef std::unique_ptr<Source> SourcePtr;

// src/implicit/sphere.rs:35-63
struct Sphere : Source {
    float radius;
    explicit Sphere(float r) : radius(r) {}
    float scalar(const Vec3& p) const override { return p.len() - radius; }
    Vec3 normal(const Vec3& p) const override { return p; }
    bool has_vector() const override { return true; }
    // sphere.rs:41-57
    Vec3 vec(const Vec3& p) const override {
        Vec3 a = p.abs();
        float r2 = radius * radius;
        float l_yz = r2 - (a.y * a.y + a.z * a.z);
        float l_xz = r2 - (a.x * a.x + a.z * a.z);
        float l_xy = r2 - (a.x * a.x + a.y * a.y);
        return Vec3(l_yz < 0.0f ? F32_MAX : a.x - std::sqrt(l_yz), l_xz < 0.0f ? F32_MAX : a.y - std::sqrt(l_xz),
                    l_xy < 0.0f ? F32_MAX : a.z - std::sqrt(l_xy));
    }
};

// src/implicit/rectangular_prism.rs:36-80
struct RectangularPrism : Source {
    Vec3 half;
    explicit RectangularPrism(Vec3 h) : half(h) {}
    float scalar(const Vec3& p) const override {
        Vec3 q = p.abs() - half;
        return q.vmax(Vec3()).len() + std::fmin(q.max_component(), 0.0f);
    }
    Vec3 normal(const Vec3& p) const override { return p.clamp_to_cardinal_axis(); }
    bool has_vector() const override { return true; }
    // rectangular_prism.rs:43-70: outside the slab of the other two axes the
    // axis line misses the box (+MAX); the mask is -MAX otherwise
    Vec3 vec(const Vec3& p) const override {
        Vec3 a = p.abs();
        Vec3 mask = Vec3((a.y - half.y > 0.0f || a.z - half.z > 0.0f) ? 1.0f : -1.0f,
                         (a.x - half.x > 0.0f || a.z - half.z > 0.0f) ? 1.0f : -1.0f,
                         (a.x - half.x > 0.0f || a.y - half.y > 0.0f) ? 1.0f : -1.0f) *
                    F32_MAX;
        Vec3 closest = (a.x < half.x && a.y < half.y && a.z < half.z) ? a.vmax(half) : a.vmin(half);
        return (a - closest).vmax(mask);
    }
};

// src/implicit/cylinder.rs:41-85
struct Cylinder : Source {
    float radius, half_length;
    Cylinder(float r, float h) : radius(r), half_length(h) {}
    float scalar(const Vec3& p) const override {
        float xy_len = std::sqrt(p.x * p.x + p.y * p.y);   // Vec2::len, fold of 2
        float q_x = std::fabs(xy_len) - radius;
        float q_z = std::fabs(p.z) - half_length;
        Vec3 d(std::fmax(q_x, 0.0f), std::fmax(q_z, 0.0f), 0.0f);
        return std::fmin(std::fmax(q_x, q_z), 0.0f) + d.len();
    }
    Vec3 normal(const Vec3& p) const override {
        float z = std::fabs(p.z) / half_length;
        float r = std::sqrt(p.x * p.x + p.y * p.y) / radius;
        if (z > r) return Vec3(0.0f, 0.0f, p.z);
        return Vec3(p.x, p.y, 0.0f);
    }
    bool has_vector() const override { return true; }
    // cylinder.rs:50-71
    Vec3 vec(const Vec3& p) const override {
        Vec3 a = p.abs();
        float r2 = radius * radius;
        return Vec3((a.z > half_length || a.y > radius) ? F32_MAX : a.x - std::sqrt(r2 - a.y * a.y),
                    (a.z > half_length || a.x > radius) ? F32_MAX : a.y - std::sqrt(r2 - a.x * a.x),
                    (a.x * a.x + a.y * a.y > r2) ? F32_MAX : a.z - half_length);
    }
};

// src/implicit/torus.rs:40-108
struct Torus : Source {
    float radius, tube;
    Torus(float R, float r) : radius(R), tube(r) {}
    float scalar(const Vec3& p) const override {
        float q_x = std::fabs(std::sqrt(p.x * p.x + p.y * p.y)) - radius;
        float len = std::sqrt(q_x * q_x + p.z * p.z);
        return len - tube;
    }
    Vec3 normal(const Vec3& p) const override {
        Vec3 ring;
        if (!Vec3(p.x, p.y, 0.0f).normalised(&ring)) ring = Vec3(1.0f, 0.0f, 0.0f);
        return p - ring * radius;
    }
    bool has_vector() const override { return true; }
    // torus.rs:48-100.  Square roots of negative numbers give NaN, which
    // f32::max (fmax) drops in favour of the other operand.
    Vec3 vec(const Vec3& p) const override {
        Vec3 a = p.abs();
        float l = std::sqrt(a.x * a.x + a.y * a.y);
        float l_xy = l - radius;
        float trz = std::sqrt(tube * tube - a.z * a.z);
        float rx = radius + trz, ry = radius - trz;
        float x, y, z;
        if (a.z > tube || a.y > radius + trz)
            x = F32_MAX;
        else if (a.x == 0.0f)
            x = std::fabs(a.y - radius) - tube;
        else
            x = std::fmax(a.x - std::sqrt(rx * rx - a.y * a.y), std::sqrt(ry * ry - a.y * a.y) - a.x);
        if (a.z > tube || a.x > radius + trz)
            y = F32_MAX;
        else if (a.y == 0.0f)
            y = std::fabs(a.x - radius) - tube;
        else
            y = std::fmax(a.y - std::sqrt(rx * rx - a.x * a.x), std::sqrt(ry * ry - a.x * a.x) - a.y);
        z = std::fabs(l_xy) > tube ? F32_MAX : a.z - std::sqrt(tube * tube - l_xy * l_xy);
        return Vec3(x, y, z);
    }
};

// src/implicit/csg.rs:22-51: min of values, component-wise min of normals
struct Union : Source {
    SourcePtr a, b;
    Union(SourcePtr x, SourcePtr y) : a(std::move(x)), b(std::move(y)) {}
    float scalar(const Vec3& p) const override { return std::fmin(a->scalar(p), b->scalar(p)); }
    bool has_normal() const override { return a->has_normal() && b->has_normal(); }
    Vec3 normal(const Vec3& p) const override { return a->normal(p).vmin(b->normal(p)); }
    bool has_vector() const override { return a->has_vector() && b->has_vector(); }
    Vec3 vec(const Vec3& p) const override { return a->vec(p).vmin(b->vec(p)); }  // csg.rs:41-45
};

// src/implicit/csg.rs:55-72 (values).  The reference defines no normal; the
// library's analytic normal is the normal of the operand that attains the max.
struct Intersection : Source {
    SourcePtr a, b;
    Intersection(SourcePtr x, SourcePtr y) : a(std::move(x)), b(std::move(y)) {}
    float scalar(const Vec3& p) const override { return std::fmax(a->scalar(p), b->scalar(p)); }
    bool has_normal() const override { return a->has_normal() && b->has_normal(); }
    Vec3 normal(const Vec3& p) const override {
        return (a->scalar(p) >= b->scalar(p)) ? a->normal(p) : b->normal(p);
    }
    bool has_vector() const override { return a->has_vector() && b->has_vector(); }
    Vec3 vec(const Vec3& p) const override { return a->vec(p).vmax(b->vec(p)); }  // csg.rs:74-78
};

// src/implicit/csg.rs:83-100: b minus a == max(b, -a).  Normal (new): normal of
// b where b >= -a, else the negated normal of a.
struct Difference : Source {
    SourcePtr a, b;
    Difference(SourcePtr x, SourcePtr y) : a(std::move(x)), b(std::move(y)) {}
    float scalar(const Vec3& p) const override { return std::fmax(b->scalar(p), -a->scalar(p)); }
    bool has_normal() const override { return a->has_normal() && b->has_normal(); }
    Vec3 normal(const Vec3& p) const override {
        return (b->scalar(p) >= -a->scalar(p)) ? b->normal(p) : -a->normal(p);
    }
    bool has_vector() const override { return a->has_vector() && b->has_vector(); }
    Vec3 vec(const Vec3& p) const override { return b->vec(p).vmax(-a->vec(p)); }  // csg.rs:102-106
};

// Polynomial smooth minimum (Inigo Quilez, "smooth minimum", 2013):
//   h = max(k - |a - b|, 0) / k ;  smin = min(a, b) - h*h*k/4
inline float smooth_min(float a, float b, float k) {
    float h = std::fmax(k - std::fabs(a - b), 0.0f) / k;
    return std::fmin(a, b) - ((h * h) * k) * 0.25f;
}

struct SmoothUnion : Source {
    SourcePtr a, b;
    float k;
    SmoothUnion(SourcePtr x, SourcePtr y, float kk) : a(std::move(x)), b(std::move(y)), k(kk) {}
    float scalar(const Vec3& p) const override { return smooth_min(a->scalar(p), b->scalar(p), k); }
    bool has_normal() const override { return a->has_normal() && b->has_normal(); }
    Vec3 normal(const Vec3& p) const override {
        return (a->scalar(p) <= b->scalar(p)) ? a->normal(p) : b->normal(p);
    }
};

// q = p - c (a Sphere moved off the origin)
struct Translate : Source {
    SourcePtr s;
    Vec3 c;
    Translate(SourcePtr x, Vec3 cc) : s(std::move(x)), c(cc) {}
    float scalar(const Vec3& p) const override { return s->scalar(p - c); }
    bool has_normal() const override { return s->has_normal(); }
    Vec3 normal(const Vec3& p) const override { return s->normal(p - c); }
    bool has_vector() const override { return s->has_vector(); }
    Vec3 vec(const Vec3& p) const override { return s->vec(p - c); }
};

// q = M (p - t); normal rotated back with M^T
struct Rigid : Source {
    SourcePtr s;
    Vec3 t;
    float m[9];
    Rigid(SourcePtr x, Vec3 tt, const float* mm) : s(std::move(x)), t(tt) { std::memcpy(m, mm, sizeof(m)); }
    Vec3 local(const Vec3& p) const {
        Vec3 d = p - t;
        return Vec3((m[0] * d.x + m[1] * d.y) + m[2] * d.z,
                    (m[3] * d.x + m[4] * d.y) + m[5] * d.z,
                    (m[6] * d.x + m[7] * d.y) + m[8] * d.z);
    }
    float scalar(const Vec3& p) const override { return s->scalar(local(p)); }
    bool has_normal() const override { return s->has_normal(); }
    Vec3 normal(const Vec3& p) const override {
        Vec3 n = s->normal(local(p));
        return Vec3((m[0] * n.x + m[3] * n.y) + m[6] * n.z,
                    (m[1] * n.x + m[4] * n.y) + m[7] * n.z,
                    (m[2] * n.x + m[5] * n.y) + m[8] * n.z);
    }
};

// q = p*scale + offset, normal passed through unchanged like the examples'
// DemoSource (examples/common/sources.rs:38-57).
struct DomainMap : Source {
    SourcePtr s;
    Vec3 scale, offset;
    DomainMap(SourcePtr x, Vec3 sc, Vec3 of) : s(std::move(x)), scale(sc), offset(of) {}
    Vec3 map(const Vec3& p) const { return p * scale + offset; }
    float scalar(const Vec3& p) const override { return s->scalar(map(p)); }
    bool has_normal() const override { return s->has_normal(); }
    Vec3 normal(const Vec3& p) const override { return s->normal(map(p)); }
    bool has_vector() const override { return s->has_vector(); }
    Vec3 vec(const Vec3& p) const override { return s->vec(map(p)); }
};

// A left fold of Union (or SmoothUnion) over translated spheres.
struct SphereSet : Source {
    std::vector<float> c;  // cx, cy, cz, r
    int smooth;
    float k;
    size_t count() const { return c.size() / 4; }
    float one(size_t i, const Vec3& p) const {
        Vec3 q = p - Vec3(c[4 * i], c[4 * i + 1], c[4 * i + 2]);
        return q.len() - c[4 * i + 3];
    }
    float scalar(const Vec3& p) const override {
        float v = one(0, p);
        for (size_t i = 1; i < count(); ++i) {
            float s = one(i, p);
            v = smooth ? smooth_min(v, s, k) : std::fmin(v, s);
        }
        return v;
    }
    Vec3 normal(const Vec3& p) const override {
        Vec3 n = p - Vec3(c[0], c[1], c[2]);
        if (!smooth) {
            for (size_t i = 1; i < count(); ++i) n = n.vmin(p - Vec3(c[4 * i], c[4 * i + 1], c[4 * i + 2]));
            return n;
        }
        float v = one(0, p);
        for (size_t i = 1; i < count(); ++i) {
            float s = one(i, p);
            if (!(v <= s)) n = p - Vec3(c[4 * i], c[4 * i + 1], c[4 * i + 2]);
            v = smooth_min(v, s, k);
        }
        return n;
    }
};

// src/source.rs:52-95, epsilon default 1e-6
struct CentralDifference : Source {
    SourcePtr s;
    float eps;
    CentralDifference(SourcePtr x, float e) : s(std::move(x)), eps(e) {}
    float scalar(const Vec3& p) const override { return s->scalar(p); }
    bool has_vector() const override { return s->has_vector(); }
    Vec3 vec(const Vec3& p) const override { return s->vec(p); }  // source.rs:76-80
    Vec3 normal(const Vec3& p) const override {
        Vec3 dx(eps, 0.0f, 0.0f), dy(0.0f, eps, 0.0f), dz(0.0f, 0.0f, eps);
        float vx = s->scalar(p + dx) - s->scalar(p - dx);
        float vy = s->scalar(p + dy) - s->scalar(p - dy);
        float vz = s->scalar(p + dz) - s->scalar(p - dz);
        return Vec3(vx, vy, vz) / (2.0f * eps);
    }
};

// ---------------------------------------------------------------------------
// Program parsing (format: include/isosurface_gpu.h, "Source programs").
// ---------------------------------------------------------------------------
enum {
    OP_PT_DOMAIN = 0x01, OP_PT_TRANSLATE = 0x02, OP_PT_RIGID = 0x03, OP_PT_POP = 0x04,
    OP_SPHERE = 0x10, OP_BOX = 0x11, OP_CYLINDER = 0x12, OP_TORUS = 0x13,
    OP_UNION = 0x20, OP_INTERSECTION = 0x21, OP_DIFFERENCE = 0x22, OP_SMOOTH_UNION = 0x23,
    OP_SPHERE_SET = 0x30, OP_CD_BEGIN = 0x40, OP_CD_END = 0x41,
};

// Builds the tree recursively from the postfix program: a point op opens a
// scope that closes at its matching PT_POP and wraps the single value that the
// scope leaves on the value stack.
struct ProgramParser {
    const uint32_t* ops;
    uint32_t n_ops;
    const float* k;
    uint32_t n_consts;
    std::string err;

    bool arg(uint32_t a, uint32_t n) {
        if ((uint64_t)a + n > n_consts) { err = "constant index out of range"; return false; }
        return true;
    }

    // parse ops[pc..end) leaving exactly one value; returns nullptr on error
    SourcePtr parse(uint32_t& pc, uint32_t end, uint32_t stop_op) {
        std::vector<SourcePtr> st;
        while (pc < end) {
            uint32_t w = ops[pc];
            uint32_t op = w & 0xFF, a = w >> 8;
            if (op == stop_op) break;
            ++pc;
            switch (op) {
            case OP_PT_DOMAIN: case OP_PT_TRANSLATE: case OP_PT_RIGID: {
                uint32_t need = op == OP_PT_DOMAIN ? 6 : op == OP_PT_TRANSLATE ? 3 : 12;
                if (!arg(a, need)) return nullptr;
                SourcePtr inner = parse(pc, end, OP_PT_POP);
                if (!inner) return nullptr;
                if (pc >= end || (ops[pc] & 0xFF) != OP_PT_POP) { err = "point scope without PT_POP"; return nullptr; }
                ++pc;
                if (op == OP_PT_DOMAIN)
                    st.emplace_back(new DomainMap(std::move(inner), Vec3(k[a], k[a + 1], k[a + 2]), Vec3(k[a + 3], k[a + 4], k[a + 5])));
                else if (op == OP_PT_TRANSLATE)
                    st.emplace_back(new Translate(std::move(inner), Vec3(k[a], k[a + 1], k[a + 2])));
                else
                    st.emplace_back(new Rigid(std::move(inner), Vec3(k[a], k[a + 1], k[a + 2]), k + a + 3));
                break;
            }
            case OP_CD_BEGIN: {
                if (!arg(a, 1)) return nullptr;
                SourcePtr inner = parse(pc, end, OP_CD_END);
                if (!inner) return nullptr;
                if (pc >= end || (ops[pc] & 0xFF) != OP_CD_END) { err = "CD_BEGIN without CD_END"; return nullptr; }
                ++pc;
                st.emplace_back(new CentralDifference(std::move(inner), k[a]));
                break;
            }
            case OP_SPHERE:
                if (!arg(a, 1)) return nullptr;
                st.emplace_back(new Sphere(k[a]));
                break;
            case OP_BOX:
                if (!arg(a, 3)) return nullptr;
                st.emplace_back(new RectangularPrism(Vec3(k[a], k[a + 1], k[a + 2])));
                break;
            case OP_CYLINDER:
                if (!arg(a, 2)) return nullptr;
                st.emplace_back(new Cylinder(k[a], k[a + 1]));
                break;
            case OP_TORUS:
                if (!arg(a, 2)) return nullptr;
                st.emplace_back(new Torus(k[a], k[a + 1]));
                break;
            case OP_UNION: case OP_INTERSECTION: case OP_DIFFERENCE: case OP_SMOOTH_UNION: {
                if (st.size() < 2) { err = "binary op needs two operands"; return nullptr; }
                SourcePtr b = std::move(st.back()); st.pop_back();
                SourcePtr x = std::move(st.back()); st.pop_back();
                if (op == OP_UNION) st.emplace_back(new Union(std::move(x), std::move(b)));
                else if (op == OP_INTERSECTION) st.emplace_back(new Intersection(std::move(x), std::move(b)));
                else if (op == OP_DIFFERENCE) st.emplace_back(new Difference(std::move(x), std::move(b)));
                else {
                    if (!arg(a, 1)) return nullptr;
                    st.emplace_back(new SmoothUnion(std::move(x), std::move(b), k[a]));
                }
                break;
            }
            case OP_SPHERE_SET: {
                if (!arg(a, 3)) return nullptr;
                float fn = k[a];
                if (!(fn >= 1.0f) || fn != std::floor(fn)) { err = "bad sphere count"; return nullptr; }
                uint32_t n = (uint32_t)fn;
                if (!arg(a + 3, 4 * n)) return nullptr;
                SphereSet* s = new SphereSet();
                s->smooth = k[a + 1] != 0.0f;
                s->k = k[a + 2];
                s->c.assign(k + a + 3, k + a + 3 + 4 * n);
                st.emplace_back(s);
                break;
            }
            default:
                err = "unknown opcode";
                return nullptr;
            }
        }
        if (st.size() != 1) { err = "scope must leave exactly one value"; return nullptr; }
        return std::move(st.back());
    }
};

inline SourcePtr parse_program(const uint8_t* bytes, size_t len, std::string* err) {
    if (len < 16) { *err = "program shorter than its header"; return nullptr; }
    uint32_t h[4];
    std::memcpy(h, bytes, 16);
    if (h[0] != 0x314F5349u) { *err = "bad magic"; return nullptr; }
    uint64_t need = 16 + 4ull * h[1] + 4ull * h[2];
    if (need != len) { *err = "length does not match header"; return nullptr; }
    std::vector<uint32_t> ops(h[1]);
    std::vector<float> consts(h[2]);
    if (h[1]) std::memcpy(ops.data(), bytes + 16, 4ull * h[1]);
    if (h[2]) std::memcpy(consts.data(), bytes + 16 + 4ull * h[1], 4ull * h[2]);
    ProgramParser p{ops.data(), h[1], consts.data(), h[2], ""};
    uint32_t pc = 0;
    SourcePtr s = p.parse(pc, h[1], 0x100);
    if (s && pc != h[1]) { p.err = "trailing ops"; s.reset(); }
    if (!s) *err = p.err;
    return s;
}

}  // namespace oracle
