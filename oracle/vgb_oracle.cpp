// vgb_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement of Vira's CPU path tracer (the oracle).  Only tests/, the
// smoke check of __graft_entry__.py and the cpu_baseline / reference legs of bench.py
// load it, and only as the checker or the timed CPU baseline.  The product
// (vira_gb300, libvgb.so) never calls it.
//
// The reference (Vira 0.8.3) is a header-only C++ library whose path tracer needs
// Embree 3.13.5, TBB and glm, none of which is available, so it cannot be compiled
// here.  This file restates the reference's arithmetic in plain C++ with glm's
// evaluation order written out, compiled with -ffp-contract=off:
//
//   unidirectional / simulatePath / processIntersection / PowerHeuristic /
//   computeShadingPoint      include/implementation/rendering/cpu_path_tracer.ipp:170-511
//   offsetIntersection       include/implementation/rendering/ray.ipp:107-139
//   Camera::pixelToRay       include/implementation/cameras/camera.ipp:1126-1163,1738-1749
//   initializeIntrinsicMatrix / initializePixelSolidAngle   camera.ipp:1526-1666
//   SphereLight::sample / getPDF   include/implementation/lights/sphere_light.ipp:31-153
//   Lambertian::evaluateBSDF include/implementation/materials/lambertian.ipp:7-15
//   cosine sampling          include/vira/materials/material_sampling.hpp:15-30,
//                            include/implementation/sampling.ipp:53-88
//   Image::sampleUVs         include/implementation/images/image.ipp:589-671
//   Mesh::calculateNormals   include/implementation/geometry/mesh.ipp:199-233
//   DEM::makeVertexBuffer    include/implementation/dems/dem.ipp:165-211,
//                            dem_projection.ipp:131-141, image_utils.ipp:364-409
//   blackBodyRadiance        include/implementation/spectral_data.ipp:613-629, math.ipp:34-59
//   ViraBLAS build/traverse  include/implementation/rendering/acceleration/vira_blas.ipp:43-254
//   Triangle::intersect      include/implementation/geometry/triangle.ipp:35-87
//   LZ4 block decoding and the DEM Quipu normal cone (quipu_io.ipp:216-231,
//                            dem_quipu.ipp:256-270); the Quipu format itself is restated in
//                            oracle/quipu.py
//
// Two things cannot be restated and are replaced, identically in oracle and product:
//   * Embree's rtcIntersect1 arithmetic (third party, not vendored).  The oracle uses the
//     watertight ray/triangle test of Woop, Benthin & Wald (JCGT 2(1), 2013) and breaks
//     ties in t by the smaller triangle id, so the closest hit does not depend on the BVH.
//     mode 1 of oracle_trace runs the reference's own Triangle::intersect instead; the
//     primary rays on which the two disagree are the reported edge-grazing count.
//   * std::mt19937 seeded from the thread id and the clock (cpu_path_tracer.ipp:67-70),
//     which is not reproducible.  The oracle uses Philox-4x32-10 (Salmon et al., SC 2011)
//     keyed by (seed, frame) with the counter (pixel, sample, frame, bounce<<8 | slot).
//
// PARITY PINNING: the reference ships no golden vectors, known-answer tests or fixtures
// for this path (its tests cover Vulkan mocks and unit conversion only), and it cannot
// be built here, so parity with the reference is UNPINNED by its own outputs.  The oracle
// is pinned instead by analytic known-answer cases derived from the reference formulas
// (flat plane under the sun: radiance = albedo/pi * cos^2 * L * Omega_fp32) and by the
// committed golden fixtures under tests/golden/.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

#include "../include/vgb.h"

#define OAPI extern "C" __attribute__((visibility("default")))

namespace {

constexpr float PI_F = 3.14159265358979323846f;
constexpr float INV_PI_F = (float)(1. / 3.141592653589793238462);
constexpr float INF_F = std::numeric_limits<float>::infinity();

// ---------------------------------------------------------------- glm-order vector math
struct V3 { float x, y, z; };
static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3 operator*(float s, V3 a) { return {s * a.x, s * a.y, s * a.z}; }
static inline V3 operator*(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
static inline float dot(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3 cross(V3 a, V3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
static inline float length(V3 a) { return std::sqrt(dot(a, a)); }
static inline V3 normalize(V3 a) { return a * (1.0f / std::sqrt(dot(a, a))); }
static inline float comp(V3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
// column-major 3x3 times vector, glm order
static inline V3 mat3_mul(const float* m, V3 v) {
    return {(m[0] * v.x + m[3] * v.y) + m[6] * v.z,
            (m[1] * v.x + m[4] * v.y) + m[7] * v.z,
            (m[2] * v.x + m[5] * v.y) + m[8] * v.z};
}

struct V3d { double x, y, z; };
static inline V3d operator-(V3d a, V3d b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline double dotd(V3d a, V3d b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline V3d crossd(V3d a, V3d b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
static inline V3d normalized(V3d a) {
    double s = 1.0 / std::sqrt(dotd(a, a));
    return {a.x * s, a.y * s, a.z * s};
}

// ---------------------------------------------------------------- Philox-4x32-10
struct U4 { uint32_t v[4]; };
static inline U4 philox(U4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += W0; k1 += W1; }
        uint64_t p0 = (uint64_t)M0 * c.v[0];
        uint64_t p1 = (uint64_t)M1 * c.v[2];
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        U4 n;
        n.v[0] = hi1 ^ c.v[1] ^ k0;
        n.v[1] = lo1;
        n.v[2] = hi0 ^ c.v[3] ^ k1;
        n.v[3] = lo0;
        c = n;
    }
    return c;
}
static inline float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

enum : uint32_t { SLOT_MAIN = 0u, SLOT_RR = 0xFEu, SLOT_JITTER = 0xFFu };

struct Rng {
    uint32_t k0, k1, pixel, sample, frame;
    U4 draw(uint32_t bounce, uint32_t slot) const {
        U4 c{{pixel, sample, frame, (bounce << 8) | slot}};
        return philox(c, k0, k1);
    }
};

// ---------------------------------------------------------------- scene
struct Scene {
    uint32_t nverts = 0, ntris = 0, nbands = 1;
    std::vector<V3> pos, nrm;
    std::vector<float> uv;       // 2 per vertex
    std::vector<float> albedo;   // B per vertex
    std::vector<uint32_t> idx;
    std::vector<float> tex;      // [th][tw][B]
    uint32_t tw = 1, th = 1;
    std::vector<float> nmap;     // [nh][nw][3] tangent-space normal map (Material::normalMap), or empty
    uint32_t nw = 0, nh = 0;
    std::vector<vgb_instance_motion> motion;   // ascending first_triangle, or empty (all at rest)
    // BVH2, vira_blas layout: leaf when count > 0
    struct Node { float lo[3], hi[3]; uint32_t left_first, count; };
    std::vector<Node> nodes;
    std::vector<uint32_t> tri_idx;
    std::vector<V3d> centroid;
};

// glm::normalize over the mesh.ipp loop
static void compute_normals(const float* p, uint32_t nv, const uint32_t* idx, uint32_t nt,
                            float* out) {
    std::vector<V3> n(nv, V3{0.f, 0.f, 0.f});
    for (uint32_t t = 0; t < nt; ++t) {
        uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
        V3 p0{p[3 * i0], p[3 * i0 + 1], p[3 * i0 + 2]};
        V3 p1{p[3 * i1], p[3 * i1 + 1], p[3 * i1 + 2]};
        V3 p2{p[3 * i2], p[3 * i2 + 1], p[3 * i2 + 2]};
        if (!std::isinf(p0.x) && !std::isinf(p1.x) && !std::isinf(p2.x)) {
            V3 fn = normalize(cross(p1 - p0, p2 - p0));
            if (!std::isnan(fn.x) && !std::isnan(fn.y) && !std::isnan(fn.z)) {
                n[i0] = n[i0] + fn;
                n[i1] = n[i1] + fn;
                n[i2] = n[i2] + fn;
            }
        }
    }
    for (uint32_t v = 0; v < nv; ++v) {
        V3 a = n[v];
        if (length(a) != 0.f) a = normalize(a);
        out[3 * v] = a.x; out[3 * v + 1] = a.y; out[3 * v + 2] = a.z;
    }
}

// ---------------------------------------------------------------- ViraBLAS build (restated)
struct Aabbd {
    double lo[3] = {INFINITY, INFINITY, INFINITY};
    double hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const V3& p) {
        double q[3] = {p.x, p.y, p.z};
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], q[k]); hi[k] = std::max(hi[k], q[k]); }
    }
    void grow(const Aabbd& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    double area() const {
        double e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
        return e0 * e1 + e1 * e2 + e2 * e0;
    }
};

struct Builder {
    Scene& s;
    std::vector<Aabbd> box;
    std::atomic<uint32_t> used{1};
    explicit Builder(Scene& sc) : s(sc) {}

    void tri_grow(Aabbd& b, uint32_t t) const {
        b.grow(s.pos[s.idx[3 * t]]); b.grow(s.pos[s.idx[3 * t + 1]]); b.grow(s.pos[s.idx[3 * t + 2]]);
    }
    void bounds(uint32_t ni) {
        Aabbd b;
        auto& n = s.nodes[ni];
        for (uint32_t i = 0; i < n.count; ++i) tri_grow(b, s.tri_idx[n.left_first + i]);
        box[ni] = b;
    }
    // vira_blas.ipp:186-254: 8 bins on the longest axis of the node box
    double best_split(uint32_t ni, int& axis, double& split) {
        auto& n = s.nodes[ni];
        const Aabbd& nb = box[ni];
        int a = 0;
        double ex = nb.hi[0] - nb.lo[0], ey = nb.hi[1] - nb.lo[1], ez = nb.hi[2] - nb.lo[2];
        double e[3] = {ex, ey, ez};
        if (e[1] > e[0]) a = 1;
        if (e[2] > e[a]) a = 2;
        double bmin = INFINITY, bmax = -INFINITY;
        for (uint32_t i = 0; i < n.count; ++i) {
            double c = (&s.centroid[s.tri_idx[n.left_first + i]].x)[a];
            bmin = std::min(bmin, c); bmax = std::max(bmax, c);
        }
        const int BINS = 8;
        Aabbd bb[BINS]; uint32_t bc[BINS] = {0};
        double scale = BINS / (bmax - bmin);
        for (uint32_t i = 0; i < n.count; ++i) {
            uint32_t t = s.tri_idx[n.left_first + i];
            double c = (&s.centroid[t].x)[a];
            size_t bi = std::min((size_t)(BINS - 1), (size_t)((c - bmin) * scale));
            bc[bi]++; tri_grow(bb[bi], t);
        }
        double la[BINS - 1], ra[BINS - 1]; uint32_t lc[BINS - 1], rc[BINS - 1];
        Aabbd lb, rb; uint32_t ls = 0, rs = 0;
        for (int i = 0; i < BINS - 1; ++i) {
            ls += bc[i]; lc[i] = ls; lb.grow(bb[i]); la[i] = lb.area();
            rs += bc[BINS - 1 - i]; rc[BINS - 2 - i] = rs; rb.grow(bb[BINS - 1 - i]);
            ra[BINS - 2 - i] = rb.area();
        }
        double best = std::numeric_limits<double>::max();
        scale = (bmax - bmin) / BINS;
        for (int i = 0; i < BINS - 1; ++i) {
            // empty sides give 0*inf = NaN in the reference, which never wins the '<'
            double cost = (double)lc[i] * la[i] + (double)rc[i] * ra[i];
            if (cost < best) { axis = a; split = bmin + scale * (double)(i + 1); best = cost; }
        }
        return best;
    }
    void subdivide(uint32_t ni, int depth) {
        auto& n = s.nodes[ni];
        if (n.count <= 2) return;
        int axis = 0; double split = 0;
        double cost = best_split(ni, axis, split);
        const Aabbd& nb = box[ni];
        double ex = nb.hi[0] - nb.lo[0], ey = nb.hi[1] - nb.lo[1], ez = nb.hi[2] - nb.lo[2];
        double node_cost = (double)n.count * (ex * ey + ey * ez + ez * ex);
        if (cost >= node_cost) return;
        // in-place partition, vira_blas.ipp:150-159
        int64_t i = n.left_first, j = (int64_t)n.left_first + n.count - 1;
        while (i <= j) {
            if ((&s.centroid[s.tri_idx[i]].x)[axis] < split) i++;
            else std::swap(s.tri_idx[i], s.tri_idx[j--]);
        }
        uint32_t left_count = (uint32_t)(i - n.left_first);
        if (left_count == 0 || left_count == n.count) return;
        uint32_t l = used.fetch_add(2);
        uint32_t r = l + 1;
        s.nodes[l].left_first = n.left_first; s.nodes[l].count = left_count;
        s.nodes[r].left_first = (uint32_t)i;  s.nodes[r].count = n.count - left_count;
        n.left_first = l; n.count = 0;
        bounds(l); bounds(r);
        // parallel recursion on large subtrees; the result is independent of scheduling
        // except for node numbering, which only changes memory order.
        if (depth < 4 && s.nodes[l].count > 100000 && s.nodes[r].count > 100000) {
            std::thread th([this, l, depth] { subdivide(l, depth + 1); });
            subdivide(r, depth + 1);
            th.join();
        } else {
            subdivide(l, depth + 1);
            subdivide(r, depth + 1);
        }
    }
};

static void build_bvh(Scene& s) {
    uint32_t nt = s.ntris;
    s.nodes.assign(nt ? 2 * (size_t)nt - 1 : 1, Scene::Node{});
    s.tri_idx.resize(nt);
    s.centroid.resize(nt);
    for (uint32_t t = 0; t < nt; ++t) {
        s.tri_idx[t] = t;
        const V3 &a = s.pos[s.idx[3 * t]], &b = s.pos[s.idx[3 * t + 1]], &c = s.pos[s.idx[3 * t + 2]];
        // Triangle::init: TMeshFloat{1.f/3.f} * (v0+v1+v2) for the double mesh type
        double third = (double)(1.f / 3.f);
        s.centroid[t] = V3d{third * (((double)a.x + b.x) + c.x), third * (((double)a.y + b.y) + c.y),
                            third * (((double)a.z + b.z) + c.z)};
    }
    Builder b(s);
    b.box.assign(s.nodes.size(), Aabbd{});
    s.nodes[0].left_first = 0; s.nodes[0].count = nt;
    if (nt) { b.bounds(0); b.subdivide(0, 0); }
    s.nodes.resize(b.used.load());
    for (size_t i = 0; i < s.nodes.size(); ++i) {
        for (int k = 0; k < 3; ++k) {
            // round outward so that the float box contains the double box
            s.nodes[i].lo[k] = std::nextafter((float)b.box[i].lo[k], -INF_F);
            s.nodes[i].hi[k] = std::nextafter((float)b.box[i].hi[k], INF_F);
        }
    }
}

// ---------------------------------------------------------------- ray / triangle
struct Hit {
    float t = INF_F;
    uint32_t tri = VGB_NO_HIT;
    float w[3] = {0, 0, 0};  // Interaction::w: weights of {v1, v2, v0}
};

struct WtRay {  // per-ray constants of the watertight test
    V3 o, d;
    int kx, ky, kz;
    float Sx, Sy, Sz;
};
static inline WtRay wt_setup(V3 o, V3 d) {
    WtRay r; r.o = o; r.d = d;
    float ax = std::fabs(d.x), ay = std::fabs(d.y), az = std::fabs(d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (comp(d, kz) < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sx = comp(d, kx) / comp(d, kz);
    r.Sy = comp(d, ky) / comp(d, kz);
    r.Sz = 1.0f / comp(d, kz);
    return r;
}

// Woop-Benthin-Wald watertight test.  Returns false on a miss; t > 0 required (Embree's
// tnear = 0, embree_tlas.ipp:131).  U,V,W are the weights of v0,v1,v2.
static inline bool wt_intersect(const WtRay& r, V3 v0, V3 v1, V3 v2, float& t_out,
                                float& U_out, float& V_out, float& W_out, float& det_out) {
    V3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float Ax = comp(A, r.kx) - r.Sx * comp(A, r.kz);
    float Ay = comp(A, r.ky) - r.Sy * comp(A, r.kz);
    float Bx = comp(B, r.kx) - r.Sx * comp(B, r.kz);
    float By = comp(B, r.ky) - r.Sy * comp(B, r.kz);
    float Cx = comp(C, r.kx) - r.Sx * comp(C, r.kz);
    float Cy = comp(C, r.ky) - r.Sy * comp(C, r.kz);
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        double CxBy = (double)Cx * (double)By, CyBx = (double)Cy * (double)Bx;
        U = (float)(CxBy - CyBx);
        double AxCy = (double)Ax * (double)Cy, AyCx = (double)Ay * (double)Cx;
        V = (float)(AxCy - AyCx);
        double BxAy = (double)Bx * (double)Ay, ByAx = (double)By * (double)Ax;
        W = (float)(BxAy - ByAx);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = U + V + W;
    if (det == 0.0f) return false;
    float Az = r.Sz * comp(A, r.kz);
    float Bz = r.Sz * comp(B, r.kz);
    float Cz = r.Sz * comp(C, r.kz);
    float T = (U * Az + V * Bz) + W * Cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t > 0.0f)) return false;
    t_out = t; U_out = U; V_out = V; W_out = W; det_out = det;
    return true;
}

// The reference's own test (triangle.ipp:47-87), tol = 1e-5.
static inline bool ref_intersect(V3 o, V3 d, V3 v0, V3 v1, V3 v2, float best_t, float& t_out,
                                 float w_out[3]) {
    const float tol = 0.00001f;
    V3 e0 = v0 - v1, e1 = v2 - v0;
    V3 n = cross(e0, e1);
    V3 c = v0 - o;
    V3 rr = cross(d, c);
    float inv_det = 1.0f / dot(n, d);
    float w0 = dot(rr, e1) * inv_det;
    float w1 = dot(rr, e0) * inv_det;
    float w2 = 1.0f - w0 - w1;
    if (w0 >= 0 && w1 >= 0 && w2 >= 0) {
        float t = dot(n, c) * inv_det;
        if (t < best_t && t > tol) { t_out = t; w_out[0] = w0; w_out[1] = w1; w_out[2] = w2; return true; }
    }
    return false;
}

static inline V3 tri_v(const Scene& s, uint32_t t, int k) { return s.pos[s.idx[3 * t + k]]; }

// slab test in double over outward-rounded float boxes: conservative
static inline bool box_hit(const Scene::Node& n, const double o[3], const double inv[3],
                           double tmax_limit, double& tnear) {
    double t0 = 0.0, t1 = tmax_limit;
    for (int k = 0; k < 3; ++k) {
        double a = ((double)n.lo[k] - o[k]) * inv[k];
        double b = ((double)n.hi[k] - o[k]) * inv[k];
        if (std::isnan(a)) a = -INFINITY;
        if (std::isnan(b)) b = INFINITY;
        if (a > b) std::swap(a, b);
        t0 = std::max(t0, a); t1 = std::min(t1, b);
    }
    tnear = t0;
    return t0 <= t1;
}

// closest hit (any_hit = 0) or first hit with t <= tmax (any_hit = 1).
// mode 0: watertight with (t, id) tie-break; mode 1: reference Triangle::intersect.
static Hit trace(const Scene& s, V3 o, V3 d, float tmax, bool any_hit, int mode,
                 uint64_t* nodes_visited = nullptr, uint64_t* tris_tested = nullptr) {
    Hit h;
    if (s.ntris == 0) return h;
    WtRay wr = wt_setup(o, d);
    double od[3] = {o.x, o.y, o.z};
    double inv[3] = {1.0 / (double)d.x, 1.0 / (double)d.y, 1.0 / (double)d.z};
    double limit = any_hit ? (double)tmax : INFINITY;
    uint32_t stack[128];
    int sp = 0;
    uint32_t ni = 0;
    double tn;
    if (!box_hit(s.nodes[0], od, inv, limit, tn)) return h;
    float bestU = 0, bestV = 0, bestW = 0, bestDet = 1;
    while (true) {
        const Scene::Node& n = s.nodes[ni];
        if (nodes_visited) (*nodes_visited)++;
        if (n.count > 0) {
            for (uint32_t i = 0; i < n.count; ++i) {
                uint32_t t = s.tri_idx[n.left_first + i];
                if (tris_tested) (*tris_tested)++;
                V3 v0 = tri_v(s, t, 0), v1 = tri_v(s, t, 1), v2 = tri_v(s, t, 2);
                if (mode == 1) {
                    float tt, ww[3];
                    if (ref_intersect(o, d, v0, v1, v2, h.t, tt, ww)) {
                        if (any_hit && tt > tmax) continue;
                        h.t = tt; h.tri = t; h.w[0] = ww[0]; h.w[1] = ww[1]; h.w[2] = ww[2];
                        if (any_hit) return h;
                    }
                } else {
                    float tt, U, V, W, det;
                    if (wt_intersect(wr, v0, v1, v2, tt, U, V, W, det)) {
                        if (any_hit) {
                            if (tt <= tmax) { h.t = tt; h.tri = t; return h; }
                            continue;
                        }
                        if (tt < h.t || (tt == h.t && t < h.tri)) {
                            h.t = tt; h.tri = t; bestU = U; bestV = V; bestW = W; bestDet = det;
                        }
                    }
                }
            }
            if (sp == 0) break;
            ni = stack[--sp];
            continue;
        }
        uint32_t c1 = n.left_first, c2 = n.left_first + 1;
        double lim = any_hit ? limit : (double)h.t;
        double d1, d2;
        bool h1 = box_hit(s.nodes[c1], od, inv, lim, d1);
        bool h2 = box_hit(s.nodes[c2], od, inv, lim, d2);
        if (h1 && h2) {
            if (d1 > d2) std::swap(c1, c2);
            stack[sp++] = c2;
            ni = c1;
        } else if (h1) {
            ni = c1;
        } else if (h2) {
            ni = c2;
        } else {
            if (sp == 0) break;
            ni = stack[--sp];
        }
        if (sp >= 127) break;  // cannot happen for depth < 127
    }
    if (mode == 0 && h.tri != VGB_NO_HIT) {
        float rcp = 1.0f / bestDet;
        // Interaction::w = {w(v1), w(v2), 1 - w(v1) - w(v2)} (embree_tlas.ipp:159-161)
        h.w[0] = bestV * rcp;
        h.w[1] = bestW * rcp;
        h.w[2] = 1.0f - h.w[0] - h.w[1];
        (void)bestU;
    }
    return h;
}

// ---------------------------------------------------------------- materials / lights
static inline void sample_uvs(const Scene& s, float u, float v, float* out) {
    float rx = (float)s.tw, ry = (float)s.th;
    float px = std::fmod(u * rx, rx), py = std::fmod(v * ry, ry);
    if (px < 0) px += rx;
    if (py < 0) py += ry;
    int x0 = (int)std::floor(px), y0 = (int)std::floor(py);
    x0 = std::min(x0, (int)s.tw - 1); y0 = std::min(y0, (int)s.th - 1);
    int x1 = std::min(x0 + 1, (int)s.tw - 1), y1 = std::min(y0 + 1, (int)s.th - 1);
    float dx = px - (float)x0, dy = py - (float)y0;
    uint32_t B = s.nbands;
    const float* p00 = &s.tex[((size_t)y0 * s.tw + x0) * B];
    const float* p10 = &s.tex[((size_t)y0 * s.tw + x1) * B];
    const float* p01 = &s.tex[((size_t)y1 * s.tw + x0) * B];
    const float* p11 = &s.tex[((size_t)y1 * s.tw + x1) * B];
    float a = (1.f - dx) * (1.f - dy), b = dx * (1.f - dy), c = (1.f - dx) * dy, e = dx * dy;
    for (uint32_t k = 0; k < B; ++k) out[k] = ((a * p00[k] + b * p10[k]) + c * p01[k]) + e * p11[k];
}

// Material::getNormal (materials/material.ipp:129-143): normalMap.sampleUVs(uv) (wrap + bilinear of
// a vec3<float> image, image.ipp:589-671), times tangentToWorld (columns tangent, bitangent, N),
// normalised; N unchanged without a map.
static inline V3 get_normal(const Scene& s, float u, float v, V3 N, V3 tangent, V3 bitangent) {
    if (s.nmap.empty()) return N;
    float rx = (float)s.nw, ry = (float)s.nh;
    float px = std::fmod(u * rx, rx), py = std::fmod(v * ry, ry);
    if (px < 0) px += rx;
    if (py < 0) py += ry;
    int x0 = (int)std::floor(px), y0 = (int)std::floor(py);
    x0 = std::min(x0, (int)s.nw - 1);
    y0 = std::min(y0, (int)s.nh - 1);
    int x1 = std::min(x0 + 1, (int)s.nw - 1), y1 = std::min(y0 + 1, (int)s.nh - 1);
    auto at = [&](int x, int y) {
        const float* q = &s.nmap[((size_t)y * s.nw + x) * 3];
        return V3{q[0], q[1], q[2]};
    };
    float dx = px - (float)x0, dy = py - (float)y0;
    V3 t = (1.f - dx) * (1.f - dy) * at(x0, y0) + dx * (1.f - dy) * at(x1, y0) + (1.f - dx) * dy * at(x0, y1) +
           dx * dy * at(x1, y1);
    V3 w{(tangent.x * t.x + bitangent.x * t.y) + N.x * t.z, (tangent.y * t.x + bitangent.y * t.y) + N.y * t.z,
         (tangent.z * t.x + bitangent.z * t.y) + N.z * t.z};
    return normalize(w);
}

// offsetIntersection (ray.ipp:107-123), float path
static inline float off1(float p, float n) {
    const float origin = 1.f / 32.f, float_scale = 1.f / 65536.f, int_scale = 256.f;
    int32_t of = (int32_t)(int_scale * n);
    int32_t pi; std::memcpy(&pi, &p, 4);
    pi += (p < 0) ? -of : of;
    float pf; std::memcpy(&pf, &pi, 4);
    return (std::fabs(p) < origin) ? p + float_scale * n : pf;
}

static inline float power_heuristic(float fpdf, float gpdf) {
    float f = 1.0f * fpdf, g = 1.0f * gpdf;
    return (f * f) / (f * f + g * g);
}

// SphereLight::getPDF (sphere_light.ipp:127-153)
static inline float light_pdf(const vgb_light& L, V3 p, V3 dir) {
    V3 c{L.position[0], L.position[1], L.position[2]};
    V3 tc = c - p;
    float dc = length(tc);
    float r = L.radius;
    if (dc <= r) return 1.0f / (4.0f * PI_F * r * r);
    V3 tcn{tc.x / dc, tc.y / dc, tc.z / dc};
    float cosmax = std::sqrt(1.0f - (r * r) / (dc * dc));
    float ca = dot(dir, tcn);
    if (ca < cosmax) return 0.0f;
    float r2 = r * r, d2 = dc * dc;
    float omega = 2 * PI_F * (1.0f - std::sqrt(d2 - r2) / dc);
    return 1.0f / omega;
}

// SphereLight::sample: RNG-free (sphere_light.ipp:31-64) or cone sampling (:67-124)
static inline void light_sample(const vgb_light& L, V3 p, bool det, float rand1, float rand2,
                                V3& dir, float& distance, float& pdf) {
    V3 c{L.position[0], L.position[1], L.position[2]};
    V3 ptl = c - p;
    distance = length(ptl);
    float dinv = 1.0f / distance;
    float r = L.radius;
    if (det) {
        dir = dinv * ptl;
        if (distance <= r) {
            if (distance < 1e-3f) dir = V3{1, 0, 0};
            distance = r;
            pdf = 1.0f / (4.0f * PI_F * r * r);
            return;
        }
        float r2 = r * r;
        float omega = 2 * PI_F * (1.f - std::sqrt((distance * distance) - r2) / distance);
        pdf = 1.f / omega;
        return;
    }
    V3 W = dinv * ptl;
    V3 N1{1, 0, 0}, N2{0, 1, 0};
    V3 N = (dot(N1, W) < dot(N2, W)) ? N1 : N2;
    V3 Vv = normalize(cross(W, N));
    V3 U = normalize(cross(W, Vv));
    float phi = 2 * PI_F * rand1;
    float zeta = rand2;
    float cc = r / distance;
    float theta = std::acos(1 - zeta + zeta * std::sqrt(1 - (cc * cc)));
    float sinT = std::sin(theta), sinP = std::sin(phi), cosT = std::cos(theta), cosP = std::cos(phi);
    float a = cosP * sinT, b = cosT, e = sinP * sinT;
    // directionInit * frame, frame columns (U0,W0,V0),(U1,W1,V1),(U2,W2,V2)
    dir = V3{(a * U.x + b * W.x) + e * Vv.x, (a * U.y + b * W.y) + e * Vv.y, (a * U.z + b * W.z) + e * Vv.z};
    float r2 = r * r;
    float omega = 2 * PI_F * (1.f - std::sqrt((distance * distance) - r2) / distance);
    pdf = 1.f / omega;
}

// ConcentricDiskSample + CosineHemisphereSample (sampling.ipp:53-84)
static inline V3 cosine_sample(float rand1, float rand2) {
    float ux = 2.f * rand1 - 1.f, uy = 2.f * rand2 - 1.f;
    float dx, dy;
    const float EPS = 1e-6f;
    if (std::fabs(ux) < EPS && std::fabs(uy) < EPS) {
        dx = 0; dy = 0;
    } else {
        float theta, r;
        const float P4 = PI_F / 4.0f, P2 = PI_F / 2.0f;
        if (std::fabs(ux) > std::fabs(uy)) { r = ux; theta = P4 * (uy / ux); }
        else { r = uy; theta = P2 - P4 * (ux / uy); }
        dx = r * std::cos(theta); dy = r * std::sin(theta);
    }
    float z = std::sqrt(std::max(0.f, 1 - dx * dx - dy * dy));
    return V3{dx, dy, z};
}

struct PixelOut {
    float total[VGB_MAX_BANDS], direct[VGB_MAX_BANDS], indirect[VGB_MAX_BANDS], albedo[VGB_MAX_BANDS];
    V3 normal;
    float depth, alpha;
    uint32_t tri;
    // first-hit passes (DataPayload defaults: 0 velocities, +inf triangle size)
    V3 vel_g{0, 0, 0}, vel_c{0, 0, 0};
    float tsz = INF_F;
};

// renderPasses.save_triangle_size / save_velocity at the first hit (cpu_path_tracer.ipp:356-372):
// vert = {v1, v2, v0}; edge lengths, the longest over Camera::calculateGSD (camera.ipp:1408-1414)
// at |P - camera|; the instance's point velocity v + w x (P - position)
// (reference_frame.ipp:367-373); the camera's point velocity at rotation * p_global (the
// reference passes intersection_global to the camera's localPointToGlobalVelocity), the
// difference taken to the camera frame by the transposed rotation.
static void point_velocities(const Scene& s, const vgb_camera& cam, uint32_t t, V3 P, V3& vel_g, V3& vel_c);

static void first_hit_passes(const Scene& s, const vgb_camera& cam, uint32_t t, V3 P, PixelOut& out) {
    const V3 a = s.pos[s.idx[3 * t + 1]], b = s.pos[s.idx[3 * t + 2]], c = s.pos[s.idx[3 * t]];
    float e01 = length(b - a), e02 = length(c - a), e12 = length(c - b);
    float edge = std::max(e01, std::max(e02, e12));
    float distance = length(P - V3{cam.origin[0], cam.origin[1], cam.origin[2]});
    float gx = distance * cam.sensor_size[0] / (cam.focal_length * (float)cam.width);
    float gy = distance * cam.sensor_size[1] / (cam.focal_length * (float)cam.height);
    out.tsz = edge / std::min(gx, gy);
    point_velocities(s, cam, t, P, out.vel_g, out.vel_c);
}

// The instance's point velocity at P and the velocity relative to the camera in the camera frame
// (the path tracer's first hit, cpu_path_tracer.ipp:365-371, and the rasterizer's fragment,
// cpu_rasterizer.ipp:213-218, compute the same).
static void point_velocities(const Scene& s, const vgb_camera& cam, uint32_t t, V3 P, V3& vel_g, V3& vel_c) {
    V3 v{0, 0, 0}, w{0, 0, 0}, o{0, 0, 0};
    for (const vgb_instance_motion& m : s.motion)
        if (m.first_triangle <= t) {
            v = V3{m.velocity[0], m.velocity[1], m.velocity[2]};
            w = V3{m.angular_rate[0], m.angular_rate[1], m.angular_rate[2]};
            o = V3{m.position[0], m.position[1], m.position[2]};
        }
    vel_g = v + cross(w, P - o);
    V3 rp = mat3_mul(cam.rotation, P) + V3{cam.rot_origin[0], cam.rot_origin[1], cam.rot_origin[2]};
    V3 cv = V3{cam.velocity[0], cam.velocity[1], cam.velocity[2]} +
            cross(V3{cam.angular_rate[0], cam.angular_rate[1], cam.angular_rate[2]}, rp);
    V3 rv = vel_g - cv;
    const float* R = cam.rotation;
    vel_c = V3{(R[0] * rv.x + R[1] * rv.y) + R[2] * rv.z, (R[3] * rv.x + R[4] * rv.y) + R[5] * rv.z,
               (R[6] * rv.x + R[7] * rv.y) + R[8] * rv.z};
}

struct RenderCounters { uint64_t closest = 0, shadow = 0; };

// ---------------------------------------------------------------- camera rays
// Lens distortion (cameras/distortions/{brown,opencv,owen}_distortion.ipp), FP32, the
// reference's operation order; Pixel is glm's vec2<float>.
struct Pix { float x, y; };
static Pix brown_delta(const float* k, Pix h) {                 // brown_distortion.ipp:24-44
    float x = h.x, y = h.y;
    float r = std::sqrt(x * x + y * y);
    float r2 = r * r, r4 = r2 * r2, r6 = r2 * r2 * r2;
    float s = (k[0] * r2 + k[1] * r4 + k[2] * r6);
    Pix rad{s * x, s * y};
    Pix tan{(2 * k[3] * x * y) + (k[4] * (r2 + 2 * x * x)), (k[3] * (r2 + 2 * y * y)) + (2 * k[4] * x * y)};
    return Pix{rad.x + tan.x, rad.y + tan.y};
}
static Pix opencv_distort(const float* k, Pix h) {              // opencv_distortion.ipp:28-54
    float x = h.x, y = h.y;
    float r = std::sqrt(x * x + y * y);
    float r2 = r * r, r4 = r2 * r2, r6 = r2 * r2 * r2;
    float numerator = 1 + k[0] * r2 + k[1] * r4 + k[2] * r6;
    float denominator = 1 + k[3] * r2 + k[4] * r4 + k[5] * r6;
    float f = numerator / denominator;
    Pix tp{(2 * k[6] * x * y) + (k[7] * (r2 + 2 * x * x)) + (k[8] * r2) + (k[9] * r4),
           (k[6] * (r2 + 2 * y * y)) + (2 * k[7] * x * y) + (k[10] * r2) + (k[11] * r4)};
    return Pix{f * x + tp.x, f * y + tp.y};
}
static Pix owen_delta(const float* e, Pix h) {                  // owen_distortion.ipp:24-46
    float x = h.x, y = h.y;
    float r = std::sqrt(x * x + y * y);
    float r2 = r * r, r3 = r * r * r;
    float rf = (e[1] * r2) + (e[3] * r2 * r2) + (e[4] * y) + (e[5] * x);
    float of = (e[0] * r) + (e[2] * r3);
    Pix rot{-y, x};
    return Pix{rf * x + of * rot.x, rf * y + of * rot.y};
}
static Pix compute_delta(const vgb_camera& c, Pix h) {
    if (c.distortion == VGB_DISTORTION_BROWN) return brown_delta(c.distortion_coeffs, h);
    if (c.distortion == VGB_DISTORTION_OWEN) return owen_delta(c.distortion_coeffs, h);
    Pix d = opencv_distort(c.distortion_coeffs, h);              // OpenCV: h - distort(h)
    return Pix{h.x - d.x, h.y - d.y};
}
static Pix undistort(const vgb_camera& c, Pix h) {              // 20 fixed-point iterations
    Pix u = h;
    for (size_t i = 0; i < 20; ++i) {
        Pix d = compute_delta(c, u);
        u = Pix{h.x - d.x, h.y - d.y};
    }
    return u;
}
static Pix distort(const vgb_camera& c, Pix h) {
    if (c.distortion == VGB_DISTORTION_OPENCV) return opencv_distort(c.distortion_coeffs, h);
    Pix d = compute_delta(c, h);
    return Pix{h.x + d.x, h.y + d.y};
}
// Camera::pixelToDirectionHelper (camera.ipp:1738-1749)
static V3 direction_helper(const vgb_camera& cam, float X, float Y) {
    const float* K = cam.kinv;
    Pix h{(K[0] * X + K[2] * Y) + K[4] * 1.0f, (K[1] * X + K[3] * Y) + K[5] * 1.0f};
    if (cam.distortion) h = undistort(cam, h);
    return V3{h.x, cam.z_dir * h.y, cam.z_dir};
}
// Camera::pixelToRay (camera.ipp:1105-1163) for one camera: the direction table of
// precomputePixelDirections (:1676-1700) when a distortion is interpolated, Image::interpolatePixel
// (image.ipp:619-671) over it, and the depth-of-field overload for samples >= 1.
struct CameraRays {
    const vgb_camera& cam;
    std::vector<V3> table;   // [H][W] normalize(direction_helper(i, j))
    CameraRays(const vgb_camera& c, int nthreads) : cam(c) {
        if (!(c.distortion && c.interpolate_directions)) return;
        const uint32_t W = c.width, H = c.height;
        table.resize((size_t)W * H);
        auto work = [&](uint32_t j0, uint32_t j1) {
            for (uint32_t j = j0; j < j1; ++j)
                for (uint32_t i = 0; i < W; ++i) table[(size_t)j * W + i] = normalize(direction_helper(c, (float)i, (float)j));
        };
        int nt = std::max(1, nthreads);
        std::vector<std::thread> th;
        for (int t = 0; t < nt; ++t) th.emplace_back(work, H * t / nt, H * (t + 1) / nt);
        for (auto& x : th) x.join();
    }
    V3 direction(float X, float Y) const {
        if (table.empty()) return direction_helper(cam, X, Y);
        int x0 = (int)std::floor(X), y0 = (int)std::floor(Y);
        x0 = std::min(x0, (int)cam.width - 1);
        y0 = std::min(y0, (int)cam.height - 1);
        int x1 = std::min(x0 + 1, (int)cam.width - 1), y1 = std::min(y0 + 1, (int)cam.height - 1);
        const V3 p00 = table[(size_t)y0 * cam.width + x0], p10 = table[(size_t)y0 * cam.width + x1];
        const V3 p01 = table[(size_t)y1 * cam.width + x0], p11 = table[(size_t)y1 * cam.width + x1];
        float dx = X - (float)x0, dy = Y - (float)y0;
        return (1.f - dx) * (1.f - dy) * p00 + dx * (1.f - dy) * p10 + (1.f - dx) * dy * p01 + dx * dy * p11;
    }
    // the ray of pixel (i, j) for `sample` (cpu_path_tracer.ipp:182-192)
    void ray(uint32_t i, uint32_t j, uint32_t sample, const Rng& rng, V3& ro, V3& dir) const {
        float X = (float)i, Y = (float)j;
        U4 jr{{0, 0, 0, 0}};
        if (sample != 0) {
            jr = rng.draw(0, SLOT_JITTER);
            X = X + u01(jr.v[0]);
            Y = Y + u01(jr.v[1]);
        }
        V3 d = direction(X, Y);
        ro = V3{cam.origin[0], cam.origin[1], cam.origin[2]};
        if (sample != 0 && cam.depth_of_field) {
            float rand1 = u01(jr.v[2]), rand2 = u01(jr.v[3]);   // UniformDiskSample (sampling.ipp:43-52)
            float r = std::sqrt(rand1);
            float theta = 2 * PI_F * rand2;
            float ax = cam.aperture_radius * (r * std::cos(theta)), ay = cam.aperture_radius * (r * std::sin(theta));
            V3 offset{ax, ay, cam.focal_length};
            ro = ro + mat3_mul(cam.rotation, offset);
            if (!std::isinf(cam.focus_distance)) d = (cam.focus_distance * normalize(d)) - offset;
        }
        dir = normalize(mat3_mul(cam.rotation, d));
    }
};

// one pixel: unidirectional() with simulatePath()/processIntersection() inlined
static void render_pixel(const Scene& s, const CameraRays& cr, const vgb_light* lights,
                         uint32_t nlights, const vgb_pt_options& o, uint32_t i, uint32_t j,
                         PixelOut& out, RenderCounters& rc) {
    const vgb_camera& cam = cr.cam;
    const uint32_t B = s.nbands;
    Rng rng{(uint32_t)o.seed, (uint32_t)(o.seed >> 32), j * cam.width + i, 0, o.frame};
    float radiance[VGB_MAX_BANDS] = {0}, direct[VGB_MAX_BANDS] = {0}, albedo_acc[VGB_MAX_BANDS] = {0};
    V3 normal_acc{0, 0, 0};
    float depth = 0;
    uint32_t count = 0, tri_first = VGB_NO_HIT;
    bool first_hit = true;
    float s1 = 0.f, s2 = 0.f;   // adaptive sampling sums
    uint32_t sample;
    for (sample = 0; sample < o.samples; ++sample) {
        rng.sample = sample;
        V3 ro, dir;
        cr.ray(i, j, sample, rng, ro, dir);
        float path[VGB_MAX_BANDS] = {0};
        float thr[VGB_MAX_BANDS];
        for (uint32_t k = 0; k < B; ++k) thr[k] = 1.f;
        for (uint32_t bounce = 0; bounce < o.bounces + 1; ++bounce) {
            Hit h = trace(s, ro, dir, INF_F, false, 0);
            rc.closest++;
            if (std::isinf(h.t)) {
                if (o.simulate_lighting && o.show_background) {
                    float x = dir.x, y = dir.y, z = dir.z;
                    float u = std::atan2(y, x) / (2 * PI_F);
                    float v = std::atan2(std::sqrt(x * x + y * y), z) / PI_F;
                    float px = std::fmod(u * 1.f, 1.f), py = std::fmod(v * 1.f, 1.f);
                    if (px < 0) px += 1.f;
                    if (py < 0) py += 1.f;
                    float dx = px - 0.f, dy = py - 0.f;
                    float a = (1.f - dx) * (1.f - dy), b = dx * (1.f - dy), c = (1.f - dx) * dy, e = dx * dy;
                    for (uint32_t k = 0; k < B; ++k) {
                        float bg = ((a * o.background[k] + b * o.background[k]) + c * o.background[k]) + e * o.background[k];
                        path[k] += thr[k] * (bg * 1.f);
                    }
                }
                break;
            }
            // ---- processIntersection
            uint32_t t = h.tri;
            uint32_t i0 = s.idx[3 * t], i1 = s.idx[3 * t + 1], i2 = s.idx[3 * t + 2];
            // vert = {v1, v2, v0}
            uint32_t vi[3] = {i1, i2, i0};
            const float* w = h.w;
            float uvx = 0, uvy = 0;
            {
                const float* a = &s.uv[2 * vi[0]]; const float* b = &s.uv[2 * vi[1]]; const float* c = &s.uv[2 * vi[2]];
                uvx = (w[0] * a[0] + w[1] * b[0]) + w[2] * c[0];
                uvy = (w[0] * a[1] + w[1] * b[1]) + w[2] * c[1];
            }
            V3 p0 = s.pos[i0], p1 = s.pos[i1], p2 = s.pos[i2];
            // Triangle::init (triangle.ipp:39-43): face_normal = -normalize(cross(v0-v1, v2-v0))
            V3 fnn = normalize(cross(p0 - p1, p2 - p0));
            V3 face_normal{-fnn.x, -fnn.y, -fnn.z};
            V3 N_local = face_normal;
            if (o.smooth_shading) {
                V3 n0 = s.nrm[vi[0]], n1 = s.nrm[vi[1]], n2 = s.nrm[vi[2]];
                N_local = normalize((w[0] * n0 + w[1] * n1) + w[2] * n2);
            }
            V3 N = N_local;  // normal matrix is the identity in the flattened scene frame
            V3 arb = (std::fabs(N.x) < 0.9f) ? V3{1, 0, 0} : V3{0, 1, 0};
            V3 tangent = normalize(cross(arb, N));
            V3 bitangent = cross(N, tangent);
            const V3 N_frame = N;   // tangent_to_global's third column, built before the normal map
            N = get_normal(s, uvx, uvy, N, tangent, bitangent);
            float alb[VGB_MAX_BANDS], texv[VGB_MAX_BANDS];
            sample_uvs(s, uvx, uvy, texv);
            for (uint32_t k = 0; k < B; ++k) {
                float va = (w[0] * s.albedo[(size_t)vi[0] * B + k] + w[1] * s.albedo[(size_t)vi[1] * B + k]) +
                           w[2] * s.albedo[(size_t)vi[2] * B + k];
                alb[k] = va * texv[k];
            }
            V3 P = (w[0] * s.pos[vi[0]] + w[1] * s.pos[vi[1]]) + w[2] * s.pos[vi[2]];
            {   // computeShadingPoint (cpu_path_tracer.ipp:494-511)
                V3 q[3];
                for (int k = 0; k < 3; ++k) {
                    V3 vp = s.pos[vi[k]], vn = s.nrm[vi[k]];
                    q[k] = P - dot(P - vp, vn) * vn;
                }
                V3 sp = (q[0] * w[0] + q[1] * w[1]) + q[2] * w[2];
                V3 diff = sp - P;
                if (dot(diff, N_local) > 0) P = sp;
            }
            if (bounce == 0) {
                if (first_hit) {
                    tri_first = t;
                    first_hit = false;
                    first_hit_passes(s, cam, t, P, out);
                }
                for (uint32_t k = 0; k < B; ++k) albedo_acc[k] += alb[k];
                normal_acc = normal_acc + N;
                depth += h.t;
                count++;
            }
            float rad[VGB_MAX_BANDS] = {0};
            if (o.simulate_lighting) {
                P = V3{off1(P.x, face_normal.x), off1(P.y, face_normal.y), off1(P.z, face_normal.z)};
                if (bounce == 0 && o.has_ambient)
                    for (uint32_t k = 0; k < B; ++k) rad[k] += thr[k] * (o.ambient[k] * alb[k]);
                U4 r0 = rng.draw(bounce, SLOT_MAIN);
                for (uint32_t l = 0; l < nlights; ++l) {
                    float ru1, ru2;
                    if (l == 0) { ru1 = u01(r0.v[0]); ru2 = u01(r0.v[1]); }
                    else { U4 rl = rng.draw(bounce, 1 + l); ru1 = u01(rl.v[0]); ru2 = u01(rl.v[1]); }
                    V3 Ld; float dist, lpdf = 0;
                    light_sample(lights[l], P, o.deterministic_light != 0, ru1, ru2, Ld, dist, lpdf);
                    if (lpdf > 0) {
                        Hit sh = trace(s, P, Ld, dist, true, 0);
                        rc.shadow++;
                        if (sh.t > dist) {
                            float nl = dot(N, Ld);
                            float cos_t = std::max(0.0f, dot(Ld, N));
                            float mpdf = (nl <= 0.f) ? 0.f : nl * INV_PI_F;
                            float wgt = power_heuristic(lpdf, mpdf);
                            for (uint32_t k = 0; k < B; ++k) {
                                float bsdf = alb[k] * INV_PI_F * std::max(nl, 0.f);
                                rad[k] += thr[k] * bsdf * lights[l].radiance[k] * cos_t * wgt / lpdf;
                            }
                        }
                    }
                }
                if (bounce < o.bounces) {
                    V3 ls = cosine_sample(u01(r0.v[2]), u01(r0.v[3]));
                    float mpdf = ls.z * INV_PI_F;
                    // tangent_to_global * ls: columns tangent, bitangent, normal (before the map)
                    V3 nd{(tangent.x * ls.x + bitangent.x * ls.y) + N_frame.x * ls.z,
                          (tangent.y * ls.x + bitangent.y * ls.y) + N_frame.y * ls.z,
                          (tangent.z * ls.x + bitangent.z * ls.y) + N_frame.z * ls.z};
                    if (mpdf > 0) {
                        float nl = dot(N, nd);
                        float cos_t = std::max(0.0f, dot(nd, N));
                        float lp = 0;
                        for (uint32_t l = 0; l < nlights; ++l) lp += light_pdf(lights[l], P, nd);
                        lp /= (float)nlights;
                        float wgt = power_heuristic(mpdf, lp);
                        for (uint32_t k = 0; k < B; ++k) {
                            float bsdf = alb[k] * INV_PI_F * std::max(nl, 0.f);
                            thr[k] *= bsdf * cos_t * wgt / mpdf;
                        }
                        ro = P; dir = nd;
                        // Russian roulette (not in the reference; off when rr_depth == 0)
                        if (o.rr_depth != 0 && bounce + 1 >= o.rr_depth) {
                            float q = 0.f;
                            for (uint32_t k = 0; k < B; ++k) q = std::max(q, thr[k]);
                            q = std::min(q, 1.0f);
                            U4 rr = rng.draw(bounce, SLOT_RR);
                            if (u01(rr.v[0]) >= q) {
                                for (uint32_t k = 0; k < B; ++k) path[k] += rad[k];
                                if (bounce == 0) for (uint32_t k = 0; k < B; ++k) direct[k] += rad[k];
                                break;
                            }
                            for (uint32_t k = 0; k < B; ++k) thr[k] = thr[k] / q;
                        }
                    }
                }
                if (bounce == 0) for (uint32_t k = 0; k < B; ++k) direct[k] += rad[k];
            }
            for (uint32_t k = 0; k < B; ++k) path[k] += rad[k];
        }
        for (uint32_t k = 0; k < B; ++k) radiance[k] += path[k];
        if (o.adaptive_sampling) {
            // unidirectional's adaptive stop (cpu_path_tracer.ipp:198-226); illum = magnitude()
            // (spectral_data.ipp:280-287)
            float sq = 0;
            for (uint32_t k = 0; k < B; ++k) sq += path[k] * path[k];
            float illum = std::sqrt(sq);
            s1 += illum;
            s2 += (illum * illum);
            if (sample % o.samples_to_detect_miss == 0 && sample != 0) {
                if (depth == 0) break;
            }
            if (sample % o.samples_per_batch == 0 && sample != 0) {
                if (s1 == 0) break;
                float n = static_cast<float>(sample) + 1.f;
                float mu = s1 / n;
                float variance = (1.f / (n - 1.f)) * (s2 - (s1 * s1) / n);
                float I = 1.96f * std::sqrt(variance / n);
                if (I <= o.sampling_tolerance * mu) break;
            }
        }
    }
    // after a break `sample` is the index of the last sample taken: the reference divides by it
    float sf = (float)sample;
    for (uint32_t k = 0; k < B; ++k) {
        out.total[k] = radiance[k] / sf;
        out.direct[k] = direct[k] / sf;
        out.indirect[k] = out.total[k] - out.direct[k];
        out.albedo[k] = albedo_acc[k] / sf;
    }
    out.normal = normalize(normal_acc);
    out.depth = (count == 0) ? INF_F : depth / (float)count;
    out.alpha = (float)count / sf;
    out.tri = tri_first;
}

}  // namespace

// ==================================================================== C interface
OAPI void oracle_philox(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    U4 c{{ctr[0], ctr[1], ctr[2], ctr[3]}};
    U4 r = philox(c, key[0], key[1]);
    for (int k = 0; k < 4; ++k) out[k] = r.v[k];
}

OAPI int oracle_compute_normals(const float* pos, uint32_t nverts, const uint32_t* idx, uint32_t ntris,
                                float* normals_out) {
    if (!pos || !idx || !normals_out) return 1;
    compute_normals(pos, nverts, idx, ntris, normals_out);
    return 0;
}

OAPI int oracle_dem_triangulate(const float* heights, uint32_t W, uint32_t H, double sx, double sy,
                                float* pos_out, uint32_t* idx_out, uint32_t* ntris_out) {
    if (!heights || !pos_out || !idx_out || !ntris_out || W < 2 || H < 2) return 1;
    // DEMProjection::initToWorld / transformToWorld, non-OGR, xoff = yoff = 0, dx = dy = 1
    double tsx = ((double)W - 1.) / 2., tsy = ((double)H - 1.) / 2.;
    double startX = -tsx, startY = -tsy;
    double scale_x = (tsx + 0.5) / (double)W, scale_y = (tsy + 0.5) / (double)H;
    for (uint32_t j = 0; j < H; ++j) {
        for (uint32_t i = 0; i < W; ++i) {
            float z = heights[(size_t)j * W + i];
            size_t v = (size_t)j * W + i;
            if (std::isinf(z) || std::isnan(z)) {
                pos_out[3 * v] = pos_out[3 * v + 1] = pos_out[3 * v + 2] = INF_F;
                continue;
            }
            double Ix = (double)(float)i + (0.0 / 1.0), Iy = (double)(float)j + (0.0 / 1.0);
            double Xs = Ix * scale_x, Ys = -Iy * scale_y;
            double x = 1.0 * sx * (startX + (2. * Xs));
            double y = 1.0 * sy * (-startY + (2. * Ys));
            pos_out[3 * v] = (float)x; pos_out[3 * v + 1] = (float)y; pos_out[3 * v + 2] = (float)(double)z;
        }
    }
    size_t k = 0;
    for (uint32_t i = 0; i + 1 < W; ++i) {
        for (uint32_t j = 0; j + 1 < H; ++j) {
            uint32_t f[2][3] = {{i + (j + 1) * W, i + 1 + j * W, i + j * W},
                                {i + 1 + j * W, i + (j + 1) * W, i + 1 + (j + 1) * W}};
            for (int q = 0; q < 2; ++q) {
                if (!std::isinf(heights[f[q][0]]) && !std::isinf(heights[f[q][1]]) && !std::isinf(heights[f[q][2]])) {
                    idx_out[k] = f[q][0]; idx_out[k + 1] = f[q][1]; idx_out[k + 2] = f[q][2];
                    k += 3;
                }
            }
        }
    }
    *ntris_out = (uint32_t)(k / 3);
    return 0;
}

OAPI int oracle_intrinsics(float focal, float sensor_x, float sensor_y, uint32_t W, uint32_t H,
                           float px, float py, float kxy_, float kyx_, float z_dir, float kinv[6]) {
    float kx_ = (float)W / sensor_x;
    float ky_ = (float)H / sensor_y;
    if (std::isinf(px)) px = (float)W / 2;
    if (std::isinf(py)) py = (float)H / 2;
    float kx = kx_, ky = z_dir * ky_;
    float ppx = z_dir * px, ppy = z_dir * py;
    float kxy = z_dir * kxy_, kyx = z_dir * kyx_;
    float fx = focal * kx, fy = focal * ky;
    float det = (fx * fy) - (kxy * kyx);
    kinv[0] = fy / det;                          // [0][0]
    kinv[1] = -kyx / det;                        // [0][1]
    kinv[2] = -kxy / det;                        // [1][0]
    kinv[3] = fx / det;                          // [1][1]
    kinv[4] = ((kxy * ppy) - (fy * ppx)) / det;  // [2][0]
    kinv[5] = ((kyx * ppx) - (fx * ppy)) / det;  // [2][1]
    return 0;
}

namespace {
V3d tangent_d(V3d p0, V3d p1) {
    V3d p = p1 - p0;
    V3d r = crossd(p0, p);
    V3d t = crossd(r, p0);
    return normalized(t);
}
double tri_solid_angle(V3d c0, V3d c1, V3d c2) {
    double a0 = std::acos(dotd(tangent_d(c0, c1), tangent_d(c0, c2)));
    double a1 = std::acos(dotd(tangent_d(c1, c0), tangent_d(c1, c2)));
    double a2 = std::acos(dotd(tangent_d(c2, c0), tangent_d(c2, c1)));
    return ((a0 + a1) + a2) - 3.141592653589793238462;
}
// pixelToDirectionHelper_d (camera.ipp:1759-1771): the distortion takes and returns glm's
// vec2<float>, so the FP64 point is converted to FP32 around undistort.
V3d corner_dir(const vgb_camera& c, double x, double y) {
    const float* K = c.kinv;
    double hx = ((double)K[0] * x + (double)K[2] * y) + (double)K[4] * 1.0;
    double hy = ((double)K[1] * x + (double)K[3] * y) + (double)K[5] * 1.0;
    if (c.distortion) {
        Pix u = undistort(c, Pix{(float)hx, (float)hy});
        hx = u.x;
        hy = u.y;
    }
    double zd = (double)c.z_dir;
    return normalized(V3d{hx, zd * hy, zd});
}
}  // namespace

// Distortion::distort (inverse = 0) or undistort (inverse = 1) of n normalised image points.
OAPI int oracle_distortion(const vgb_camera* cam, const float* xy, uint32_t n, int inverse, float* out) {
    if (!cam || !xy || !out) return 1;
    for (uint32_t k = 0; k < n; ++k) {
        Pix h{xy[2 * k], xy[2 * k + 1]};
        Pix r = !cam->distortion ? h : (inverse ? undistort(*cam, h) : distort(*cam, h));
        out[2 * k] = r.x;
        out[2 * k + 1] = r.y;
    }
    return 0;
}

OAPI int oracle_pixel_solid_angle(const vgb_camera* cam, float* out, int nthreads) {
    if (!cam || !out) return 1;
    uint32_t W = cam->width, H = cam->height;
    auto work = [&](uint32_t j0, uint32_t j1) {
        for (uint32_t j = j0; j < j1; ++j)
            for (uint32_t i = 0; i < W; ++i) {
                V3d c0 = corner_dir(*cam, i, j), c1 = corner_dir(*cam, i + 1, j);
                V3d c2 = corner_dir(*cam, i + 1, j + 1), c3 = corner_dir(*cam, i, j + 1);
                out[(size_t)j * W + i] = (float)(tri_solid_angle(c0, c1, c2) + tri_solid_angle(c0, c2, c3));
            }
    };
    int nt = std::max(1, nthreads);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(work, H * t / nt, H * (t + 1) / nt);
    for (auto& x : th) x.join();
    return 0;
}

// blackBodyRadiance for one band [lmin, lmax] in metres (FP32 band edges as the reference
// stores them), steps samples, trapezoid in FP64.
OAPI double oracle_blackbody_band(double T, float lmin_m, float lmax_m, uint32_t steps) {
    const double c = 299792458.0, h = 6.62607015e-34, kB = 1.380649e-23;
    double mn = lmin_m, mx = lmax_m;
    double step = (mx - mn) / (double)(steps - 1);
    std::vector<double> lam(steps), rad(steps);
    for (uint32_t i = 0; i < steps; ++i) {
        lam[i] = mn + ((double)i * step);
        double l5 = std::pow(lam[i], 5.);
        double coeff = 2 * h * c * c / l5;
        rad[i] = coeff * 1. / (std::exp(h * c / (lam[i] * kB * T)) - 1.);
    }
    double area = 0;
    for (uint32_t i = 0; i + 1 < steps; ++i) {
        double dx = lam[i + 1] - lam[i];
        area += dx * (rad[i] + rad[i + 1]) / 2.;
    }
    return area;
}

OAPI void* oracle_scene_create(const float* pos, uint32_t nverts, const uint32_t* idx, uint32_t ntris,
                               uint32_t nbands, const float* albedo, const float* normals,
                               const float* uv, const float* tex, uint32_t tw, uint32_t th) {
    if (!pos || !idx || nbands == 0 || nbands > VGB_MAX_BANDS) return nullptr;
    for (size_t k = 0; k < (size_t)3 * ntris; ++k) if (idx[k] >= nverts) return nullptr;
    auto* s = new Scene();
    s->nverts = nverts; s->ntris = ntris; s->nbands = nbands;
    s->pos.resize(nverts); s->nrm.resize(nverts);
    for (uint32_t v = 0; v < nverts; ++v) s->pos[v] = V3{pos[3 * v], pos[3 * v + 1], pos[3 * v + 2]};
    s->idx.assign(idx, idx + (size_t)3 * ntris);
    std::vector<float> n(3 * (size_t)nverts);
    if (normals) std::memcpy(n.data(), normals, n.size() * 4);
    else compute_normals(pos, nverts, idx, ntris, n.data());
    for (uint32_t v = 0; v < nverts; ++v) s->nrm[v] = V3{n[3 * v], n[3 * v + 1], n[3 * v + 2]};
    s->uv.assign(2 * (size_t)nverts, 0.f);
    if (uv) std::memcpy(s->uv.data(), uv, s->uv.size() * 4);
    s->albedo.assign((size_t)nverts * nbands, 1.f);
    if (albedo) std::memcpy(s->albedo.data(), albedo, s->albedo.size() * 4);
    if (tex && tw && th) { s->tw = tw; s->th = th; s->tex.assign(tex, tex + (size_t)tw * th * nbands); }
    else { s->tw = s->th = 1; s->tex.assign(nbands, 1.f); }
    build_bvh(*s);
    return s;
}

OAPI void oracle_scene_destroy(void* h) { delete static_cast<Scene*>(h); }

OAPI int oracle_scene_motion(void* h, const vgb_instance_motion* m, uint32_t n) {
    if (!h) return 1;
    Scene& s = *static_cast<Scene*>(h);
    s.motion.assign(m, m + (m ? n : 0));
    return 0;
}

OAPI int oracle_scene_normal_map(void* h, const float* nmap, uint32_t w, uint32_t hh) {
    if (!h) return 1;
    Scene& s = *static_cast<Scene*>(h);
    s.nmap.clear();
    s.nw = s.nh = 0;
    if (nmap && w && hh) {
        s.nmap.assign(nmap, nmap + (size_t)w * hh * 3);
        s.nw = w;
        s.nh = hh;
    }
    return 0;
}

OAPI uint32_t oracle_scene_bvh_nodes(void* h) { return (uint32_t) static_cast<Scene*>(h)->nodes.size(); }

OAPI int oracle_trace(void* h, const float* orig, const float* dirs, const float* tmax, uint32_t n,
                      int any_hit, int mode, uint32_t* tri_out, float* t_out, float* bary_out,
                      int nthreads, uint64_t* nodes_out, uint64_t* tris_out) {
    if (!h || !orig || !dirs || !tri_out) return 1;
    const Scene& s = *static_cast<Scene*>(h);
    int nt = std::max(1, nthreads);
    std::vector<uint64_t> nv(nt, 0), tv(nt, 0);
    auto work = [&](int tid, uint32_t a, uint32_t b) {
        for (uint32_t r = a; r < b; ++r) {
            V3 o{orig[3 * r], orig[3 * r + 1], orig[3 * r + 2]};
            V3 d{dirs[3 * r], dirs[3 * r + 1], dirs[3 * r + 2]};
            float tm = tmax ? tmax[r] : INF_F;
            Hit hh = trace(s, o, d, tm, any_hit != 0, mode, &nv[tid], &tv[tid]);
            tri_out[r] = hh.tri;
            if (t_out) t_out[r] = hh.t;
            if (bary_out) { bary_out[3 * r] = hh.w[0]; bary_out[3 * r + 1] = hh.w[1]; bary_out[3 * r + 2] = hh.w[2]; }
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(work, t, (uint32_t)((uint64_t)n * t / nt), (uint32_t)((uint64_t)n * (t + 1) / nt));
    for (auto& x : th) x.join();
    uint64_t ns = 0, ts = 0;
    for (int t = 0; t < nt; ++t) { ns += nv[t]; ts += tv[t]; }
    if (nodes_out) *nodes_out = ns;
    if (tris_out) *tris_out = ts;
    return 0;
}

// Renders rows row_begin, row_begin + row_step, ... (below row_end) into host film planes of the
// full image size.  ray_counts_out[0] = closest-hit queries, [1] = shadow queries.
OAPI int oracle_render(void* h, const vgb_camera* cam, const vgb_light* lights, uint32_t nlights,
                       const vgb_pt_options* opts, vgb_film* film, uint32_t row_begin,
                       uint32_t row_end, uint32_t row_step, int nthreads, uint64_t* ray_counts_out) {
    if (!h || !cam || !opts || !film || row_step == 0) return 1;
    if (opts->samples == 0 || (nlights && !lights)) return 1;
    if (opts->adaptive_sampling && (opts->samples_per_batch == 0 || opts->samples_to_detect_miss == 0)) return 1;
    const Scene& s = *static_cast<Scene*>(h);
    if (opts->nbands != s.nbands) return 1;
    const uint32_t W = cam->width, H = cam->height, B = s.nbands;
    row_end = std::min(row_end, H);
    const size_t plane = (size_t)W * H;
    int nt = std::max(1, nthreads);
    const CameraRays cr(*cam, nt);
    // threads take chunks of 32 pixels of the selected rows in row-major order, so a band of one
    // row keeps every thread busy too
    constexpr uint64_t kChunk = 32;
    const uint64_t nrows = row_end > row_begin ? (row_end - row_begin + row_step - 1) / row_step : 0;
    const uint64_t last = nrows * W;
    std::atomic<uint64_t> next_px{0};
    std::vector<RenderCounters> rcs(nt);
    auto work = [&](int tid) {
        while (true) {
            const uint64_t p0 = next_px.fetch_add(kChunk);
            if (p0 >= last) break;
            const uint64_t p1 = std::min(last, p0 + kChunk);
            for (uint64_t pp = p0; pp < p1; ++pp) {
                const uint32_t i = (uint32_t)(pp % W), j = row_begin + (uint32_t)(pp / W) * row_step;
                PixelOut po;
                render_pixel(s, cr, lights, nlights, *opts, i, j, po, rcs[tid]);
                size_t p = (size_t)j * W + i;
                for (uint32_t k = 0; k < B; ++k) {
                    if (film->total_radiance) film->total_radiance[k * plane + p] = po.total[k];
                    if (film->direct_radiance) film->direct_radiance[k * plane + p] = po.direct[k];
                    if (film->indirect_radiance) film->indirect_radiance[k * plane + p] = po.indirect[k];
                    if (film->albedo) film->albedo[k * plane + p] = po.albedo[k];
                    if (film->received_power && film->pixel_solid_angle)
                        film->received_power[k * plane + p] =
                            (cam->power_scale[k] * film->pixel_solid_angle[p]) * po.total[k];
                }
                if (film->normal_global) {
                    film->normal_global[p] = po.normal.x;
                    film->normal_global[plane + p] = po.normal.y;
                    film->normal_global[2 * plane + p] = po.normal.z;
                }
                if (film->depth) film->depth[p] = po.depth;
                if (film->alpha) film->alpha[p] = po.alpha;
                if (film->triangle_id) film->triangle_id[p] = po.tri;
                if (film->triangle_size) film->triangle_size[p] = po.tsz;
                if (film->velocity_global) {
                    film->velocity_global[p] = po.vel_g.x;
                    film->velocity_global[plane + p] = po.vel_g.y;
                    film->velocity_global[2 * plane + p] = po.vel_g.z;
                }
                if (film->velocity_camera) {
                    film->velocity_camera[p] = po.vel_c.x;
                    film->velocity_camera[plane + p] = po.vel_c.y;
                    film->velocity_camera[2 * plane + p] = po.vel_c.z;
                }
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(work, t);
    for (auto& x : th) x.join();
    if (ray_counts_out) {
        uint64_t c = 0, sh = 0;
        for (auto& r : rcs) { c += r.closest; sh += r.shadow; }
        ray_counts_out[0] = c; ray_counts_out[1] = sh;
    }
    return 0;
}


// ==================================================================== FP64 adjoint (path replay)
// The same sampled paths as oracle_render (FP32, identical arithmetic), with the gradient of
// sum_k g_k I_k (g = dL/dI / spp) formed in FP64: albedo through the suffix radiance / albedo
// of every path vertex; vertex positions through the shading normal in every NEE term (flat:
// the hit triangle's face normal; smooth: the interpolated vertex normals, then the normals of
// the 1-ring faces, vnormal_backward) and through the hit-point motion on the triangle
// (barycentrics -> uv -> bilinear texture, interpolated vertex albedo and normal).  Visibility,
// the rotation of sampled directions with the normal and the motion of the shading point are
// excluded, as in the product's vgb_adjoint_positions.
namespace {

struct AVtx {
    uint32_t tri;
    float w0, w1, uvx, uvy;
    double m[3][2], gn[3];   // M^-1 e_a (b1, b2) for a = x, y, z; dL/dN
    float alb[VGB_MAX_BANDS], va[VGB_MAX_BANDS], tex[VGB_MAX_BANDS], rad[VGB_MAX_BANDS];
};

static inline V3d v3d(V3 a) { return V3d{a.x, a.y, a.z}; }
static inline V3d addd(V3d a, V3d b) { return V3d{a.x + b.x, a.y + b.y, a.z + b.z}; }
static inline V3d subd(V3d a, V3d b) { return V3d{a.x - b.x, a.y - b.y, a.z - b.z}; }
static inline V3d muld(V3d a, double k) { return V3d{a.x * k, a.y * k, a.z * k}; }

// Gradients of sum(g * I) for one pixel, added into gtex ([th][tw][B]), gpos ([nverts][3]) and,
// with smooth shading, gvn ([nverts][3], the vertex-normal gradients that
// vnormal_backward carries to the positions).
static void adjoint_pixel(const Scene& s, const CameraRays& cr, const vgb_light* lights, uint32_t nlights,
                          const vgb_pt_options& o, uint32_t i, uint32_t j, const double* g, double* gtex, double* gpos,
                          double* gvn) {
    const vgb_camera& cam = cr.cam;
    const uint32_t B = s.nbands;
    Rng rng{(uint32_t)o.seed, (uint32_t)(o.seed >> 32), j * cam.width + i, 0, o.frame};
    for (uint32_t sample = 0; sample < o.samples; ++sample) {
        rng.sample = sample;
        V3 ro, dir;
        cr.ray(i, j, sample, rng, ro, dir);
        float thr[VGB_MAX_BANDS], bgc[VGB_MAX_BANDS] = {0};
        for (uint32_t k = 0; k < B; ++k) thr[k] = 1.f;
        AVtx vx[4];
        int nv = 0;
        for (uint32_t bounce = 0; bounce < o.bounces + 1 && nv < 4; ++bounce) {
            Hit h = trace(s, ro, dir, INF_F, false, 0);
            if (std::isinf(h.t)) {
                if (o.simulate_lighting && o.show_background) {
                    float x = dir.x, y = dir.y, z = dir.z;
                    float u = std::atan2(y, x) / (2 * PI_F);
                    float v = std::atan2(std::sqrt(x * x + y * y), z) / PI_F;
                    float px = std::fmod(u * 1.f, 1.f), py = std::fmod(v * 1.f, 1.f);
                    if (px < 0) px += 1.f;
                    if (py < 0) py += 1.f;
                    float a = (1.f - px) * (1.f - py), b = px * (1.f - py), c = (1.f - px) * py, e = px * py;
                    for (uint32_t k = 0; k < B; ++k) {
                        float bgv = o.background[k];
                        bgc[k] = thr[k] * ((((a * bgv + b * bgv) + c * bgv) + e * bgv) * 1.f);
                    }
                }
                break;
            }
            AVtx& V = vx[nv++];
            const uint32_t t = h.tri;
            const uint32_t i0 = s.idx[3 * t], i1 = s.idx[3 * t + 1], i2 = s.idx[3 * t + 2];
            const uint32_t vi[3] = {i1, i2, i0};
            const float* w = h.w;
            V.tri = t; V.w0 = w[0]; V.w1 = w[1];
            {
                const float* a = &s.uv[2 * vi[0]]; const float* b = &s.uv[2 * vi[1]]; const float* c = &s.uv[2 * vi[2]];
                V.uvx = (w[0] * a[0] + w[1] * b[0]) + w[2] * c[0];
                V.uvy = (w[0] * a[1] + w[1] * b[1]) + w[2] * c[1];
            }
            V3 p0 = s.pos[i0], p1 = s.pos[i1], p2 = s.pos[i2];
            V3 fnn = normalize(cross(p0 - p1, p2 - p0));
            V3 fnrm{-fnn.x, -fnn.y, -fnn.z};
            V3 N_local = fnrm;
            if (o.smooth_shading) N_local = normalize((w[0] * s.nrm[vi[0]] + w[1] * s.nrm[vi[1]]) + w[2] * s.nrm[vi[2]]);
            V3 N = N_local;
            V3 arb = (std::fabs(N.x) < 0.9f) ? V3{1, 0, 0} : V3{0, 1, 0};
            V3 tangent = normalize(cross(arb, N));
            V3 bitangent = cross(N, tangent);
            sample_uvs(s, V.uvx, V.uvy, V.tex);
            for (uint32_t k = 0; k < B; ++k) {
                V.va[k] = (w[0] * s.albedo[(size_t)vi[0] * B + k] + w[1] * s.albedo[(size_t)vi[1] * B + k]) +
                          w[2] * s.albedo[(size_t)vi[2] * B + k];
                V.alb[k] = V.va[k] * V.tex[k];
            }
            // M^-1 e_a for the hit-point motion, FP64 (caller order A=v0, B=v1, C=v2), M = [d | A-B | A-C]
            {
                V3d A{p0.x, p0.y, p0.z}, Bv{p1.x, p1.y, p1.z}, Cv{p2.x, p2.y, p2.z}, d{dir.x, dir.y, dir.z};
                V3d c1 = A - Bv, c2 = A - Cv;
                double det = dotd(d, crossd(c1, c2));
                for (int a = 0; a < 3; ++a) {
                    V3d e{a == 0 ? 1.0 : 0.0, a == 1 ? 1.0 : 0.0, a == 2 ? 1.0 : 0.0};
                    V.m[a][0] = det != 0 ? dotd(d, crossd(e, c2)) / det : 0.0;
                    V.m[a][1] = det != 0 ? dotd(d, crossd(c1, e)) / det : 0.0;
                }
            }
            V.gn[0] = V.gn[1] = V.gn[2] = 0.0;
            for (uint32_t k = 0; k < B; ++k) V.rad[k] = 0.f;
            V3 P = (w[0] * s.pos[vi[0]] + w[1] * s.pos[vi[1]]) + w[2] * s.pos[vi[2]];
            {
                V3 q[3];
                for (int k = 0; k < 3; ++k) { V3 vp = s.pos[vi[k]], vn = s.nrm[vi[k]]; q[k] = P - dot(P - vp, vn) * vn; }
                V3 sp = (q[0] * w[0] + q[1] * w[1]) + q[2] * w[2];
                if (dot(sp - P, N_local) > 0) P = sp;
            }
            if (!o.simulate_lighting) break;
            P = V3{off1(P.x, fnrm.x), off1(P.y, fnrm.y), off1(P.z, fnrm.z)};
            if (bounce == 0 && o.has_ambient)
                for (uint32_t k = 0; k < B; ++k) V.rad[k] += thr[k] * (o.ambient[k] * V.alb[k]);
            U4 r0 = rng.draw(bounce, SLOT_MAIN);
            for (uint32_t l = 0; l < nlights; ++l) {
                float ru1, ru2;
                if (l == 0) { ru1 = u01(r0.v[0]); ru2 = u01(r0.v[1]); }
                else { U4 rl = rng.draw(bounce, 1 + l); ru1 = u01(rl.v[0]); ru2 = u01(rl.v[1]); }
                V3 Ld; float dist, lpdf = 0;
                light_sample(lights[l], P, o.deterministic_light != 0, ru1, ru2, Ld, dist, lpdf);
                if (!(lpdf > 0)) continue;
                Hit sh = trace(s, P, Ld, dist, true, 0);
                if (!(sh.t > dist)) continue;
                float nl = dot(N, Ld);
                float cos_t = std::max(0.0f, dot(Ld, N));
                float mpdf = (nl <= 0.f) ? 0.f : nl * INV_PI_F;
                float wgt = power_heuristic(lpdf, mpdf);
                double gc = 0;
                for (uint32_t k = 0; k < B; ++k) {
                    float bsdf = V.alb[k] * INV_PI_F * std::max(nl, 0.f);
                    float con = thr[k] * bsdf * lights[l].radiance[k] * cos_t * wgt / lpdf;
                    V.rad[k] += con;
                    gc += g[k] * (double)con;
                }
                if (nl > 0.f && wgt > 0.f) {
                    double m = (double)nl / 3.141592653589793238462;
                    double lp = lpdf;
                    double dw_over_w = -2.0 * m / 3.141592653589793238462 / (lp * lp + m * m);
                    double sc = gc * (2.0 / nl + dw_over_w);
                    V.gn[0] += sc * Ld.x; V.gn[1] += sc * Ld.y; V.gn[2] += sc * Ld.z;
                }
            }
            if (bounce >= o.bounces) break;
            V3 ls = cosine_sample(u01(r0.v[2]), u01(r0.v[3]));
            float mpdf = ls.z * INV_PI_F;
            V3 nd{(tangent.x * ls.x + bitangent.x * ls.y) + N.x * ls.z, (tangent.y * ls.x + bitangent.y * ls.y) + N.y * ls.z,
                  (tangent.z * ls.x + bitangent.z * ls.y) + N.z * ls.z};
            if (mpdf > 0) {
                float nl = dot(N, nd);
                float cos_t = std::max(0.0f, dot(nd, N));
                float lp = 0;
                for (uint32_t l = 0; l < nlights; ++l) lp += light_pdf(lights[l], P, nd);
                lp /= (float)nlights;
                float wgt = power_heuristic(mpdf, lp);
                for (uint32_t k = 0; k < B; ++k) {
                    float bsdf = V.alb[k] * INV_PI_F * std::max(nl, 0.f);
                    thr[k] *= bsdf * cos_t * wgt / mpdf;
                }
                ro = P; dir = nd;
                if (o.rr_depth != 0 && bounce + 1 >= o.rr_depth) {
                    float q = 0.f;
                    for (uint32_t k = 0; k < B; ++k) q = std::max(q, thr[k]);
                    q = std::min(q, 1.0f);
                    U4 rr = rng.draw(bounce, SLOT_RR);
                    if (u01(rr.v[0]) >= q) break;
                    for (uint32_t k = 0; k < B; ++k) thr[k] = thr[k] / q;
                }
            }
        }
        double S[VGB_MAX_BANDS];
        for (uint32_t k = 0; k < B; ++k) S[k] = bgc[k];
        for (int b = nv - 1; b >= 0; --b) {
            const AVtx& V = vx[b];
            double ga[VGB_MAX_BANDS];
            for (uint32_t k = 0; k < B; ++k) {
                S[k] += V.rad[k];
                ga[k] = V.alb[k] != 0.f ? g[k] * S[k] / (double)V.alb[k] : 0.0;
            }
            float rx = (float)s.tw, ry = (float)s.th;
            float px = std::fmod(V.uvx * rx, rx), py = std::fmod(V.uvy * ry, ry);
            if (px < 0) px += rx;
            if (py < 0) py += ry;
            int x0 = std::min((int)std::floor(px), (int)s.tw - 1), y0 = std::min((int)std::floor(py), (int)s.th - 1);
            int x1 = std::min(x0 + 1, (int)s.tw - 1), y1 = std::min(y0 + 1, (int)s.th - 1);
            double dx = px - (float)x0, dy = py - (float)y0;
            double wt[4] = {(1 - dx) * (1 - dy), dx * (1 - dy), (1 - dx) * dy, dx * dy};
            size_t tx[4] = {(size_t)y0 * s.tw + x0, (size_t)y0 * s.tw + x1, (size_t)y1 * s.tw + x0, (size_t)y1 * s.tw + x1};
            if (gtex)
                for (uint32_t k = 0; k < B; ++k)
                    for (int q = 0; q < 4; ++q) gtex[tx[q] * B + k] += ga[k] * V.va[k] * wt[q];
            if (gpos) {
                uint32_t ia = s.idx[3 * V.tri], ib = s.idx[3 * V.tri + 1], ic = s.idx[3 * V.tri + 2];
                V3d A{s.pos[ia].x, s.pos[ia].y, s.pos[ia].z}, Bv{s.pos[ib].x, s.pos[ib].y, s.pos[ib].z};
                V3d Cv{s.pos[ic].x, s.pos[ic].y, s.pos[ic].z};
                const V3d gN{V.gn[0], V.gn[1], V.gn[2]};
                const double wA = 1.0 - (double)V.w0 - (double)V.w1;
                V3d gp[3] = {V3d{0, 0, 0}, V3d{0, 0, 0}, V3d{0, 0, 0}};   // A, B, C
                double e0 = 0, e1 = 0;   // dL/dw0, dL/dw1 through the interpolated normal
                if (!o.smooth_shading) {
                    // N = -n/|n|, n = cross(a, bb): dL/dn, then dL/da = bb x dL/dn, dL/dbb = dL/dn x a
                    V3d a = A - Bv, bb = Cv - A;
                    V3d n = crossd(a, bb);
                    double ln = std::sqrt(dotd(n, n));
                    if (ln > 0) {
                        V3d nh = muld(n, 1.0 / ln);
                        V3d gn = muld(subd(gN, muld(nh, dotd(nh, gN))), -1.0 / ln);
                        V3d ga_ = crossd(bb, gn), gb_ = crossd(gn, a);
                        gp[0] = subd(ga_, gb_); gp[1] = muld(ga_, -1.0); gp[2] = gb_;
                    }
                } else {
                    // N = S/|S|, S = w0 n_B + w1 n_C + wA n_A
                    V3d nA = v3d(s.nrm[ia]), nB = v3d(s.nrm[ib]), nC = v3d(s.nrm[ic]);
                    V3d S = addd(addd(muld(nB, V.w0), muld(nC, V.w1)), muld(nA, wA));
                    double lS = std::sqrt(dotd(S, S));
                    if (lS > 0) {
                        V3d Nn = muld(S, 1.0 / lS);
                        V3d gS = muld(subd(gN, muld(Nn, dotd(Nn, gN))), 1.0 / lS);
                        e0 = dotd(gS, subd(nB, nA));
                        e1 = dotd(gS, subd(nC, nA));
                        const uint32_t vid[3] = {ia, ib, ic};
                        const double wv[3] = {wA, V.w0, V.w1};
                        for (int q = 0; q < 3; ++q) {
                            gvn[3 * (size_t)vid[q] + 0] += wv[q] * gS.x;
                            gvn[3 * (size_t)vid[q] + 1] += wv[q] * gS.y;
                            gvn[3 * (size_t)vid[q] + 2] += wv[q] * gS.z;
                        }
                    }
                }
                const float* uvA = &s.uv[2 * ia]; const float* uvB = &s.uv[2 * ib]; const float* uvC = &s.uv[2 * ic];
                double d0 = 0, d1 = 0;
                for (uint32_t k = 0; k < B; ++k) {
                    double t00 = s.tex[tx[0] * B + k], t10 = s.tex[tx[1] * B + k], t01 = s.tex[tx[2] * B + k], t11 = s.tex[tx[3] * B + k];
                    double dtdx = (1 - dy) * (t10 - t00) + dy * (t11 - t01);
                    double dtdy = (1 - dx) * (t01 - t00) + dx * (t11 - t10);
                    double dt0 = dtdx * rx * ((double)uvB[0] - uvA[0]) + dtdy * ry * ((double)uvB[1] - uvA[1]);
                    double dt1 = dtdx * rx * ((double)uvC[0] - uvA[0]) + dtdy * ry * ((double)uvC[1] - uvA[1]);
                    double aA = s.albedo[(size_t)ia * B + k], aB = s.albedo[(size_t)ib * B + k], aC = s.albedo[(size_t)ic * B + k];
                    d0 += ga[k] * ((aB - aA) * V.tex[k] + (double)V.va[k] * dt0);
                    d1 += ga[k] * ((aC - aA) * V.tex[k] + (double)V.va[k] * dt1);
                }
                d0 += e0;
                d1 += e1;
                double wv[3] = {wA, V.w0, V.w1};
                uint32_t vid[3] = {ia, ib, ic};
                for (int q = 0; q < 3; ++q)
                    for (int a = 0; a < 3; ++a) {
                        const double gpa = a == 0 ? gp[q].x : (a == 1 ? gp[q].y : gp[q].z);
                        gpos[3 * (size_t)vid[q] + a] += gpa + (d0 * V.m[a][0] + d1 * V.m[a][1]) * wv[q];
                    }
            }
        }
    }
}

}  // namespace

// Vertex-normal gradients to position gradients (FP64): n_v = A_v/|A_v|, A_v the sum of the
// unit normals u_f of the faces of v (vgb_compute_vertex_normals), u_f = c/|c|,
// c = cross(p1 - p0, p2 - p0).
static void vnormal_backward(const Scene& s, const double* gvn, double* gpos) {
    std::vector<V3d> A(s.nverts, V3d{0, 0, 0});
    auto face = [&](uint32_t t, V3d& e1, V3d& e2, V3d& c, double& lc) {
        V3d p0 = v3d(s.pos[s.idx[3 * t]]), p1 = v3d(s.pos[s.idx[3 * t + 1]]), p2 = v3d(s.pos[s.idx[3 * t + 2]]);
        if (std::isinf(p0.x) || std::isinf(p1.x) || std::isinf(p2.x)) return false;
        e1 = subd(p1, p0); e2 = subd(p2, p0);
        c = crossd(e1, e2);
        lc = std::sqrt(dotd(c, c));
        return lc > 0;
    };
    for (uint32_t t = 0; t < s.ntris; ++t) {
        V3d e1, e2, c; double lc;
        if (!face(t, e1, e2, c, lc)) continue;
        for (int q = 0; q < 3; ++q) A[s.idx[3 * t + q]] = addd(A[s.idx[3 * t + q]], muld(c, 1.0 / lc));
    }
    for (uint32_t t = 0; t < s.ntris; ++t) {
        V3d e1, e2, c; double lc;
        if (!face(t, e1, e2, c, lc)) continue;
        V3d gu{0, 0, 0};
        for (int q = 0; q < 3; ++q) {
            const uint32_t v = s.idx[3 * t + q];
            double la = std::sqrt(dotd(A[v], A[v]));
            if (!(la > 0)) continue;
            V3d n = muld(A[v], 1.0 / la), G{gvn[3 * (size_t)v], gvn[3 * (size_t)v + 1], gvn[3 * (size_t)v + 2]};
            gu = addd(gu, muld(subd(G, muld(n, dotd(n, G))), 1.0 / la));
        }
        V3d u = muld(c, 1.0 / lc);
        V3d gc = muld(subd(gu, muld(u, dotd(u, gu))), 1.0 / lc);
        V3d g1 = crossd(e2, gc), g2 = crossd(gc, e1), g0 = muld(addd(g1, g2), -1.0);
        const V3d gq[3] = {g0, g1, g2};
        for (int q = 0; q < 3; ++q) {
            const size_t o = 3 * (size_t)s.idx[3 * t + q];
            gpos[o] += gq[q].x; gpos[o + 1] += gq[q].y; gpos[o + 2] += gq[q].z;
        }
    }
}

// Adds the FP64 gradients of sum(dL/dI * I) into gtex ([th][tw][B]) and gpos ([nverts][3]).
OAPI int oracle_adjoint_positions(void* h, const vgb_camera* cam, const vgb_light* lights, uint32_t nlights,
                                  const vgb_pt_options* opts, const float* dldi, double* gtex, double* gpos,
                                  int nthreads) {
    if (!h || !cam || !opts || !dldi || opts->samples == 0) return 1;
    const Scene& s = *static_cast<Scene*>(h);
    if (opts->nbands != s.nbands || opts->bounces > 3) return 1;
    const uint32_t W = cam->width, H = cam->height, B = s.nbands;
    const size_t npix = (size_t)W * H, ntex = (size_t)s.tw * s.th * B, n3 = 3 * (size_t)s.nverts;
    const bool smooth = gpos && opts->smooth_shading;
    int nt = std::max(1, nthreads);
    const CameraRays cr(*cam, nt);
    std::vector<std::vector<double>> tb(nt), pb(nt), nb(nt);
    std::atomic<uint32_t> next{0};
    auto work = [&](int tid) {
        if (gtex) tb[tid].assign(ntex, 0.0);
        if (gpos) pb[tid].assign(n3, 0.0);
        if (smooth) nb[tid].assign(n3, 0.0);
        while (true) {
            uint32_t j = next.fetch_add(1);
            if (j >= H) break;
            for (uint32_t i = 0; i < W; ++i) {
                double g[VGB_MAX_BANDS];
                bool any = false;
                for (uint32_t k = 0; k < B; ++k) {
                    g[k] = (double)dldi[k * npix + (size_t)j * W + i] / (double)(float)opts->samples;
                    any |= g[k] != 0.0;
                }
                if (any) adjoint_pixel(s, cr, lights, nlights, *opts, i, j, g, gtex ? tb[tid].data() : nullptr,
                                       gpos ? pb[tid].data() : nullptr, smooth ? nb[tid].data() : nullptr);
            }
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(work, t);
    for (auto& x : th) x.join();
    std::vector<double> gvn(smooth ? n3 : 0, 0.0);
    for (int t = 0; t < nt; ++t) {
        if (gtex) for (size_t q = 0; q < ntex; ++q) gtex[q] += tb[t][q];
        if (gpos) for (size_t q = 0; q < n3; ++q) gpos[q] += pb[t][q];
        if (smooth) for (size_t q = 0; q < n3; ++q) gvn[q] += nb[t][q];
    }
    if (smooth) vnormal_backward(s, gvn.data(), gpos);
    return 0;
}

// Adds the FP64 gradients of sum(dL/dI * I) into gtex ([th][tw][B]) and gz (per vertex, z).
OAPI int oracle_adjoint(void* h, const vgb_camera* cam, const vgb_light* lights, uint32_t nlights,
                        const vgb_pt_options* opts, const float* dldi, double* gtex, double* gz, int nthreads) {
    if (!h) return 1;
    const Scene& s = *static_cast<Scene*>(h);
    std::vector<double> gp(gz ? 3 * (size_t)s.nverts : 0, 0.0);
    int rc = oracle_adjoint_positions(h, cam, lights, nlights, opts, dldi, gtex, gz ? gp.data() : nullptr, nthreads);
    if (rc == 0 && gz)
        for (size_t v = 0; v < s.nverts; ++v) gz[v] += gp[3 * v + 2];
    return rc;
}

// ==================================================================== EATWT denoiser
// denoiseSpectralRadianceEATWT (include/implementation/rendering/cpu_denoise.ipp:9-214) with the
// reference's image indexing restated: Image(i, j) is data[i + j * width] (image.ipp:134-140) and
// the denoiser calls Image(y, x), so every access below is at(y, x) = y + x * width.  That is
// only in range for square images, so other sizes are rejected.  Planes are planar ([B][H][W],
// [H][W], [3][H][W]); direct and indirect are filtered in place.  std::exp and std::pow as in
// the reference.
OAPI int oracle_denoise(float* direct, float* indirect, const float* albedo, const float* depth,
                        const float* normal, uint32_t width, uint32_t height, uint32_t nbands,
                        uint32_t levels_direct, uint32_t levels_indirect, float depth_threshold,
                        float normal_threshold, float min_normal_weight, float epsilon) {
    if (!direct || !indirect || !albedo || !depth || !normal || width == 0 || width != height || nbands == 0 ||
        nbands > VGB_MAX_BANDS)
        return 1;
    static constexpr float K1[5] = {1.0f / 16.0f, 4.0f / 16.0f, 6.0f / 16.0f, 4.0f / 16.0f, 1.0f / 16.0f};
    const int W = (int)width, H = (int)height;
    const size_t P = (size_t)W * H;
    const uint32_t B = nbands;
    auto at = [&](int i, int j) { return (size_t)i + (size_t)j * (size_t)W; };
    std::vector<float> dil(B * P), iil(B * P);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t q = at(y, x);
            for (uint32_t c = 0; c < B; ++c) {
                dil[c * P + q] = direct[c * P + q] / std::max(albedo[c * P + q], epsilon);
                iil[c * P + q] = indirect[c * P + q] / std::max(albedo[c * P + q], epsilon);
            }
        }
    auto filter_pixel = [&](const std::vector<float>& input, int cx, int cy, int step, bool horizontal,
                            std::vector<float>& output) {
        float sum[VGB_MAX_BANDS] = {0};
        float weight_sum = 0.0f;
        const float center_depth = depth[at(cy, cx)];
        const size_t cq = at(cy, cx);
        const float cnx = normal[cq], cny = normal[P + cq], cnz = normal[2 * P + cq];
        for (int k = -2; k <= 2; ++k) {
            int sx = horizontal ? cx + k * step : cx;
            int sy = horizontal ? cy : cy + k * step;
            sx = std::clamp(sx, 0, W - 1);
            sy = std::clamp(sy, 0, H - 1);
            const float kernel_weight = K1[k + 2];
            const size_t sq = at(sy, sx);
            const float sample_depth = depth[sq];
            const float depth_ratio = std::max(center_depth, sample_depth) / (std::min(center_depth, sample_depth) + epsilon);
            const float depth_weight = depth_ratio < (1.0f + depth_threshold) ? 1.0f : std::exp(-(depth_ratio - 1.0f) / depth_threshold);
            const float normal_dot = cnx * normal[sq] + cny * normal[P + sq] + cnz * normal[2 * P + sq];
            const float normal_similarity = std::max(0.0f, normal_dot);
            const float normal_weight = std::max(min_normal_weight,
                                                 std::exp(-std::pow(1.0f - normal_similarity, 2.0f) / normal_threshold));
            const float total_weight = kernel_weight * depth_weight * normal_weight;
            for (uint32_t c = 0; c < B; ++c) sum[c] += input[c * P + sq] * total_weight;
            weight_sum += total_weight;
        }
        if (weight_sum > epsilon) {
            for (uint32_t c = 0; c < B; ++c) output[c * P + cq] = sum[c] / weight_sum;
        } else {
            for (uint32_t c = 0; c < B; ++c) output[c * P + cq] = input[c * P + cq];
        }
    };
    auto denoise = [&](std::vector<float>& illum, uint32_t max_levels) {
        std::vector<float> temp(B * P);
        std::vector<float>* current = &illum;
        std::vector<float>* next = &temp;
        for (uint32_t level = 0; level < max_levels; ++level) {
            const int step = 1 << level;
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x) filter_pixel(*current, x, y, step, true, *next);
            std::swap(current, next);
            for (int y = 0; y < H; ++y)
                for (int x = 0; x < W; ++x) filter_pixel(*current, x, y, step, false, *next);
            std::swap(current, next);
        }
        if (current != &illum) illum = *current;
    };
    denoise(dil, levels_direct);
    denoise(iil, levels_indirect);
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t q = at(y, x);
            for (uint32_t c = 0; c < B; ++c) {
                direct[c * P + q] = dil[c * P + q] * albedo[c * P + q];
                indirect[c * P + q] = iil[c * P + q] * albedo[c * P + q];
            }
        }
    return 0;
}

// ==================================================================== sensor chain (noise-free)
// Camera::getPhotonCounts without photon noise (cameras/camera.ipp:1286-1330) and
// Photosite::exposePixel (photosites/photosite.ipp:125-136) with zero noise electrons:
// photons_k = (t_exp * P_k [* mosaic_k]) / E_k, electrons = sum_k QE_k photons_k,
// out = min(gain * electrons, max_adu) / max_adu.  Planar [B][H][W] in, [H][W] out.
OAPI int oracle_sensor(const float* power, const float* mosaic, uint32_t width, uint32_t height, uint32_t nbands,
                       float exposure_time, const float* photon_energy, const float* qe, float gain, float max_adu,
                       float* out) {
    if (!power || !photon_energy || !qe || !out || nbands == 0 || nbands > VGB_MAX_BANDS || !(max_adu > 0.f)) return 1;
    const size_t P = (size_t)width * height;
    for (size_t p = 0; p < P; ++p) {
        float ph[VGB_MAX_BANDS];
        for (uint32_t k = 0; k < nbands; ++k) {
            float e = exposure_time * power[k * P + p];
            if (mosaic) e = e * mosaic[k * P + p];
            ph[k] = e / photon_energy[k];
        }
        float electrons = 0;
        for (uint32_t k = 0; k < nbands; ++k) electrons += qe[k] * ph[k];
        electrons = electrons + 0.0f;
        const float amplified = std::min(gain * electrons, max_adu);
        out[p] = amplified / max_adu;
    }
    return 0;
}

// SpectralData::integrateOver (spectral_data.ipp:306-333) of n bands [bmin, bmax] with values v.
static float integrate_over(const float* bmin_, const float* bmax_, const float* v, uint32_t n, float minLam,
                            float maxLam) {
    if (minLam > maxLam) std::swap(minLam, maxLam);
    if (minLam == maxLam) return 0.f;
    float integral = 0;
    for (uint32_t i = 0; i < n; ++i) {
        float bmin = bmin_[i], bmax = bmax_[i];
        if (bmin > maxLam || bmax < minLam) continue;
        float bound1 = std::max(bmin, minLam);
        float bound2 = std::min(bmax, maxLam);
        float dLam = bound2 - bound1;
        integral += (dLam * v[i]);
    }
    return integral;
}

// Camera::simulateSensorRGB without noise (camera.ipp:1253-1282, 1337-1380; photosite.ipp:
// 145-154): spectralConvert to ColorRGB, photons per channel, qe_rgb * photons + 0, gain, / ADU.
// rgb = {rgb_min[3], rgb_max[3], rgb_bandwidth[3], rgb_photon_energy[3], rgb_qe[3]}.
OAPI int oracle_sensor_rgb(const float* power, const float* mosaic, uint32_t width, uint32_t height, uint32_t nbands,
                           const float* band_min, const float* band_max, const float* rgb, float exposure_time,
                           float gain, float max_adu, float* out) {
    if (!power || !band_min || !band_max || !rgb || !out || nbands == 0 || nbands > VGB_MAX_BANDS) return 1;
    const size_t P = (size_t)width * height;
    for (size_t p = 0; p < P; ++p) {
        float v[VGB_MAX_BANDS];
        for (uint32_t k = 0; k < nbands; ++k) v[k] = mosaic ? power[k * P + p] * mosaic[k * P + p] : power[k * P + p];
        for (int c = 0; c < 3; ++c) {
            float received = integrate_over(band_min, band_max, v, nbands, rgb[c], rgb[3 + c]) / rgb[6 + c];
            float energy = exposure_time * received;
            float photons = energy / rgb[9 + c];
            float electrons = (rgb[12 + c] * photons) + 0.0f;
            float amplified = gain * electrons;
            out[c * P + p] = amplified / max_adu;
        }
    }
    return 0;
}

// Image::convolveSpatial (images/image.ipp:1267-1340) for a planar spectral image: per band,
// out(x, y) = sum over ky outer, kx inner of in(x + kx - kw/2, y + ky - kh/2) * kernel(kx, ky),
// zero outside the image.  kernel is [B][kh][kw].
OAPI int oracle_psf(const float* in, uint32_t width, uint32_t height, uint32_t nbands, const float* kernel,
                    uint32_t kw, uint32_t kh, float* out) {
    if (!in || !kernel || !out || nbands == 0) return 1;
    const int W = (int)width, H = (int)height, hw = (int)kw / 2, hh = (int)kh / 2;
    const size_t P = (size_t)W * H;
    for (uint32_t b = 0; b < nbands; ++b)
        for (int y = 0; y < H; ++y)
            for (int x = 0; x < W; ++x) {
                float sum = 0.f;
                for (int ky = 0; ky < (int)kh; ++ky)
                    for (int kx = 0; kx < (int)kw; ++kx) {
                        const int ix = x + kx - hw, iy = y + ky - hh;
                        if (ix >= 0 && ix < W && iy >= 0 && iy < H)
                            sum += in[b * P + (size_t)iy * W + ix] * kernel[((size_t)b * kh + ky) * kw + kx];
                    }
                out[b * P + (size_t)y * W + x] = sum;
            }
    return 0;
}

// ---------------------------------------------------------------- DEM Quipu helpers
// LZ4 block decompression as LZ4_decompress_safe (lz4 1.9.4, the version the reference pins in
// dependencies/vcpkg.json) performs it for quipu::decompressData (quipu_io.ipp:216-231),
// restated from the published LZ4 block format: token, literal-length run, literals, 2-byte
// little-endian offset, match-length run; the last sequence carries literals only.  Copies
// byte by byte.  Returns the decoded size or -1.
OAPI int64_t oracle_lz4_decompress(const uint8_t* in, uint64_t n, uint8_t* out, uint64_t cap) {
    uint64_t i = 0, o = 0;
    if (n == 0) return -1;
    while (i < n) {
        const uint8_t token = in[i++];
        uint64_t run = token >> 4;
        if (run == 15) {
            for (;;) {
                if (i >= n) return -1;
                const uint8_t b = in[i++];
                run += b;
                if (b != 255) break;
            }
        }
        for (uint64_t k = 0; k < run; ++k) {
            if (i >= n || o >= cap) return -1;
            out[o++] = in[i++];
        }
        if (i == n) return (int64_t)o;
        if (i + 2 > n) return -1;
        const uint64_t back = (uint64_t)in[i] + 256u * (uint64_t)in[i + 1];
        i += 2;
        if (back == 0 || back > o) return -1;
        uint64_t len = token & 15;
        if (len == 15) {
            for (;;) {
                if (i >= n) return -1;
                const uint8_t b = in[i++];
                len += b;
                if (b != 255) break;
            }
        }
        len += 4;
        for (uint64_t k = 0; k < len; ++k) {
            if (o >= cap) return -1;
            out[o] = out[o - back];
            ++o;
        }
    }
    return -1;  // ended right after a match
}

// The normal cone DEMQuipu::write stores (dem_quipu.ipp:256-270): the glm-normalised sum of the
// coarsest LoD's vertex normals, and the largest std::acos(dot(n, mean)) in FP32 (std::max,
// so NaN angles drop out).  out = {mean.x, mean.y, mean.z, angle}.
OAPI int oracle_normal_cone(const float* normals, uint64_t nv, float* out) {
    float s[3] = {0.f, 0.f, 0.f};
    for (uint64_t v = 0; v < nv; ++v)
        for (int k = 0; k < 3; ++k) s[k] += normals[3 * v + k];
    const float dd = (s[0] * s[0] + s[1] * s[1]) + s[2] * s[2];
    const float inv = 1.0f / std::sqrt(dd);
    const float m[3] = {s[0] * inv, s[1] * inv, s[2] * inv};
    float cone = 0.f;
    for (uint64_t v = 0; v < nv; ++v) {
        const float d = (normals[3 * v] * m[0] + normals[3 * v + 1] * m[1]) + normals[3 * v + 2] * m[2];
        cone = std::max(cone, std::acos(d));
    }
    out[0] = m[0]; out[1] = m[1]; out[2] = m[2]; out[3] = cone;
    return 0;
}

// ---------------------------------------------------------------- rasterizer
// CPURasterizer::render (include/implementation/rendering/cpu_rasterizer.ipp:29-270), literally:
// triangles in buffer order, pixel boxes walked X outer / Y inner at integer corners, the depth
// test `current < previous` against +inf, and the passes overwritten by every fragment that
// passes it (passes.ipp:80-128).  The camera frame is R^T (p - origin) from the vgb_camera and
// the fragment's scene position R p_cam + origin (FP32), as vgb_rasterize defines them.
// static_cast<int>(float) is taken as x86-64 performs it: out-of-range values and NaN give INT_MIN.
static inline int x86_int(float x) { return (x >= -2147483648.f && x < 2147483648.f) ? (int)x : INT32_MIN; }
static inline float edge_fn(float ax, float ay, float bx, float by, float cx, float cy) {
    return (cx - ax) * (by - ay) - (cy - ay) * (bx - ax);
}

// tsz_o, velg_o, velc_o (optional): the triangle-size pass (the longest projected edge in pixels,
// cpu_rasterizer.ipp:123-129) and the velocity passes (:211-218) of the fragment that stays.
OAPI int oracle_rasterize(void* h, const vgb_camera* cam, const float* K, const vgb_light* lights, uint32_t nlights,
                          int lighting, int smooth, float* depth_o, float* alpha_o, float* albedo_o, float* normal_o,
                          uint32_t* tri_o, float* total_o, float* power_o, const float* omega, float* tsz_o,
                          float* velg_o, float* velc_o) {
    const Scene& s = *static_cast<Scene*>(h);
    const uint32_t W = cam->width, H = cam->height, B = s.nbands;
    const size_t P = (size_t)W * H;
    for (size_t v = 0; v < P; ++v) {
        depth_o[v] = INFINITY; alpha_o[v] = 0.f; tri_o[v] = 0xFFFFFFFFu;
        for (int k = 0; k < 3; ++k) normal_o[k * P + v] = 0.f;
        for (uint32_t b = 0; b < B; ++b) { albedo_o[b * P + v] = 0.f; if (total_o) total_o[b * P + v] = 0.f; }
        if (tsz_o) tsz_o[v] = INFINITY;   // DataPayload defaults
        for (int k = 0; k < 3; ++k) {
            if (velg_o) velg_o[k * P + v] = 0.f;
            if (velc_o) velc_o[k * P + v] = 0.f;
        }
    }
    const V3 O{cam->origin[0], cam->origin[1], cam->origin[2]};
    const V3 ax{cam->rotation[0], cam->rotation[1], cam->rotation[2]};
    const V3 ay{cam->rotation[3], cam->rotation[4], cam->rotation[5]};
    const V3 az{cam->rotation[6], cam->rotation[7], cam->rotation[8]};
    for (uint32_t t = 0; t < s.ntris; ++t) {
        const uint32_t vi[3] = {s.idx[3 * t], s.idx[3 * t + 1], s.idx[3 * t + 2]};
        if (std::isinf(s.pos[vi[0]].x) || std::isinf(s.pos[vi[1]].x) || std::isinf(s.pos[vi[2]].x)) continue;
        V3 vc[3];
        for (int k = 0; k < 3; ++k) {
            const V3 d = s.pos[vi[k]] - O;
            vc[k] = V3{dot(ax, d), dot(ay, d), dot(az, d)};
        }
        bool behind = false;
        for (int k = 0; k < 3; ++k) behind = behind || ((-cam->z_dir * vc[k].z) >= 0);
        if (behind) continue;
        float px[3], py[3];
        for (int k = 0; k < 3; ++k) {
            Pix hm{vc[k].x / vc[k].z, vc[k].y / vc[k].z};     // Camera::projectCameraPoint (camera.ipp:1060-1080)
            if (cam->distortion) hm = distort(*cam, hm);
            const float hx = hm.x, hy = hm.y;
            float X = (K[0] * hx + K[1] * hy) + K[2];
            const float Y = (K[3] * hx + K[4] * hy) + K[5];
            if (cam->z_dir < 0) X = (float)(W - 1) - X;
            px[k] = X; py[k] = Y;
        }
        const int sx = x86_int(std::floor(std::min(px[0], std::min(px[1], px[2]))));
        const int sy = x86_int(std::floor(std::min(py[0], std::min(py[1], py[2]))));
        const int ex = x86_int(std::ceil(std::max(px[0], std::max(px[1], px[2]))));
        const int ey = x86_int(std::ceil(std::max(py[0], std::max(py[1], py[2]))));
        if (ex < 0 || sx > (int)W || ey < 0 || sy > (int)H) continue;
        const int x0 = std::clamp(sx, 0, (int)W), y0 = std::clamp(sy, 0, (int)H);
        const int x1 = std::clamp(ex, 0, (int)W), y1 = std::clamp(ey, 0, (int)H);
        const float d0 = length(vc[0]), d1 = length(vc[1]), d2 = length(vc[2]);
        const float area = edge_fn(px[0], py[0], px[1], py[1], px[2], py[2]);
        // size of the triangle: glm's length of the projected edges
        const float e01 = std::sqrt((px[1] - px[0]) * (px[1] - px[0]) + (py[1] - py[0]) * (py[1] - py[0]));
        const float e02 = std::sqrt((px[2] - px[0]) * (px[2] - px[0]) + (py[2] - py[0]) * (py[2] - py[0]));
        const float e12 = std::sqrt((px[2] - px[1]) * (px[2] - px[1]) + (py[2] - py[1]) * (py[2] - py[1]));
        const float tri_size = std::max(e01, std::max(e02, e12));
        for (int X = x0; X < x1; ++X) {
            for (int Y = y0; Y < y1; ++Y) {
                const float fx = (float)X, fy = (float)Y;
                const float w0 = edge_fn(px[1], py[1], px[2], py[2], fx, fy) / area;
                const float w1 = edge_fn(px[2], py[2], px[0], py[0], fx, fy) / area;
                const float w2 = edge_fn(px[0], py[0], px[1], py[1], fx, fy) / area;
                if (!(w0 >= 0 && w1 >= 0 && w2 >= 0)) continue;
                const size_t v = (size_t)Y * W + X;
                const float cur = ((w0 * d0) + (w1 * d1)) + (w2 * d2);
                if (!(cur < depth_o[v])) continue;
                depth_o[v] = cur;
                const float uvx = (w0 * s.uv[2 * vi[0]] + w1 * s.uv[2 * vi[1]]) + w2 * s.uv[2 * vi[2]];
                const float uvy = (w0 * s.uv[2 * vi[0] + 1] + w1 * s.uv[2 * vi[1] + 1]) + w2 * s.uv[2 * vi[2] + 1];
                float texv[VGB_MAX_BANDS], alb[VGB_MAX_BANDS];
                sample_uvs(s, uvx, uvy, texv);
                for (uint32_t b = 0; b < B; ++b) {
                    const float va = (w0 * s.albedo[(size_t)vi[0] * B + b] + w1 * s.albedo[(size_t)vi[1] * B + b]) +
                                     w2 * s.albedo[(size_t)vi[2] * B + b];
                    alb[b] = va * texv[b];
                }
                const V3 fn = normalize(cross(s.pos[vi[0]] - s.pos[vi[1]], s.pos[vi[2]] - s.pos[vi[0]]));
                V3 N{-fn.x, -fn.y, -fn.z};
                if (smooth) N = normalize((w0 * s.nrm[vi[0]] + w1 * s.nrm[vi[1]]) + w2 * s.nrm[vi[2]]);
                {   // tangent frame and Material::getNormal (cpu_rasterizer.ipp:177-191)
                    V3 arb = (std::fabs(N.x) < 0.9f) ? V3{1, 0, 0} : V3{0, 1, 0};
                    V3 tangent = normalize(cross(arb, N));
                    V3 bitangent = cross(N, tangent);
                    N = get_normal(s, uvx, uvy, N, tangent, bitangent);
                }
                float rad[VGB_MAX_BANDS] = {0};
                const V3 fc = (w0 * vc[0] + w1 * vc[1]) + w2 * vc[2];
                const float* R = cam->rotation;
                const V3 fg{((R[0] * fc.x + R[3] * fc.y) + R[6] * fc.z) + cam->origin[0],
                            ((R[1] * fc.x + R[4] * fc.y) + R[7] * fc.z) + cam->origin[1],
                            ((R[2] * fc.x + R[5] * fc.y) + R[8] * fc.z) + cam->origin[2]};
                if (tsz_o) tsz_o[v] = tri_size;
                if (velg_o || velc_o) {
                    V3 vg, vcam;
                    point_velocities(s, *cam, t, fg, vg, vcam);
                    if (velg_o) { velg_o[v] = vg.x; velg_o[P + v] = vg.y; velg_o[2 * P + v] = vg.z; }
                    if (velc_o) { velc_o[v] = vcam.x; velc_o[P + v] = vcam.y; velc_o[2 * P + v] = vcam.z; }
                }
                if (lighting) {
                    for (uint32_t l = 0; l < nlights; ++l) {
                        V3 L; float dist, pdf;
                        light_sample(lights[l], fg, true, 0.f, 0.f, L, dist, pdf);
                        const float nl = std::max(dot(N, L), 0.f);
                        for (uint32_t b = 0; b < B; ++b) {
                            const float bsdf = ((alb[b] * INV_PI_F) * nl) / pdf;
                            rad[b] = rad[b] + lights[l].radiance[b] * bsdf;
                        }
                    }
                }
                alpha_o[v] = INFINITY;
                tri_o[v] = t + 1;
                normal_o[v] = N.x; normal_o[P + v] = N.y; normal_o[2 * P + v] = N.z;
                for (uint32_t b = 0; b < B; ++b) {
                    albedo_o[b * P + v] = alb[b];
                    if (total_o) total_o[b * P + v] = rad[b];
                }
            }
        }
    }
    if (lighting && power_o && omega)
        for (size_t v = 0; v < P; ++v)
            for (uint32_t b = 0; b < B; ++b) power_o[b * P + v] = (cam->power_scale[b] * omega[v]) * total_o[b * P + v];
    return 0;
}
