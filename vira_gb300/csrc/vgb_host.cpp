// vgb_host.cpp -- host-side C++ of the hot path: mesh normals, DEM triangulation, camera
// intrinsics and the binned-SAH BVH builder.  Compiled with -ffp-contract=off so that the
// FP32 expressions restated from the reference round exactly as written.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <thread>
#include <vector>

#include "../../include/vgb.h"
#include "vgb_internal.h"

namespace {

struct F3 { float x, y, z; };
inline F3 sub(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline F3 add(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float dot3(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
inline F3 cross3(F3 a, F3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
inline F3 scale3(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline F3 normalize3(F3 a) { return scale3(a, 1.0f / std::sqrt(dot3(a, a))); }

}  // namespace

// Mesh::calculateNormals, include/implementation/geometry/mesh.ipp:199-233.
extern "C" VGB_API vgb_status vgb_compute_vertex_normals(const float* p, uint32_t nv, const uint32_t* idx,
                                                         uint32_t nt, float* out) try {
    if (!p || !idx || !out) return VGB_ERR_INVALID_ARGUMENT;
    for (size_t k = 0; k < (size_t)3 * nt; ++k)
        if (idx[k] >= nv) return VGB_ERR_INVALID_ARGUMENT;
    std::vector<F3> n(nv, F3{0.f, 0.f, 0.f});
    for (uint32_t t = 0; t < nt; ++t) {
        uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
        F3 p0{p[3 * i0], p[3 * i0 + 1], p[3 * i0 + 2]};
        F3 p1{p[3 * i1], p[3 * i1 + 1], p[3 * i1 + 2]};
        F3 p2{p[3 * i2], p[3 * i2 + 1], p[3 * i2 + 2]};
        if (std::isinf(p0.x) || std::isinf(p1.x) || std::isinf(p2.x)) continue;
        F3 fn = normalize3(cross3(sub(p1, p0), sub(p2, p0)));
        if (std::isnan(fn.x) || std::isnan(fn.y) || std::isnan(fn.z)) continue;
        n[i0] = add(n[i0], fn);
        n[i1] = add(n[i1], fn);
        n[i2] = add(n[i2], fn);
    }
    for (uint32_t v = 0; v < nv; ++v) {
        F3 a = n[v];
        if (std::sqrt(dot3(a, a)) != 0.f) a = normalize3(a);
        out[3 * v] = a.x; out[3 * v + 1] = a.y; out[3 * v + 2] = a.z;
    }
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(nullptr);
}

// DEM::makeVertexBuffer (dem.ipp:165-211) with DEMProjection's non-OGR mapping
// (dem_projection.ipp:66-71, 131-141); Pixel{i, j} holds floats, exact for i, j < 2^24.
void vgb::dem_vertices_host(const float* h, uint32_t W, uint32_t H, const DemPose& pose, float* pos) {
    for (uint32_t j = 0; j < H; ++j) {
        for (uint32_t i = 0; i < W; ++i) {
            const size_t v = (size_t)j * W + i;
            const float z = h[v];
            if (std::isinf(z) || std::isnan(z)) {
                pos[3 * v] = pos[3 * v + 1] = pos[3 * v + 2] = std::numeric_limits<float>::infinity();
                continue;
            }
            const double xs = ((double)i + pose.xo) * pose.scale_x, ys = -((double)j + pose.yo) * pose.scale_y;
            pos[3 * v] = (float)(pose.ax * (-pose.half_x + 2. * xs));
            pos[3 * v + 1] = (float)(pose.ay * (pose.half_y + 2. * ys));
            pos[3 * v + 2] = z;
        }
    }
}

// imageToIndexBuffer (image_utils.ipp:364-409): quad (i, j) gives {(i,j+1),(i+1,j),(i,j)} and
// {(i+1,j),(i,j+1),(i+1,j+1)}, i outer, j inner, skipping infinite heights.
void vgb::dem_faces_host(const float* h, uint32_t W, uint32_t H, uint32_t* idx, uint32_t* nt_out) {
    size_t k = 0;
    for (uint32_t i = 0; i + 1 < W; ++i) {
        for (uint32_t j = 0; j + 1 < H; ++j) {
            const uint32_t a = i + (j + 1) * W, b = i + 1 + j * W, c = i + j * W, d = i + 1 + (j + 1) * W;
            if (!std::isinf(h[a]) && !std::isinf(h[b]) && !std::isinf(h[c])) {
                idx[k++] = a; idx[k++] = b; idx[k++] = c;
            }
            if (!std::isinf(h[b]) && !std::isinf(h[a]) && !std::isinf(h[d])) {
                idx[k++] = b; idx[k++] = a; idx[k++] = d;
            }
        }
    }
    *nt_out = (uint32_t)(k / 3);
}

// A DEM of posts `sx` x `sy` metres, no tile offset, dx = dy = 1.
extern "C" VGB_API vgb_status vgb_dem_triangulate(const float* h, uint32_t W, uint32_t H, double sx,
                                                  double sy, float* pos, uint32_t* idx, uint32_t* nt_out) try {
    if (!h || !pos || !idx || !nt_out || W < 2 || H < 2) return VGB_ERR_INVALID_ARGUMENT;
    vgb::dem_vertices_host(h, W, H, vgb::dem_pose_of(1.0 * sx, 1.0 * sy, 0.0, 0.0, W, H), pos);
    vgb::dem_faces_host(h, W, H, idx, nt_out);
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(nullptr);
}

// Camera::initializeIntrinsicMatrix, camera.ipp:1526-1568, in FP32.
extern "C" VGB_API vgb_status vgb_camera_intrinsics(float focal, float sensor_x, float sensor_y, uint32_t W,
                                                    uint32_t H, float px, float py, float kxy, float kyx,
                                                    float z_dir, float kinv[6]) try {
    if (!kinv || W == 0 || H == 0 || !(focal > 0) || !(sensor_x > 0) || !(sensor_y > 0))
        return VGB_ERR_INVALID_ARGUMENT;
    const float kx0 = (float)W / sensor_x, ky0 = (float)H / sensor_y;
    if (std::isinf(px)) px = (float)W / 2;
    if (std::isinf(py)) py = (float)H / 2;
    const float kx = kx0, ky = z_dir * ky0;
    const float ppx = z_dir * px, ppy = z_dir * py;
    const float sxy = z_dir * kxy, syx = z_dir * kyx;
    const float fx = focal * kx, fy = focal * ky;
    const float det = (fx * fy) - (sxy * syx);
    kinv[0] = fy / det;
    kinv[1] = -syx / det;
    kinv[2] = -sxy / det;
    kinv[3] = fx / det;
    kinv[4] = ((sxy * ppy) - (fy * ppx)) / det;
    kinv[5] = ((syx * ppx) - (fx * ppy)) / det;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(nullptr);
}

// ====================================================================== BVH builder
namespace vgb {
namespace {

struct Box {
    float lo[3] = {INFINITY, INFINITY, INFINITY};
    float hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    void grow(const Box& b) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], b.lo[k]); hi[k] = std::max(hi[k], b.hi[k]); }
    }
    void growp(const float* p) {
        for (int k = 0; k < 3; ++k) { lo[k] = std::min(lo[k], p[k]); hi[k] = std::max(hi[k], p[k]); }
    }
    float half_area() const {
        float e0 = hi[0] - lo[0], e1 = hi[1] - lo[1], e2 = hi[2] - lo[2];
        if (!(e0 >= 0) || !(e1 >= 0) || !(e2 >= 0)) return 0.f;
        return e0 * e1 + e1 * e2 + e2 * e0;
    }
};

// A node of the build tree.  Children refer to other nodes of the same arena (inner) or,
// for the top part of the tree, to the root of another arena.
struct BNode {
    Box box;
    int64_t child[2] = {-1, -1};  // encoded (arena << 32 | index); -1 = none
    uint32_t first = 0, count = 0;
    bool leaf = false;
};

constexpr int kBins = 32;
// Surface-area-heuristic cost of one node traversal step relative to one triangle test.  On the
// path-traced frame (33.5M triangles) 1.5, 2 and 3 built smaller trees with larger leaves that
// rendered 0-7 % slower.
#ifndef VGB_SAH_TRAVERSAL_COST
#define VGB_SAH_TRAVERSAL_COST 1.0f
#endif

struct Ctx {
    const std::vector<Box>* tbox;
    const std::vector<float>* cent;  // 3 per triangle
    std::vector<uint32_t>* order;
    uint32_t max_leaf;
    uint32_t threads;
};

inline int64_t enc(uint32_t arena, uint32_t index) { return ((int64_t)arena << 32) | index; }

struct Split { int axis = -1; int bin = 0; float cost = INFINITY; float cmin = 0, scale = 0; };

// Binned SAH over [first, first+count); parallel binning for large ranges.
Split find_split(const Ctx& c, uint32_t first, uint32_t count, const Box& nb, uint32_t nthreads) {
    Box cb;
    auto& cent = *c.cent;
    auto& ord = *c.order;
    for (uint32_t i = 0; i < count; ++i) cb.growp(&cent[3 * (size_t)ord[first + i]]);
    Split best;
    struct Bins { Box b[3][kBins]; uint32_t n[3][kBins]; };
    float cmin[3], scale[3];
    bool valid[3];
    for (int a = 0; a < 3; ++a) {
        float ext = cb.hi[a] - cb.lo[a];
        valid[a] = ext > 0.f;
        cmin[a] = cb.lo[a];
        scale[a] = valid[a] ? (float)kBins / ext : 0.f;
    }
    auto bin_range = [&](uint32_t a0, uint32_t a1, Bins& bn) {
        for (int a = 0; a < 3; ++a) for (int b = 0; b < kBins; ++b) { bn.b[a][b] = Box(); bn.n[a][b] = 0; }
        for (uint32_t i = a0; i < a1; ++i) {
            uint32_t t = ord[first + i];
            const float* cc = &cent[3 * (size_t)t];
            for (int a = 0; a < 3; ++a) {
                if (!valid[a]) continue;
                int b = (int)((cc[a] - cmin[a]) * scale[a]);
                b = std::min(std::max(b, 0), kBins - 1);
                bn.b[a][b].grow((*c.tbox)[t]);
                bn.n[a][b]++;
            }
        }
    };
    std::unique_ptr<Bins> total(new Bins());
    uint32_t nt = (count > (1u << 18)) ? std::max(1u, nthreads) : 1u;
    if (nt == 1) {
        bin_range(0, count, *total);
    } else {
        std::vector<std::unique_ptr<Bins>> part(nt);
        for (uint32_t k = 0; k < nt; ++k) part[k].reset(new Bins());
        vgb::parallel_for_each(nt, [&](uint32_t k) {
            bin_range((uint32_t)((uint64_t)count * k / nt), (uint32_t)((uint64_t)count * (k + 1) / nt), *part[k]);
        });
        for (int a = 0; a < 3; ++a) for (int b = 0; b < kBins; ++b) {
            total->b[a][b] = Box(); total->n[a][b] = 0;
            for (uint32_t k = 0; k < nt; ++k) { total->b[a][b].grow(part[k]->b[a][b]); total->n[a][b] += part[k]->n[a][b]; }
        }
    }
    const float parent = nb.half_area();
    for (int a = 0; a < 3; ++a) {
        if (!valid[a]) continue;
        float rarea[kBins]; uint32_t rcnt[kBins];
        Box r; uint32_t rc = 0;
        for (int b = kBins - 1; b > 0; --b) {
            r.grow(total->b[a][b]); rc += total->n[a][b];
            rarea[b] = r.half_area(); rcnt[b] = rc;
        }
        Box l; uint32_t lc = 0;
        for (int b = 0; b < kBins - 1; ++b) {
            l.grow(total->b[a][b]); lc += total->n[a][b];
            if (lc == 0 || rcnt[b + 1] == 0) continue;
            float cost = VGB_SAH_TRAVERSAL_COST + ((float)lc * l.half_area() + (float)rcnt[b + 1] * rarea[b + 1]) /
                                    std::max(parent, 1e-30f);
            if (cost < best.cost) { best.cost = cost; best.axis = a; best.bin = b; best.cmin = cmin[a]; best.scale = scale[a]; }
        }
    }
    return best;
}

struct Arena { std::vector<BNode> nodes; };

// Recursive build into one arena.  Returns the node index.
uint32_t build_rec(const Ctx& c, Arena& ar, uint32_t arena_id, uint32_t first, uint32_t count,
                   uint32_t nthreads, uint32_t depth, uint32_t& max_depth) {
    uint32_t me = (uint32_t)ar.nodes.size();
    ar.nodes.emplace_back();
    Box nb;
    for (uint32_t i = 0; i < count; ++i) nb.grow((*c.tbox)[(*c.order)[first + i]]);
    ar.nodes[me].box = nb;
    max_depth = std::max(max_depth, depth);
    auto make_leaf = [&]() { ar.nodes[me].leaf = true; ar.nodes[me].first = first; ar.nodes[me].count = count; return me; };
    if (count <= 1) return make_leaf();
    Split s = find_split(c, first, count, nb, nthreads);
    if (count <= c.max_leaf && (s.axis < 0 || s.cost >= (float)count)) return make_leaf();
    uint32_t mid;
    auto& ord = *c.order;
    if (s.axis < 0) {
        mid = first + count / 2;  // all centroids coincide: split by position in the list
    } else {
        auto it = std::partition(ord.begin() + first, ord.begin() + first + count, [&](uint32_t t) {
            int b = (int)(((*c.cent)[3 * (size_t)t + s.axis] - s.cmin) * s.scale);
            b = std::min(std::max(b, 0), kBins - 1);
            return b <= s.bin;
        });
        mid = (uint32_t)(it - ord.begin());
        if (mid == first || mid == first + count) mid = first + count / 2;
    }
    uint32_t l = build_rec(c, ar, arena_id, first, mid - first, nthreads, depth + 1, max_depth);
    uint32_t r = build_rec(c, ar, arena_id, mid, first + count - mid, nthreads, depth + 1, max_depth);
    ar.nodes[me].child[0] = enc(arena_id, l);
    ar.nodes[me].child[1] = enc(arena_id, r);
    return me;
}

}  // namespace

bool build_bvh(const float* pos, uint32_t nverts, const uint32_t* idx, uint32_t ntris, uint32_t max_leaf,
               uint32_t threads, uint32_t layout, BvhHost& out, const char** err) {
    if (layout != 2 && layout != 8) { *err = "unknown BVH layout"; return false; }
    if (max_leaf == 0) max_leaf = (layout == 8) ? kMaxLeaf8 : 4;
    if (max_leaf > kMaxLeaf) max_leaf = kMaxLeaf;
    if (layout == 8 && max_leaf > kMaxLeaf8) max_leaf = kMaxLeaf8;
    if (threads == 0) threads = std::max(1u, std::thread::hardware_concurrency());
    if (ntris == 0) { *err = "scene has no triangles"; return false; }
    if ((uint64_t)ntris >= (1ull << (31 - kLeafShift))) { *err = "too many triangles for the leaf encoding"; return false; }
    std::vector<Box> tbox(ntris);
    std::vector<float> cent(3 * (size_t)ntris);
    std::vector<uint32_t> order(ntris);
    for (uint32_t t = 0; t < ntris; ++t) {
        Box b;
        for (int k = 0; k < 3; ++k) {
            uint32_t v = idx[3 * (size_t)t + k];
            if (v >= nverts) { *err = "triangle index out of range"; return false; }
            b.growp(&pos[3 * (size_t)v]);
        }
        for (int k = 0; k < 3; ++k) {
            if (!std::isfinite(b.lo[k]) || !std::isfinite(b.hi[k])) {
                // a triangle with an infinite vertex can never be hit: collapse it to a point
                // far outside the scene is not safe either, so give it an empty box at 0
                b.lo[k] = 0.f; b.hi[k] = 0.f;
            }
            cent[3 * (size_t)t + k] = 0.5f * b.lo[k] + 0.5f * b.hi[k];
        }
        tbox[t] = b;
        order[t] = t;
    }
    Ctx c{&tbox, &cent, &order, max_leaf, threads};

    // Top of the tree: split sequentially (with parallel binning) until there are enough
    // independent subtrees, then build those on threads, one arena each.
    std::vector<Arena> arenas(1);
    struct Task { uint32_t first, count; uint32_t parent; int side; uint32_t arena; };
    std::vector<Task> tasks;
    uint32_t max_depth = 0;
    const uint32_t task_min = std::max<uint32_t>(4096, ntris / (8 * threads));
    std::function<uint32_t(uint32_t, uint32_t, uint32_t)> top = [&](uint32_t first, uint32_t count, uint32_t depth) -> uint32_t {
        Arena& ar = arenas[0];
        uint32_t me = (uint32_t)ar.nodes.size();
        ar.nodes.emplace_back();
        Box nb;
        for (uint32_t i = 0; i < count; ++i) nb.grow(tbox[order[first + i]]);
        ar.nodes[me].box = nb;
        max_depth = std::max(max_depth, depth);
        Split s = find_split(c, first, count, nb, threads);
        if (count <= max_leaf && (s.axis < 0 || s.cost >= (float)count)) {
            ar.nodes[me].leaf = true; ar.nodes[me].first = first; ar.nodes[me].count = count; return me;
        }
        uint32_t mid;
        if (s.axis < 0) mid = first + count / 2;
        else {
            auto it = std::partition(order.begin() + first, order.begin() + first + count, [&](uint32_t t) {
                int b = (int)((cent[3 * (size_t)t + s.axis] - s.cmin) * s.scale);
                b = std::min(std::max(b, 0), kBins - 1);
                return b <= s.bin;
            });
            mid = (uint32_t)(it - order.begin());
            if (mid == first || mid == first + count) mid = first + count / 2;
        }
        uint32_t ranges[2][2] = {{first, mid - first}, {mid, first + count - mid}};
        for (int side = 0; side < 2; ++side) {
            uint32_t f = ranges[side][0], n = ranges[side][1];
            if (n > task_min && threads > 1) {
                uint32_t ch = top(f, n, depth + 1);
                arenas[0].nodes[me].child[side] = enc(0, ch);
            } else {
                uint32_t aid = (uint32_t)arenas.size();
                arenas.emplace_back();
                tasks.push_back(Task{f, n, me, side, aid});
                arenas[0].nodes[me].child[side] = enc(aid, 0);
            }
        }
        return me;
    };
    if (ntris > task_min && threads > 1) {
        top(0, ntris, 0);
    } else {
        build_rec(c, arenas[0], 0, 0, ntris, threads, 0, max_depth);
    }
    if (!tasks.empty()) {
        std::atomic<size_t> next{0};
        std::vector<uint32_t> depths(threads, 0);
        vgb::parallel_for_each(threads, [&](uint32_t k) {
            while (true) {
                size_t ti = next.fetch_add(1);
                if (ti >= tasks.size()) break;
                const Task& t = tasks[ti];
                uint32_t md = 0;
                build_rec(c, arenas[t.arena], t.arena, t.first, t.count, 1, 0, md);
                depths[k] = std::max(depths[k], md);
            }
        });
        uint32_t md = 0;
        for (uint32_t d : depths) md = std::max(md, d);
        max_depth += md + 1;
    }

    out.nodes.clear(); out.tris.clear(); out.parent.clear();
    out.tris.reserve(12 * (size_t)ntris);
    out.layout = layout;
    out.max_depth = max_depth;
    auto get = [&](int64_t ref) -> const BNode& { return arenas[(size_t)(ref >> 32)].nodes[(uint32_t)ref]; };
    auto emit_tri = [&](uint32_t t) {
        for (int k = 0; k < 3; ++k) {
            const float* p = &pos[3 * (size_t)idx[3 * (size_t)t + k]];
            out.tris.push_back(p[0]); out.tris.push_back(p[1]); out.tris.push_back(p[2]);
            uint32_t w = (k == 0) ? t : 0u;
            float wf; std::memcpy(&wf, &w, 4);
            out.tris.push_back(wf);
        }
    };
    const BNode& root = get(enc(0, 0));
    for (int k = 0; k < 3; ++k) { out.root_lo[k] = root.box.lo[k]; out.root_hi[k] = root.box.hi[k]; }
    std::vector<uint32_t>& words = out.nodes;

    if (layout == 2) {
        // ---- binary layout, depth first
        auto emit_leaf = [&](const BNode& n) -> int32_t {
            uint32_t start = (uint32_t)(out.tris.size() / 12);
            for (uint32_t i = 0; i < n.count; ++i) emit_tri(order[n.first + i]);
            return ~(int32_t)((start << kLeafShift) | (n.count - 1));
        };
        struct Item { int64_t ref; uint32_t slot; };
        std::vector<Item> stack;
        auto alloc = [&]() {
            uint32_t sl = (uint32_t)(words.size() / 16);
            words.resize(words.size() + 16, 0u);
            out.parent.push_back(kNoParent);
            return sl;
        };
        auto fbits = [](float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; };
        auto put_child = [&](uint32_t slot, int side, const Box& b, int32_t link) {
            uint32_t* n = &words[16 * (size_t)slot];
            if (side == 0) {
                n[0] = fbits(b.lo[0]); n[1] = fbits(b.hi[0]); n[2] = fbits(b.lo[1]); n[3] = fbits(b.hi[1]);
                n[8] = fbits(b.lo[2]); n[9] = fbits(b.hi[2]);
            } else {
                n[4] = fbits(b.lo[0]); n[5] = fbits(b.hi[0]); n[6] = fbits(b.lo[1]); n[7] = fbits(b.hi[1]);
                n[10] = fbits(b.lo[2]); n[11] = fbits(b.hi[2]);
            }
            n[12 + side] = (uint32_t)link;
        };
        uint32_t root_slot = alloc();
        if (root.leaf) {
            // both children are the root leaf: tested twice, found once
            int32_t link = emit_leaf(root);
            put_child(root_slot, 0, root.box, link);
            put_child(root_slot, 1, root.box, link);
        } else {
            stack.push_back(Item{enc(0, 0), root_slot});
            while (!stack.empty()) {
                Item it = stack.back(); stack.pop_back();
                const BNode& n = get(it.ref);
                for (int side = 0; side < 2; ++side) {
                    int64_t cr = n.child[side];
                    const BNode& ch = get(cr);
                    if (ch.leaf) {
                        put_child(it.slot, side, ch.box, emit_leaf(ch));
                    } else {
                        uint32_t sl = alloc();
                        out.parent[sl] = (it.slot << 1) | (uint32_t)side;
                        put_child(it.slot, side, ch.box, (int32_t)sl);
                        stack.push_back(Item{cr, sl});
                    }
                }
            }
        }
        out.num_nodes = (uint32_t)(words.size() / 16);
        return true;
    }

    // ---- 8-wide compressed layout (20 words per node), breadth first
    // w0..2 origin p (float), w3 biased exponents ex|ey<<8|ez<<16 and the internal-child mask <<24,
    // w4 first internal child, w5 first triangle, w6..7 meta bytes (0 empty, 0x80 internal,
    // count<<5|offset for a leaf of 1..3 triangles), w8..19 qlo_x, qlo_y, qlo_z, qhi_x, qhi_y,
    // qhi_z (8 bytes each).  Child boxes dequantise to p + 2^e * q, rounded outward so that the
    // FP32 evaluation contains the exact box.
    auto fbits = [](float f) { uint32_t u; std::memcpy(&u, &f, 4); return u; };
    std::vector<std::pair<int64_t, uint32_t>> queue;  // (build node, device node index)
    queue.reserve(ntris / 4 + 16);
    words.resize(20, 0u);
    queue.push_back({enc(0, 0), 0u});
    for (size_t qi = 0; qi < queue.size(); ++qi) {
        const int64_t ref = queue[qi].first;
        const uint32_t slot_index = queue[qi].second;
        const BNode& bn = get(ref);
        // collapse: open the largest internal child until there are 8
        std::vector<int64_t> ch;
        if (bn.leaf) ch.push_back(ref);
        else { ch.push_back(bn.child[0]); ch.push_back(bn.child[1]); }
        while (ch.size() < 8) {
            int best = -1; float best_area = -1.f;
            for (size_t c = 0; c < ch.size(); ++c) {
                const BNode& cn = get(ch[c]);
                if (cn.leaf) continue;
                float a = cn.box.half_area();
                if (a > best_area) { best_area = a; best = (int)c; }
            }
            if (best < 0) break;
            const BNode& op = get(ch[best]);
            int64_t l = op.child[0], r = op.child[1];
            ch[best] = l;
            ch.push_back(r);
        }
        const size_t nc = ch.size();
        Box nb;
        for (int64_t c : ch) nb.grow(get(c).box);
        // octant slots: the child in slot s is the nearest one for rays whose direction signs
        // are s (bit 0: x < 0, bit 1: y < 0, bit 2: z < 0); greedy assignment on
        // cost(c, s) = dot(centroid_c - centroid_node, D(s)), D(s) = (+-1, +-1, +-1)
        float pc[3];
        for (int k = 0; k < 3; ++k) pc[k] = 0.5f * nb.lo[k] + 0.5f * nb.hi[k];
        float cost[8][8];
        for (size_t c = 0; c < nc; ++c) {
            const Box& b = get(ch[c]).box;
            float d[3];
            for (int k = 0; k < 3; ++k) d[k] = (0.5f * b.lo[k] + 0.5f * b.hi[k]) - pc[k];
            for (int sl = 0; sl < 8; ++sl)
                cost[c][sl] = ((sl & 1) ? -d[0] : d[0]) + ((sl & 2) ? -d[1] : d[1]) + ((sl & 4) ? -d[2] : d[2]);
        }
        int slot_of[8];
        bool used_c[8] = {false}, used_s[8] = {false};
        for (size_t round = 0; round < nc; ++round) {
            int bc = -1, bs = -1; float bv = INFINITY;
            for (size_t c = 0; c < nc; ++c) {
                if (used_c[c]) continue;
                for (int sl = 0; sl < 8; ++sl)
                    if (!used_s[sl] && cost[c][sl] < bv) { bv = cost[c][sl]; bc = (int)c; bs = sl; }
            }
            used_c[bc] = true; used_s[bs] = true; slot_of[bc] = bs;
        }
        int64_t at_slot[8];
        for (int sl = 0; sl < 8; ++sl) at_slot[sl] = -1;
        for (size_t c = 0; c < nc; ++c) at_slot[slot_of[c]] = ch[c];
        // children records
        uint32_t imask = 0, n_internal = 0;
        for (int sl = 0; sl < 8; ++sl)
            if (at_slot[sl] >= 0 && !get(at_slot[sl]).leaf) { imask |= 1u << sl; n_internal++; }
        const uint32_t child_base = (uint32_t)(words.size() / 20);
        words.resize(words.size() + 20 * (size_t)n_internal, 0u);
        const uint32_t tri_base = (uint32_t)(out.tris.size() / 12);
        uint8_t meta[8] = {0};
        uint32_t off = 0, ci = 0;
        for (int sl = 0; sl < 8; ++sl) {
            if (at_slot[sl] < 0) continue;
            const BNode& cn = get(at_slot[sl]);
            if (cn.leaf) {
                meta[sl] = (uint8_t)((cn.count << 5) | off);
                for (uint32_t i = 0; i < cn.count; ++i) emit_tri(order[cn.first + i]);
                off += cn.count;
            } else {
                meta[sl] = 0x80;
                queue.push_back({at_slot[sl], child_base + ci});
                ci++;
            }
        }
        // quantisation
        uint8_t qlo[3][8], qhi[3][8];
        int ebias[3];
        float p[3];
        for (int a = 0; a < 3; ++a) {
            p[a] = nb.lo[a];
            const double ext = (double)nb.hi[a] - (double)nb.lo[a];
            int e = -126;
            if (ext > 0) {
                int ex;
                std::frexp(ext / 255.0, &ex);  // ext/255 < 2^ex
                e = std::max(-126, std::min(127, ex));
            }
            for (;; ++e) {
                const float scale = std::ldexp(1.0f, e);
                bool ok = (float)(p[a] + scale * 255.0f) >= nb.hi[a];
                for (int sl = 0; sl < 8 && ok; ++sl) {
                    if (at_slot[sl] < 0) { qlo[a][sl] = 0; qhi[a][sl] = 0; continue; }
                    const Box& b = get(at_slot[sl]).box;
                    double lo_q = std::floor(((double)b.lo[a] - (double)p[a]) / (double)scale);
                    double hi_q = std::ceil(((double)b.hi[a] - (double)p[a]) / (double)scale);
                    int lq = (int)std::max(0.0, std::min(255.0, lo_q));
                    int hq = (int)std::max(0.0, std::min(255.0, hi_q));
                    while (lq > 0 && (float)(p[a] + scale * (float)lq) > b.lo[a]) lq--;
                    while (hq < 255 && (float)(p[a] + scale * (float)hq) < b.hi[a]) hq++;
                    if ((float)(p[a] + scale * (float)lq) > b.lo[a] || (float)(p[a] + scale * (float)hq) < b.hi[a]) ok = false;
                    qlo[a][sl] = (uint8_t)lq; qhi[a][sl] = (uint8_t)hq;
                }
                if (ok || e >= 127) break;
            }
            ebias[a] = e + 127;
        }
        uint32_t* w = &words[20 * (size_t)slot_index];
        w[0] = fbits(p[0]); w[1] = fbits(p[1]); w[2] = fbits(p[2]);
        w[3] = (uint32_t)ebias[0] | ((uint32_t)ebias[1] << 8) | ((uint32_t)ebias[2] << 16) | (imask << 24);
        w[4] = child_base;
        w[5] = tri_base;
        w[6] = (uint32_t)meta[0] | ((uint32_t)meta[1] << 8) | ((uint32_t)meta[2] << 16) | ((uint32_t)meta[3] << 24);
        w[7] = (uint32_t)meta[4] | ((uint32_t)meta[5] << 8) | ((uint32_t)meta[6] << 16) | ((uint32_t)meta[7] << 24);
        auto pack8 = [](const uint8_t* q, uint32_t& lo, uint32_t& hi) {
            lo = (uint32_t)q[0] | ((uint32_t)q[1] << 8) | ((uint32_t)q[2] << 16) | ((uint32_t)q[3] << 24);
            hi = (uint32_t)q[4] | ((uint32_t)q[5] << 8) | ((uint32_t)q[6] << 16) | ((uint32_t)q[7] << 24);
        };
        pack8(qlo[0], w[8], w[9]); pack8(qlo[1], w[10], w[11]); pack8(qlo[2], w[12], w[13]);
        pack8(qhi[0], w[14], w[15]); pack8(qhi[1], w[16], w[17]); pack8(qhi[2], w[18], w[19]);
    }
    out.num_nodes = (uint32_t)(words.size() / 20);
    return true;
}

}  // namespace vgb
