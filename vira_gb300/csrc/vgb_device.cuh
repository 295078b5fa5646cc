// vgb_device.cuh -- device helpers of the hot path: counter-based RNG, the reference's FP32
// expression order, the watertight ray/triangle test and BVH traversal.
//
// The translation unit is compiled with --fmad=false: every `a * b + c` below rounds the
// product and the sum separately, exactly as the oracle (built with -ffp-contract=off) and
// the reference's glm code do.  Fused multiply-adds appear only where written explicitly.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/vgb.h"

namespace vgbd {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = (float)(1. / 3.141592653589793238462);
constexpr uint32_t kSlotMain = 0u, kSlotRR = 0xFEu, kSlotJitter = 0xFFu;

// device error word bits
constexpr uint32_t kErrStack = 1u, kErrIter = 2u;

constexpr int kStackSize = 64;
// 1: the wavefront traversal kernels postpone leaves speculatively (traverse_spec_rt).
#ifndef VGB_TRAV_SPECULATIVE
#define VGB_TRAV_SPECULATIVE 0
#endif
// 1: traverse_rt keeps each pushed child's entry distance on the stack and, for closest-hit
// rays, drops a popped entry whose box starts beyond the current closest hit without fetching it
// (the box test re-evaluated with the new bound; results unchanged).  Off: on the path-traced
// frame the closest-hit launches took 82.2 against 81.5 ms per frame with it.
#ifndef VGB_TRAV_CULL
#define VGB_TRAV_CULL 0
#endif
constexpr uint32_t kIterCap = 1u << 22;  // default traversal steps per ray before giving up

// ------------------------------------------------------------------ Philox-4x32-10
// Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC 2011.
struct U4 { uint32_t x, y, z, w; };
__device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1) {
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        if (r) { k0 += W0; k1 += W1; }
        uint32_t hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
        uint32_t hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
        c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    }
    return c;
}
__device__ __forceinline__ float u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

// std::max / std::min semantics (first argument wins on NaN comparisons)
__device__ __forceinline__ float smax(float a, float b) { return (a < b) ? b : a; }
__device__ __forceinline__ float smin(float a, float b) { return (b < a) ? b : a; }

struct F3 { float x, y, z; };
__device__ __forceinline__ F3 f3(float x, float y, float z) { return F3{x, y, z}; }
__device__ __forceinline__ F3 operator+(F3 a, F3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ F3 operator-(F3 a, F3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ F3 operator*(float s, F3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ F3 operator*(F3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ float dot(F3 a, F3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ F3 cross(F3 a, F3 b) {
    return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y};
}
__device__ __forceinline__ float length(F3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ F3 normalize(F3 a) { return a * (1.0f / sqrtf(dot(a, a))); }
__device__ __forceinline__ float pick(F3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
__device__ __forceinline__ F3 ld3(const float4& v) { return F3{v.x, v.y, v.z}; }

// offsetIntersection, float path (include/implementation/rendering/ray.ipp:107-123)
__device__ __forceinline__ float offset1(float p, float n) {
    const float origin = 1.f / 32.f, float_scale = 1.f / 65536.f, int_scale = 256.f;
    int32_t of = (int32_t)(int_scale * n);
    int32_t pi = __float_as_int(p) + ((p < 0) ? -of : of);
    return (fabsf(p) < origin) ? p + float_scale * n : __int_as_float(pi);
}

// ------------------------------------------------------------------ watertight test
// Woop, Benthin, Wald, "Watertight Ray/Triangle Intersection", JCGT 2(1), 2013.
struct WRay {
    F3 o, d;
    int kx, ky, kz;
    float Sx, Sy, Sz;
    float ix, iy, iz;  // slab reciprocals, |d| clamped away from 0
};

__device__ __forceinline__ float safe_rcp(float d) {
    const float tiny = 1e-30f;
    float a = fabsf(d) < tiny ? copysignf(tiny, d) : d;
    return 1.0f / a;
}

__device__ __forceinline__ WRay make_wray(F3 o, F3 d) {
    WRay r;
    r.o = o; r.d = d;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (pick(d, kz) < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.kx = kx; r.ky = ky; r.kz = kz;
    float dz = pick(d, kz);
    r.Sx = pick(d, kx) / dz;
    r.Sy = pick(d, ky) / dz;
    r.Sz = 1.0f / dz;
    r.ix = safe_rcp(d.x); r.iy = safe_rcp(d.y); r.iz = safe_rcp(d.z);
    return r;
}

// Returns false on a miss.  t > 0 required.  U, V, W: unnormalised weights of v0, v1, v2.
__device__ __forceinline__ bool wt_test(const WRay& r, F3 v0, F3 v1, F3 v2, float& t_out, float& U_out,
                                        float& V_out, float& W_out, float& det_out) {
    F3 A = v0 - r.o, B = v1 - r.o, C = v2 - r.o;
    float Akz = pick(A, r.kz), Bkz = pick(B, r.kz), Ckz = pick(C, r.kz);
    float Ax = pick(A, r.kx) - r.Sx * Akz;
    float Ay = pick(A, r.ky) - r.Sy * Akz;
    float Bx = pick(B, r.kx) - r.Sx * Bkz;
    float By = pick(B, r.ky) - r.Sy * Bkz;
    float Cx = pick(C, r.kx) - r.Sx * Ckz;
    float Cy = pick(C, r.ky) - r.Sy * Ckz;
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
    float T = (U * (r.Sz * Akz) + V * (r.Sz * Bkz)) + W * (r.Sz * Ckz);
    float t = T * (1.0f / det);
    if (!(t > 0.0f)) return false;
    t_out = t; U_out = U; V_out = V; W_out = W; det_out = det;
    return true;
}

// ------------------------------------------------------------------ BVH2 traversal
struct HitOut {
    float t;
    uint32_t id;
    float U, V, W, det;
};

struct Counters { uint32_t nodes, tris; };

__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}

// Per-ray constants of the slab test.  A plane distance is one fused multiply-add,
// fma(plane, 1/d, -(o/d) -+ e): with o/d rounded once, its error is a relative part below
// 2^-23 (the reciprocal and the fma) plus an absolute part below 2^-24 |o/d|, so each axis
// shifts its near plane down and its far plane up by e = 2^-20 |o/d| (16x that bound), and the
// exit distance is widened by 2^-20 for the relative part (Ize 2013).  No box that the exact
// slab test keeps is culled, so the closest hit does not depend on this arithmetic.
struct SlabRay {
    float ix, iy, iz, lx, hx, ly, hy, lz, hz;  // reciprocals; offsets of the lo and hi planes
};
__device__ __forceinline__ SlabRay make_slab(const WRay& r) {
    SlabRay q;
    q.ix = r.ix; q.iy = r.iy; q.iz = r.iz;
    const float ox = r.o.x * r.ix, oy = r.o.y * r.iy, oz = r.o.z * r.iz;
    const float ex = fabsf(ox) * 0x1p-20f, ey = fabsf(oy) * 0x1p-20f, ez = fabsf(oz) * 0x1p-20f;
    q.lx = (r.ix >= 0.f) ? (-ox - ex) : (-ox + ex);
    q.hx = (r.ix >= 0.f) ? (-ox + ex) : (-ox - ex);
    q.ly = (r.iy >= 0.f) ? (-oy - ey) : (-oy + ey);
    q.hy = (r.iy >= 0.f) ? (-oy + ey) : (-oy - ey);
    q.lz = (r.iz >= 0.f) ? (-oz - ez) : (-oz + ez);
    q.hz = (r.iz >= 0.f) ? (-oz + ez) : (-oz - ez);
    return q;
}

// Entry and exit distances of the box [lo, hi] clipped to [0, tfar] (exit widened).
__device__ __forceinline__ void slab(const SlabRay& q, float lox, float hix, float loy, float hiy, float loz,
                                     float hiz, float tfar, float& tn, float& tf) {
    const float widen = 1.0f + 0x1p-20f;
    const float a0 = fmaf(lox, q.ix, q.lx), a1 = fmaf(hix, q.ix, q.hx);
    const float b0 = fmaf(loy, q.iy, q.ly), b1 = fmaf(hiy, q.iy, q.hy);
    const float c0 = fmaf(loz, q.iz, q.lz), c1 = fmaf(hiz, q.iz, q.hz);
    tn = fmax3(fminf(a0, a1), fminf(b0, b1), fmaxf(fminf(c0, c1), 0.0f));
    tf = fmin3(fmaxf(a0, a1), fmaxf(b0, b1), fminf(fmaxf(c0, c1), tfar)) * widen;
}

// Closest hit (any = false; ties in t go to the smaller id) or occlusion (any = true, any
// hit with t <= tmax).  Box tests are conservative (make_slab).
// One body for both kinds of ray; the templated wrapper below passes `any` as a constant.
template <bool COUNT>
__device__ __forceinline__ void traverse_rt(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                            const WRay& r, float tmax, const bool any, HitOut& h, uint32_t& err,
                                            Counters& cnt, uint32_t cap) {
    int stack[kStackSize];
#if VGB_TRAV_CULL
    float stack_tn[kStackSize];   // entry distance of each stacked child's box
#endif
    int sp = 0;
    int node = 0;
    float best = any ? tmax : __int_as_float(0x7f800000);
    h.t = __int_as_float(0x7f800000);
    h.id = VGB_NO_HIT;
    uint32_t iter = 0;
    const SlabRay q = make_slab(r);
    // The next stacked node, or false when the stack is empty.  With culling, a closest-hit
    // ray skips entries whose box test, re-run against the current closest hit, would fail: the
    // test passes iff tn <= min(tf, best) * widen, and tn <= tf * widen held when it was pushed.
    auto pop = [&](int& nd) -> bool {
#if VGB_TRAV_CULL
        const float bound = best * (1.0f + 0x1p-20f);
        while (sp > 0) {
            --sp;
            if (!any && stack_tn[sp] > bound) continue;
            nd = stack[sp];
            return true;
        }
        return false;
#else
        if (sp == 0) return false;
        nd = stack[--sp];
        return true;
#endif
    };
    while (true) {
        while (node >= 0) {
            if (++iter > cap) { err |= kErrIter; return; }
            const float4 n0 = __ldg(&nodes[4 * node + 0]);
            const float4 n1 = __ldg(&nodes[4 * node + 1]);
            const float4 n2 = __ldg(&nodes[4 * node + 2]);
            const float4 n3 = __ldg(&nodes[4 * node + 3]);
            if (COUNT) cnt.nodes++;
            float tn0, tf0, tn1, tf1;
            slab(q, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, best, tn0, tf0);
            slab(q, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, best, tn1, tf1);
            const bool h0 = tn0 <= tf0, h1 = tn1 <= tf1;
            const int ch0 = __float_as_int(n3.x), ch1 = __float_as_int(n3.y);
            if (h0 && h1) {
                int nearc = ch0, farc = ch1;
                float tfar = tn1;
                if (tn1 < tn0) { nearc = ch1; farc = ch0; tfar = tn0; }
                if (sp >= kStackSize) { err |= kErrStack; return; }
#if VGB_TRAV_CULL
                stack_tn[sp] = tfar;
#else
                (void)tfar;
#endif
                stack[sp++] = farc;
                node = nearc;
            } else if (h0) {
                node = ch0;
            } else if (h1) {
                node = ch1;
            } else {
                if (!pop(node)) return;
            }
        }
        // leaf
        const uint32_t x = ~(uint32_t)node;
        const uint32_t start = x >> 3, cntl = (x & 7u) + 1u;
        for (uint32_t k = 0; k < cntl; ++k) {
            const float4 t0 = __ldg(&tris[3 * (start + k) + 0]);
            const float4 t1 = __ldg(&tris[3 * (start + k) + 1]);
            const float4 t2 = __ldg(&tris[3 * (start + k) + 2]);
            if (COUNT) cnt.tris++;
            float tt, U, V, W, det;
            if (wt_test(r, ld3(t0), ld3(t1), ld3(t2), tt, U, V, W, det)) {
                const uint32_t id = __float_as_uint(t0.w);
                if (any) {
                    if (tt <= tmax) { h.t = tt; h.id = id; return; }
                } else if (tt < h.t || (tt == h.t && id < h.id)) {
                    h.t = tt; h.id = id; h.U = U; h.V = V; h.W = W; h.det = det;
                    best = tt;
                }
            }
        }
        if (!pop(node)) return;
    }
}

// Resumable form of traverse_rt for the persistent traversal kernels: the state of one ray's
// traversal between calls (the stack itself lives in the caller's per-thread array).
struct TravState {
    int node;       // next node (>= 0 inner; < 0 a leaf to test)
    int sp;         // stack depth
    float best;     // closest-hit t so far (tmax for occlusion rays)
    uint32_t iter;  // inner nodes visited
};

__device__ __forceinline__ TravState trav_start(float tmax, bool any, HitOut& h) {
    h.t = __int_as_float(0x7f800000);
    h.id = VGB_NO_HIT;
    h.U = h.V = h.W = 0.f;
    h.det = 1.f;
    return TravState{0, 0, any ? tmax : __int_as_float(0x7f800000), 0u};
}

// Continues the traversal of ray r for at most `budget` inner-node visits.  Returns true when the
// ray is finished (h holds its answer), false when it stopped early; the next call resumes where it
// stopped.  Node order, box and triangle tests are traverse_rt's, so the answer is the same.
template <bool COUNT>
__device__ __forceinline__ bool traverse_resume(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                                const WRay& r, const SlabRay& q, float tmax, const bool any,
                                                int* stack, TravState& ts, HitOut& h, uint32_t& err, Counters& cnt,
                                                uint32_t cap, int budget) {
    int node = ts.node, sp = ts.sp;
    float best = ts.best;
    uint32_t iter = ts.iter;
    while (true) {
        while (node >= 0) {
            if (budget-- <= 0) {
                ts.node = node; ts.sp = sp; ts.best = best; ts.iter = iter;
                return false;
            }
            if (++iter > cap) { err |= kErrIter; return true; }
            const float4 n0 = __ldg(&nodes[4 * node + 0]);
            const float4 n1 = __ldg(&nodes[4 * node + 1]);
            const float4 n2 = __ldg(&nodes[4 * node + 2]);
            const float4 n3 = __ldg(&nodes[4 * node + 3]);
            if (COUNT) cnt.nodes++;
            float tn0, tf0, tn1, tf1;
            slab(q, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, best, tn0, tf0);
            slab(q, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, best, tn1, tf1);
            const bool h0 = tn0 <= tf0, h1 = tn1 <= tf1;
            const int ch0 = __float_as_int(n3.x), ch1 = __float_as_int(n3.y);
            if (h0 && h1) {
                int nearc = ch0, farc = ch1;
                if (tn1 < tn0) { nearc = ch1; farc = ch0; }
                if (sp >= kStackSize) { err |= kErrStack; return true; }
                stack[sp++] = farc;
                node = nearc;
            } else if (h0) {
                node = ch0;
            } else if (h1) {
                node = ch1;
            } else {
                if (sp == 0) return true;
                node = stack[--sp];
            }
        }
        const uint32_t x = ~(uint32_t)node;
        const uint32_t start = x >> 3, cntl = (x & 7u) + 1u;
        for (uint32_t k = 0; k < cntl; ++k) {
            const float4 t0 = __ldg(&tris[3 * (start + k) + 0]);
            const float4 t1 = __ldg(&tris[3 * (start + k) + 1]);
            const float4 t2 = __ldg(&tris[3 * (start + k) + 2]);
            if (COUNT) cnt.tris++;
            float tt, U, V, W, det;
            if (wt_test(r, ld3(t0), ld3(t1), ld3(t2), tt, U, V, W, det)) {
                const uint32_t id = __float_as_uint(t0.w);
                if (any) {
                    if (tt <= tmax) { h.t = tt; h.id = id; return true; }
                } else if (tt < h.t || (tt == h.t && id < h.id)) {
                    h.t = tt; h.id = id; h.U = U; h.V = V; h.W = W; h.det = det;
                    best = tt;
                }
            }
        }
        if (sp == 0) return true;
        node = stack[--sp];
    }
}

// Warp-packet traversal of the binary BVH for coherent rays (a warp's 8x4 pixel tile of camera
// rays, or their shadow rays towards one light).  Every lane of the warp calls it together; a
// lane with active = false only takes part.  The warp walks one node sequence: each node is
// fetched once for all lanes (the same address, one broadcast load), every active lane tests
// both child boxes against its own ray and current best distance, and a child is entered when
// any lane's ray overlaps it, the one more lanes reach first.  Leaves are tested by every active
// lane.  A lane thus tests a superset of the triangles its own traversal would test, with the
// same conservative box test and the same acceptance rule (closest t, ties to the smaller id;
// any hit within tmax), so its answer is the same as traverse_rt's: the closest hit does not
// depend on which boxes are opened, and an occlusion test only reports whether some triangle
// lies within tmax.  The warp's node stack (kStackSize = 64 entries) is spread over the lanes'
// registers: entry i is held by lane i % 32 in its register s0 (i < 32) or s1.
template <bool ANY>
__device__ __forceinline__ void traverse_packet(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                                const WRay& r, float tmax, bool active, HitOut& h, uint32_t& err,
                                                uint32_t cap) {
    static_assert(kStackSize == 64, "two stack registers per lane");
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    h.t = __int_as_float(0x7f800000);
    h.id = VGB_NO_HIT;
    float best = ANY ? tmax : __int_as_float(0x7f800000);
    bool live = active;
    const SlabRay q = make_slab(r);
    int sp = 0, node = 0, s0 = 0, s1 = 0;
    uint32_t iter = 0;
    if (!__any_sync(full, live)) return;
    while (true) {
        while (node >= 0) {
            if (++iter > cap) { if (live) err |= kErrIter; return; }
            const float4 n0 = __ldg(&nodes[4 * node + 0]);
            const float4 n1 = __ldg(&nodes[4 * node + 1]);
            const float4 n2 = __ldg(&nodes[4 * node + 2]);
            const float4 n3 = __ldg(&nodes[4 * node + 3]);
            bool h0 = false, h1 = false, near0 = false;
            if (live) {
                float tn0, tf0, tn1, tf1;
                slab(q, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, best, tn0, tf0);
                slab(q, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, best, tn1, tf1);
                h0 = tn0 <= tf0;
                h1 = tn1 <= tf1;
                near0 = h0 && (!h1 || tn0 <= tn1);
            }
            const unsigned m0 = __ballot_sync(full, h0), m1 = __ballot_sync(full, h1);
            const int ch0 = __float_as_int(n3.x), ch1 = __float_as_int(n3.y);
            if (m0 && m1) {
                const unsigned nm = __ballot_sync(full, near0);
                const bool first0 = 2 * __popc(nm) >= __popc(m0 | m1);
                if (sp >= kStackSize) { if (live) err |= kErrStack; return; }
                if (lane == (sp & 31)) {
                    if (sp < 32) s0 = first0 ? ch1 : ch0;
                    else s1 = first0 ? ch1 : ch0;
                }
                ++sp;
                node = first0 ? ch0 : ch1;
            } else if (m0) {
                node = ch0;
            } else if (m1) {
                node = ch1;
            } else {
                if (sp == 0) return;
                --sp;
                node = __shfl_sync(full, sp < 32 ? s0 : s1, sp & 31);
            }
        }
        const uint32_t x = ~(uint32_t)node;
        const uint32_t start = x >> 3, cntl = (x & 7u) + 1u;
        for (uint32_t k = 0; k < cntl; ++k) {
            const float4 t0 = __ldg(&tris[3 * (start + k) + 0]);
            const float4 t1 = __ldg(&tris[3 * (start + k) + 1]);
            const float4 t2 = __ldg(&tris[3 * (start + k) + 2]);
            float tt, U, V, W, det;
            if (live && wt_test(r, ld3(t0), ld3(t1), ld3(t2), tt, U, V, W, det)) {
                const uint32_t id = __float_as_uint(t0.w);
                if (ANY) {
                    if (tt <= tmax) { h.t = tt; h.id = id; live = false; }
                } else if (tt < h.t || (tt == h.t && id < h.id)) {
                    h.t = tt; h.id = id; h.U = U; h.V = V; h.W = W; h.det = det;
                    best = tt;
                }
            }
        }
        if (ANY && !__any_sync(full, live)) return;
        if (sp == 0) return;
        --sp;
        node = __shfl_sync(full, sp < 32 ? s0 : s1, sp & 31);
    }
}

// traverse_rt with speculative leaf postponing (Aila and Laine, HPG 2009, "speculative
// while-while"): a lane that reaches a leaf while others are still among inner nodes keeps the
// leaf aside and goes on to the next inner node; the warp tests leaves once every converged lane
// holds one.  The set of leaves tested and the acceptance rule are traverse_rt's, only their
// order changes, so the answer is the same (the closest hit does not depend on the order).
template <bool COUNT>
__device__ __forceinline__ void traverse_spec_rt(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                                 const WRay& r, float tmax, const bool any, HitOut& h,
                                                 uint32_t& err, Counters& cnt, uint32_t cap) {
    constexpr int kDone = 0x7fffffff;   // beyond every node index: traversal finished
    int stack[kStackSize];
    int sp = 0;
    int node = 0, leaf = kDone;          // leaf < 0: a postponed leaf
    float best = any ? tmax : __int_as_float(0x7f800000);
    h.t = __int_as_float(0x7f800000);
    h.id = VGB_NO_HIT;
    uint32_t iter = 0;
    const SlabRay q = make_slab(r);
    while (node != kDone || leaf < 0) {
        while (node >= 0 && node != kDone) {
            if (++iter > cap) { err |= kErrIter; return; }
            const float4 n0 = __ldg(&nodes[4 * node + 0]);
            const float4 n1 = __ldg(&nodes[4 * node + 1]);
            const float4 n2 = __ldg(&nodes[4 * node + 2]);
            const float4 n3 = __ldg(&nodes[4 * node + 3]);
            if (COUNT) cnt.nodes++;
            float tn0, tf0, tn1, tf1;
            slab(q, n0.x, n0.y, n0.z, n0.w, n2.x, n2.y, best, tn0, tf0);
            slab(q, n1.x, n1.y, n1.z, n1.w, n2.z, n2.w, best, tn1, tf1);
            const bool h0 = tn0 <= tf0, h1 = tn1 <= tf1;
            const int ch0 = __float_as_int(n3.x), ch1 = __float_as_int(n3.y);
            if (h0 && h1) {
                int nearc = ch0, farc = ch1;
                if (tn1 < tn0) { nearc = ch1; farc = ch0; }
                if (sp >= kStackSize) { err |= kErrStack; return; }
                stack[sp++] = farc;
                node = nearc;
            } else if (h0) {
                node = ch0;
            } else if (h1) {
                node = ch1;
            } else {
                node = sp ? stack[--sp] : kDone;
            }
            if (node < 0 && leaf >= 0) {   // postpone the first leaf, keep descending
                leaf = node;
                node = sp ? stack[--sp] : kDone;
            }
            if (!__any_sync(__activemask(), leaf >= 0)) break;
        }
        while (leaf < 0) {
            const uint32_t x = ~(uint32_t)leaf;
            const uint32_t start = x >> 3, cntl = (x & 7u) + 1u;
            for (uint32_t k = 0; k < cntl; ++k) {
                const float4 t0 = __ldg(&tris[3 * (start + k) + 0]);
                const float4 t1 = __ldg(&tris[3 * (start + k) + 1]);
                const float4 t2 = __ldg(&tris[3 * (start + k) + 2]);
                if (COUNT) cnt.tris++;
                float tt, U, V, W, det;
                if (wt_test(r, ld3(t0), ld3(t1), ld3(t2), tt, U, V, W, det)) {
                    const uint32_t id = __float_as_uint(t0.w);
                    if (any) {
                        if (tt <= tmax) { h.t = tt; h.id = id; return; }
                    } else if (tt < h.t || (tt == h.t && id < h.id)) {
                        h.t = tt; h.id = id; h.U = U; h.V = V; h.W = W; h.det = det;
                        best = tt;
                    }
                }
            }
            leaf = node;                   // the current node may be a leaf too
            if (node < 0) node = sp ? stack[--sp] : kDone;
        }
    }
}

template <bool ANY, bool COUNT>
__device__ __forceinline__ void traverse(const float4* __restrict__ nodes, const float4* __restrict__ tris,
                                         const WRay& r, float tmax, HitOut& h, uint32_t& err, Counters& cnt,
                                         uint32_t cap) {
#if VGB_TRAV_SPECULATIVE
    traverse_spec_rt<COUNT>(nodes, tris, r, tmax, ANY, h, err, cnt, cap);
#else
    traverse_rt<COUNT>(nodes, tris, r, tmax, ANY, h, err, cnt, cap);
#endif
}

// ------------------------------------------------------------------ compressed 8-wide traversal
// Node (80 bytes, five 16-byte words): origin p, biased exponents and internal-child mask,
// first internal child, first triangle, eight meta bytes and six arrays of eight 8-bit
// quantised bounds.  The child in slot s is the nearest for rays whose direction-sign octant
// is s; a ray of octant o visits slots o^0, o^1, ..., o^7.  The stack holds node groups: the
// first child index, the internal-child mask and the not-yet-visited hit slots in visiting order.
constexpr int kStack8 = 32;

__device__ __forceinline__ uint32_t octant_order(uint32_t m, uint32_t o) {
    // bit k of the result = bit (o ^ k) of m
    if (o & 1u) m = ((m & 0x55u) << 1) | ((m & 0xAAu) >> 1);
    if (o & 2u) m = ((m & 0x33u) << 2) | ((m & 0xCCu) >> 2);
    if (o & 4u) m = ((m & 0x0Fu) << 4) | ((m & 0xF0u) >> 4);
    return m;
}

// Quantised coordinate `byte` of w as a float, exactly: the byte goes into the mantissa of
// 2^23 (byte permute) and 2^23 is subtracted, so no integer-to-float conversion is issued.
__device__ __forceinline__ float q8(uint32_t w, int byte) {
    return __uint_as_float(__byte_perm(w, 0x4B000000u, 0x7440u | (uint32_t)byte)) - 8388608.0f;
}

// Nonzero bytes of w as a 4-bit mask (bit k: byte k != 0).
__device__ __forceinline__ uint32_t nonzero_bytes(uint32_t w) {
    const uint32_t m = ((w & 0x7F7F7F7Fu) + 0x7F7F7F7Fu | w) & 0x80808080u;
    return ((m >> 7) & 1u) | ((m >> 14) & 2u) | ((m >> 21) & 4u) | ((m >> 28) & 8u);
}

// Plane distances of one node axis for the ray: t(q) = fma(q, a, b -+ e) with a = 2^e_axis / d
// (exact) and b = (p - o) / d.  Against (p + 2^e q - o) / d in exact arithmetic the error is a
// relative part below 2^-23 (the final fma and the relative part of b), an absolute part below
// 2^-23 |b| (b's two roundings) and, because the builder bounds the FP32-rounded dequantised
// plane, not the exact one, an absolute part below 2^-24 |p + 2^e q| / |d|.  The margin
// e = 2^-20 (|b| + |1/d| (|p| + 255 * 2^e)) covers the absolute parts 8x; the relative part is
// covered by widening the exit distance by 2^-20, as in the binary test.
struct AxisPlanes { float a, bn, bf; };
__device__ __forceinline__ AxisPlanes axis_planes(float p, float s, float o, float inv) {
    const float a = s * inv;
    const float b = (p - o) * inv;
    const float e = 0x1p-20f * fmaf(fabsf(inv), fmaf(255.0f, s, fabsf(p)), fabsf(b));
    return AxisPlanes{a, b - e, b + e};
}

template <bool COUNT>
__device__ __forceinline__ void traverse8_rt(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                             const WRay& r, float tmax, const bool any, HitOut& h, uint32_t& err,
                                             Counters& cnt, uint32_t cap) {
    const float widen = 1.0f + 0x1p-20f;
    const uint32_t oct = (r.d.x < 0.f ? 1u : 0u) | (r.d.y < 0.f ? 2u : 0u) | (r.d.z < 0.f ? 4u : 0u);
    // the near plane of an axis is the box's low side for a positive reciprocal, else the high side
    const bool nx = r.ix < 0.f, ny = r.iy < 0.f, nz = r.iz < 0.f;
    uint2 stack[kStack8];
    int sp = 0;
    uint32_t node = 0;
    float best = any ? tmax : __int_as_float(0x7f800000);
    h.t = __int_as_float(0x7f800000);
    h.id = VGB_NO_HIT;
    uint32_t iter = 0;
    while (true) {
        if (++iter > cap) { err |= kErrIter; return; }
        const uint4 w0 = __ldg(&nodes[5 * node + 0]);
        const uint4 w1 = __ldg(&nodes[5 * node + 1]);
        const uint4 w2 = __ldg(&nodes[5 * node + 2]);
        const uint4 w3 = __ldg(&nodes[5 * node + 3]);
        const uint4 w4 = __ldg(&nodes[5 * node + 4]);
        if (COUNT) cnt.nodes++;
        const AxisPlanes X = axis_planes(__uint_as_float(w0.x), __uint_as_float((w0.w & 0xFFu) << 23), r.o.x, r.ix);
        const AxisPlanes Y = axis_planes(__uint_as_float(w0.y), __uint_as_float(((w0.w >> 8) & 0xFFu) << 23), r.o.y, r.iy);
        const AxisPlanes Z = axis_planes(__uint_as_float(w0.z), __uint_as_float(((w0.w >> 16) & 0xFFu) << 23), r.o.z, r.iz);
        const uint32_t imask = w0.w >> 24;
        const uint32_t child_base = w1.x, tri_base = w1.y;
        const uint32_t valid = nonzero_bytes(w1.z) | (nonzero_bytes(w1.w) << 4);
        // quantised near / far planes per axis, slots 0-3 and 4-7
        const uint32_t nx0 = nx ? w3.z : w2.x, nx1 = nx ? w3.w : w2.y, fx0 = nx ? w2.x : w3.z, fx1 = nx ? w2.y : w3.w;
        const uint32_t ny0 = ny ? w4.x : w2.z, ny1 = ny ? w4.y : w2.w, fy0 = ny ? w2.z : w4.x, fy1 = ny ? w2.w : w4.y;
        const uint32_t nz0 = nz ? w4.z : w3.x, nz1 = nz ? w4.w : w3.y, fz0 = nz ? w3.x : w4.z, fz1 = nz ? w3.y : w4.w;
        uint32_t hits = 0;
#pragma unroll
        for (int sl = 0; sl < 8; ++sl) {
            const int b = sl & 3;
            const float tnx = fmaf(q8(sl < 4 ? nx0 : nx1, b), X.a, X.bn), tfx = fmaf(q8(sl < 4 ? fx0 : fx1, b), X.a, X.bf);
            const float tny = fmaf(q8(sl < 4 ? ny0 : ny1, b), Y.a, Y.bn), tfy = fmaf(q8(sl < 4 ? fy0 : fy1, b), Y.a, Y.bf);
            const float tnz = fmaf(q8(sl < 4 ? nz0 : nz1, b), Z.a, Z.bn), tfz = fmaf(q8(sl < 4 ? fz0 : fz1, b), Z.a, Z.bf);
            const float tn = fmax3(tnx, tny, fmaxf(tnz, 0.0f));
            const float tf = fmin3(tfx, tfy, fminf(tfz, best)) * widen;
            hits |= (tn <= tf ? 1u : 0u) << sl;
        }
        hits &= valid;
        // triangles of the hit leaves of this node
        uint32_t leaves = hits & ~imask, tbits = 0;
        while (leaves) {
            const uint32_t sl = __ffs(leaves) - 1;
            leaves &= leaves - 1;
            const uint32_t meta = ((sl < 4 ? w1.z : w1.w) >> (8 * (sl & 3))) & 0xFFu;
            tbits |= ((1u << (meta >> 5)) - 1u) << (meta & 31u);
        }
        while (tbits) {
            const uint32_t k = __ffs(tbits) - 1;
            tbits &= tbits - 1;
            const uint32_t ti = tri_base + k;
            const float4 t0 = __ldg(&tris[3 * ti + 0]);
            const float4 t1 = __ldg(&tris[3 * ti + 1]);
            const float4 t2 = __ldg(&tris[3 * ti + 2]);
            if (COUNT) cnt.tris++;
            float tt, U, V, W, det;
            if (wt_test(r, ld3(t0), ld3(t1), ld3(t2), tt, U, V, W, det)) {
                const uint32_t id = __float_as_uint(t0.w);
                if (any) {
                    if (tt <= tmax) { h.t = tt; h.id = id; return; }
                } else if (tt < h.t || (tt == h.t && id < h.id)) {
                    h.t = tt; h.id = id; h.U = U; h.V = V; h.W = W; h.det = det;
                    best = tt;
                }
            }
        }
        // next node: the nearest remaining hit child of this node, else of the stacked groups
        uint32_t pending = octant_order(hits & imask, oct), base = child_base, im = imask;
        if (!pending) {
            if (sp == 0) return;
            const uint2 g = stack[--sp];
            base = g.x; pending = g.y & 0xFFu; im = g.y >> 8;
        }
        const uint32_t k = __ffs(pending) - 1;
        pending &= pending - 1;
        const uint32_t slot = oct ^ k;
        node = base + __popc(im & ((1u << slot) - 1u));
        if (pending) {
            if (sp >= kStack8) { err |= kErrStack; return; }
            stack[sp++] = make_uint2(base, pending | (im << 8));
        }
    }
}

template <bool ANY, bool COUNT>
__device__ __forceinline__ void traverse8(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                          const WRay& r, float tmax, HitOut& h, uint32_t& err, Counters& cnt,
                                          uint32_t cap) {
    traverse8_rt<COUNT>(nodes, tris, r, tmax, ANY, h, err, cnt, cap);
}

// Dispatch on the node layout (2: binary, 8: compressed 8-wide).  `cap`: traversal steps per
// ray before the ray gives up and sets kErrIter.
template <int LAYOUT, bool ANY, bool COUNT>
__device__ __forceinline__ void traverse_any_layout(const uint4* __restrict__ nodes, const float4* __restrict__ tris,
                                                    const WRay& r, float tmax, HitOut& h, uint32_t& err, Counters& cnt,
                                                    uint32_t cap) {
    if (LAYOUT == 8) traverse8<ANY, COUNT>(nodes, tris, r, tmax, h, err, cnt, cap);
    else traverse<ANY, COUNT>(reinterpret_cast<const float4*>(nodes), tris, r, tmax, h, err, cnt, cap);
}

}  // namespace vgbd
