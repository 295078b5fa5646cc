// vgb_cuda.cu -- wavefront path-tracing kernels for sm_103a and the C ABI around them.
//
// Stages of one render (CPUPathTracer::render, cpu_path_tracer.ipp:29-161), per sample:
//   k_trace   (bounce 0: camera rays over all pixels, 8x4-pixel warp tiles; bounce b>0: the
//              compacted queue of live paths)  closest-hit traversal, one hit record per ray;
//   k_shade   processIntersection for the same items: AOVs, shading point, origin offset, NEE
//              shadow-ray enqueue (one queue per light), cosine bounce sampling, throughput
//              update, live-path enqueue (warp ballot);
//   k_shadow  (one launch per light)  occlusion traversal of the queued shadow rays, adding
//              each unoccluded contribution to the path's per-bounce radiance;
//   k_end_sample  per pixel: folds the last bounce's radiance into the path and the path into
//              the pixel; on the last sample writes the RenderPasses planes.
// Path state, queues and accumulators are structure-of-arrays planes indexed by pixel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <type_traits>
#include <vector>

#include "../../include/vgb.h"
#include "vgb_device.cuh"
#include "vgb_internal.h"

using namespace vgbd;

#define VGB_MAX_LIGHTS 8

// Minimum resident blocks per SM requested from the register allocator (occupancy knobs).
// Defaults from a sweep on the path-traced workload (GB300, 256-thread blocks).
#ifndef VGB_TRACE_MINB
#define VGB_TRACE_MINB 5
#endif
#ifndef VGB_SHADE_MINB
#define VGB_SHADE_MINB 4
#endif
// k_batch without bounces: 2 blocks of 256 threads cap it at 128 registers; with the traversal
// out of line this measured fastest on the trajectory workload (64 and 80 registers spill).
#ifndef VGB_BATCH_DIRECT_MINB
#define VGB_BATCH_DIRECT_MINB 2
#endif
// k_batch_direct: per-lane register sums, no shared memory; 4 blocks of 256 threads per SM cap it
// at 64 registers.  On the 256-frame trajectory: 1.16-1.17 s at 64 registers, 1.21 s at 5 blocks
// (48 registers), 1.36 s at 6, 1.26 s at 80 registers, 1.47 s at 128.
#ifndef VGB_BATCH_LEAN_MINB
#define VGB_BATCH_LEAN_MINB 4
#endif
// 1: k_batch_direct calls the out-of-line traversal (trace_ool) for camera and shadow rays
// instead of inlining a closest-hit and an occlusion copy of the loop.  On the 256-frame
// trajectory: 1.07 s against 1.17 s inlined (64 registers both; 1.11 s at 48, 1.14 s at 85).
#ifndef VGB_BATCH_LEAN_OOL
#define VGB_BATCH_LEAN_OOL 1
#endif
// 1: k_batch_direct traces a tile's camera rays and shadow rays as warp packets (binary layout).
// Off: on the 256-frame trajectory the packets took 1.45 s against 1.17 s for one traversal per
// lane (same results; 64 registers each).
#ifndef VGB_BATCH_PACKET
#define VGB_BATCH_PACKET 0
#endif
// >= 0: the shared-memory carveout (percent of the maximum) requested for the traversal and
// shading kernels, which use no shared memory; the rest of the SM's 256 KB is L1.  -1 leaves the
// driver's choice, which measured the same as 0 on the path-traced frame (100 lost 12 %).
#ifndef VGB_L1_CARVEOUT
#define VGB_L1_CARVEOUT -1
#endif
// > 0: before each continuation bounce, k_bin_rays sorts the live-path queue into this many
// bins by the rays' vertical direction component, and k_trace takes its items bin by bin (the
// hit records keep the queue order, so k_shade reads them unchanged).  Up to 8.  Off: on the
// path-traced frame 4 bins cut the closest-hit time by under 2 % and the binning pass cost more
// (3469 and 3485 Mrays/s with 4 and 8 bins against 3639).
#ifndef VGB_TRACE_BINS
#define VGB_TRACE_BINS 0
#endif
#ifndef VGB_SHADOW_MINB
#define VGB_SHADOW_MINB 5
#endif
// the same two knobs for the compressed 8-wide layout (k_trace<8>, k_shadow<NB, 8>)
#ifndef VGB_TRACE8_MINB
#define VGB_TRACE8_MINB 5
#endif
#ifndef VGB_SHADOW8_MINB
#define VGB_SHADOW8_MINB 5
#endif
// Grids of the wavefront kernels (grid-stride loops over the bounce's items), in blocks per SM;
// 0 launches one 256-thread block per 256 items.  Many waves of short blocks let the block
// scheduler even out rays of uneven cost: on the path-traced frame (2048^2 items) the closest-hit
// launch fell from 380 us at 8 blocks per SM to 332 us at 60, and the frame from 249 to 224 ms.
#ifndef VGB_TRACE_GRID
#define VGB_TRACE_GRID 60
#endif
#ifndef VGB_SHADE_GRID
#define VGB_SHADE_GRID 48
#endif
#ifndef VGB_END_GRID
#define VGB_END_GRID 8
#endif
// Threads per block of the closest-hit, occlusion and shading launches (the grids above and the
// minimum resident blocks scale with it, so occupancy and threads per SM stay the same).  Small
// blocks retire as soon as their own warps finish, so fewer warp slots idle behind the slowest
// ray of a block: on the path-traced frame 3653 Mrays/s at 256 threads, 3763 at 128, 3788 at 64
// for k_trace and k_shadow.
#ifndef VGB_TRACE_BLOCK
#define VGB_TRACE_BLOCK 64
#endif
#ifndef VGB_SHADOW_BLOCK
#define VGB_SHADOW_BLOCK 64
#endif
#ifndef VGB_SHADE_BLOCK
#define VGB_SHADE_BLOCK 256
#endif
#ifndef VGB_SHADOW_GRID
#define VGB_SHADOW_GRID 60
#endif
// k_adjoint (128-thread blocks over the frame's pixels): blocks per SM as above, and pixels per
// block before the cap.  One pixel per thread replayed the inversion workload's 16 views of 512^2
// in 0.156 s against 0.169 s at two per thread (16 blocks per SM).
// k_trace_batch (vgb_trace_rays), in blocks per SM as above: 4.2M device-resident closest-hit rays
// on a 2049^2 DEM (8.4M triangles) took 0.326 / 1.44 ms (one eye / scattered origins and random
// directions) at 60 blocks per SM against 0.418 / 2.01 ms at 8.
#ifndef VGB_RAYS_GRID
#define VGB_RAYS_GRID 60
#endif
// Persistent traversal kernels (off by default, vgb_set_wavefront_tuning): inner-node visits a
// lane's ray advances between hand-outs of new rays, and how many free lanes of a warp trigger a
// hand-out.  On the path-traced frame (GB300, 64 registers) they ran at 3096-3361 Mrays/s
// (budget 8-64, refill 1-16; best budget 32, refill 8) against 3639 for the grid-stride kernels:
// the closest-hit launches broke even at budget 32 and the occlusion launches lost 25 %.
#ifndef VGB_TRACEP_MINB
#define VGB_TRACEP_MINB 4
#endif
#ifndef VGB_SHADOWP_MINB
#define VGB_SHADOWP_MINB 4
#endif
#ifndef VGB_TRAV_BUDGET
#define VGB_TRAV_BUDGET 32
#endif
#ifndef VGB_TRAV_REFILL
#define VGB_TRAV_REFILL 8
#endif
#ifndef VGB_ADJOINT_GRID
#define VGB_ADJOINT_GRID 32
#endif
#ifndef VGB_ADJOINT_BLOCK_ITEMS
#define VGB_ADJOINT_BLOCK_ITEMS 128
#endif
// threads per block of k_adjoint and of k_trace_batch (vgb_trace_rays).  4.2M device-resident
// closest-hit rays on a 2049^2 DEM: 0.954 / 0.806 ms (from one eye / scattered) at 256 threads,
// 0.918 / 0.674 at 128, 0.913 / 0.654 at 64.  The inversion workload's backward pass: 0.159 s
// at 128 threads, 0.154 s at 256 (same threads per SM in the grid), 0.160 s at 64.
#ifndef VGB_ADJOINT_BLOCK
#define VGB_ADJOINT_BLOCK 256
#endif
#ifndef VGB_RAYS_BLOCK
#define VGB_RAYS_BLOCK 64
#endif

namespace {

// ------------------------------------------------------------------ device data
struct DevScene {
    const uint4* nodes;    // binary (4 words per node) or compressed 8-wide (5 words per node)
    const float4* tris;
    const uint32_t* idx;   // 3 per triangle, caller order
    const float4* vpos;    // xyz
    const float4* vnrm;    // xyz
    const float2* vuv;
    const float* valb;     // B per vertex (unused when albedo_uniform)
    const float* tex;      // [th][tw][B], or [th][tw] when tex_mono
    uint32_t tw, th;
    const float* nmap;     // [nh][nw][3] tangent-space normal map, or null (Material::normalMap)
    uint32_t nw, nh;
    const vgb_instance_motion* motion;   // per-instance motion, ascending first_triangle, or null
    uint32_t nmotion;
    uint32_t iter_cap;                // traversal steps per ray before it gives up (device error word)
    uint32_t albedo_uniform;          // every vertex has the albedo `albedo_value`
    uint32_t tex_mono;                // every texel has the same value in all bands
    float albedo_value[VGB_MAX_BANDS];
};

struct DevState {
    // per-pixel path state
    float* org;    // [3][P]
    float* dir;    // [3][P]
    float* thr;    // [B][P]
    float* prad;   // [B][P]   radiance of the current sample's path
    float* brad;   // [B][P]   radiance of the current bounce (ambient + NEE)
    uint32_t* pend;  // [P]    0: nothing to fold, 1: bounce-0 radiance, 2: later bounce
    // per-pixel accumulators over samples
    float* arad;   // [B][P]
    float* adir;   // [B][P]
    float* aalb;   // [B][P]
    float* anrm;   // [3][P]
    float* adep;   // [P]
    uint32_t* acnt;   // [P]
    uint32_t* atri;   // [P]
    // queues
    uint32_t* pq[2];  // path queues (slots)
    float* sq_org[VGB_MAX_LIGHTS];   // [3][P]
    float* sq_dir[VGB_MAX_LIGHTS];   // [3][P]
    float* sq_tmax[VGB_MAX_LIGHTS];  // [P]
    uint32_t* sq_slot[VGB_MAX_LIGHTS];
    float* sq_con[VGB_MAX_LIGHTS];   // [B][P]
    float4* hit;         // [P] closest-hit record per queue item: (t, id bits, w(v1), w(v2))
    uint32_t* binq;      // [VGB_TRACE_BINS][P] queue items binned by ray direction (null: off)
    // adaptive sampling: per pixel the sums of the path-radiance magnitude and of its square,
    // and the sample index at which the pixel stopped (0 while it samples on)
    float* as1;
    float* as2;
    uint32_t* anum;
    uint32_t* counters;  // see C_* below
    uint64_t* stats;     // [0] nodes, [1] tris, [2] closest rays, [3] shadow rays
    size_t P;            // plane stride
};

// Device counters: live-path queue lengths, shadow queue lengths per light, the item counters of
// the persistent closest-hit and occlusion launches (reset with the shadow queues each bounce),
// the error word and the batch kernels' work counter.
enum {
    C_PQ0 = 0, C_PQ1 = 1, C_SQ = 2, C_FTRACE = 2 + VGB_MAX_LIGHTS, C_FSHADOW = 3 + VGB_MAX_LIGHTS,
    C_ERR = 3 + 2 * VGB_MAX_LIGHTS, C_BATCH = 4 + 2 * VGB_MAX_LIGHTS, C_BIN = 5 + 2 * VGB_MAX_LIGHTS,
    C_COUNT = C_BIN + 8
};
// counters cleared at the start of every bounce: the shadow queues and the persistent item counters
constexpr int kBounceResetWords = 1 + 2 * VGB_MAX_LIGHTS;

struct FrameParams {
    vgb_camera cam;
    vgb_pt_options opt;
    vgb_light lights[VGB_MAX_LIGHTS];
    uint32_t nlights;
    uint32_t nb;
    uint32_t tiles_x, tiles_y;
    uint32_t aux;   // AUX_* bits: the per-pixel sums the requested film planes need
    // first-hit film planes k_shade writes directly (null when not requested)
    float *vel_g, *vel_c, *tsz;
};

// Per-pixel sums kept over the samples only when a requested film plane reads them (the total
// radiance sum is always kept): albedo, normal, direct radiance (direct and indirect planes),
// depth and hit count (depth and alpha planes), first triangle.
enum : uint32_t { AUX_ALB = 1u, AUX_NRM = 2u, AUX_DIR = 4u, AUX_DEP = 8u, AUX_TRI = 16u };

// Fold state of a pixel's path (DevState::pend): bits 0-1 what the bounce radiance holds
// (0 nothing, 1 bounce-0 radiance, 2 a later bounce's), bit 2 set while the path radiance has
// not been written this sample (it reads as 0).
constexpr uint32_t kPendMask = 3u, kPradEmpty = 4u;

struct FilmOut {
    float *total, *direct, *indirect, *power, *albedo, *normal, *depth, *alpha;
    uint32_t* tri;
    const float* omega;
    float *vel_g, *vel_c, *tsz;   // first-hit passes (velocity in the scene and camera frames, triangle size)
};

// The AUX_* sums that the planes of a film read.
inline uint32_t aux_for(const FilmOut& f) {
    // the first-hit passes find a pixel's first hit through its first-triangle sum
    return (f.albedo ? AUX_ALB : 0u) | (f.normal ? AUX_NRM : 0u) | ((f.direct || f.indirect) ? AUX_DIR : 0u) |
           ((f.depth || f.alpha) ? AUX_DEP : 0u) | ((f.tri || f.vel_g || f.vel_c || f.tsz) ? AUX_TRI : 0u);
}

__device__ __forceinline__ void warp_reduce_add(uint64_t* dst, uint32_t v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0 && v) atomicAdd((unsigned long long*)dst, (unsigned long long)v);
}

// warp-aggregated queue append; every lane of the warp must call it
__device__ __forceinline__ uint32_t warp_append(uint32_t* count, bool pred) {
    const unsigned mask = __ballot_sync(0xffffffffu, pred);
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (mask) {
        const int leader = __ffs(mask) - 1;
        if (lane == leader) base = atomicAdd(count, (uint32_t)__popc(mask));
        base = __shfl_sync(0xffffffffu, base, leader);
    }
    return base + (uint32_t)__popc(mask & ((1u << lane) - 1u));
}

// SphereLight::sample with and without RNG (sphere_light.ipp:31-124)
__device__ __forceinline__ void light_sample(const vgb_light& L, F3 p, bool det, float rand1, float rand2,
                                             F3& dir, float& distance, float& pdf) {
    F3 c{L.position[0], L.position[1], L.position[2]};
    F3 ptl = c - p;
    distance = length(ptl);
    float dinv = 1.0f / distance;
    float r = L.radius;
    if (det) {
        dir = dinv * ptl;
        if (distance <= r) {
            if (distance < 1e-3f) dir = F3{1, 0, 0};
            distance = r;
            pdf = 1.0f / (4.0f * kPi * r * r);
            return;
        }
        float r2 = r * r;
        float omega = 2 * kPi * (1.f - sqrtf((distance * distance) - r2) / distance);
        pdf = 1.f / omega;
        return;
    }
    F3 W = dinv * ptl;
    F3 N1{1, 0, 0}, N2{0, 1, 0};
    F3 N = (dot(N1, W) < dot(N2, W)) ? N1 : N2;
    F3 Vv = normalize(cross(W, N));
    F3 U = normalize(cross(W, Vv));
    float phi = 2 * kPi * rand1;
    float zeta = rand2;
    float cc = r / distance;
    float theta = acosf(1 - zeta + zeta * sqrtf(1 - (cc * cc)));
    float sinT = sinf(theta), sinP = sinf(phi), cosT = cosf(theta), cosP = cosf(phi);
    float a = cosP * sinT, b = cosT, e = sinP * sinT;
    dir = F3{(a * U.x + b * W.x) + e * Vv.x, (a * U.y + b * W.y) + e * Vv.y, (a * U.z + b * W.z) + e * Vv.z};
    float r2 = r * r;
    float omega = 2 * kPi * (1.f - sqrtf((distance * distance) - r2) / distance);
    pdf = 1.f / omega;
}

// SphereLight::getPDF (sphere_light.ipp:127-153)
__device__ __forceinline__ float light_pdf(const vgb_light& L, F3 p, F3 dir) {
    F3 c{L.position[0], L.position[1], L.position[2]};
    F3 tc = c - p;
    float dc = length(tc);
    float r = L.radius;
    if (dc <= r) return 1.0f / (4.0f * kPi * r * r);
    F3 tcn{tc.x / dc, tc.y / dc, tc.z / dc};
    float cosmax = sqrtf(1.0f - (r * r) / (dc * dc));
    float ca = dot(dir, tcn);
    if (ca < cosmax) return 0.0f;
    float r2 = r * r, d2 = dc * dc;
    float omega = 2 * kPi * (1.0f - sqrtf(d2 - r2) / dc);
    return 1.0f / omega;
}

__device__ __forceinline__ float power_heuristic(float fpdf, float gpdf) {
    float f = 1.0f * fpdf, g = 1.0f * gpdf;
    return (f * f) / (f * f + g * g);
}

// ConcentricDiskSample + CosineHemisphereSample (sampling.ipp:53-84)
__device__ __forceinline__ F3 cosine_sample(float rand1, float rand2) {
    float ux = 2.f * rand1 - 1.f, uy = 2.f * rand2 - 1.f;
    float dx, dy;
    if (fabsf(ux) < 1e-6f && fabsf(uy) < 1e-6f) {
        dx = 0; dy = 0;
    } else {
        float theta, r;
        const float P4 = kPi / 4.0f, P2 = kPi / 2.0f;
        if (fabsf(ux) > fabsf(uy)) { r = ux; theta = P4 * (uy / ux); }
        else { r = uy; theta = P2 - P4 * (ux / uy); }
        dx = r * cosf(theta); dy = r * sinf(theta);
    }
    float z = sqrtf(smax(0.f, 1 - dx * dx - dy * dy));
    return F3{dx, dy, z};
}

// Image::sampleUVs + interpolatePixel (image.ipp:589-671), one band
template <int NB>
__device__ __forceinline__ void sample_uvs(const DevScene& s, uint32_t nb, float u, float v, float* out) {
    float rx = (float)s.tw, ry = (float)s.th;
    float px = fmodf(u * rx, rx), py = fmodf(v * ry, ry);
    if (px < 0) px += rx;
    if (py < 0) py += ry;
    int x0 = (int)floorf(px), y0 = (int)floorf(py);
    x0 = min(x0, (int)s.tw - 1); y0 = min(y0, (int)s.th - 1);
    int x1 = min(x0 + 1, (int)s.tw - 1), y1 = min(y0 + 1, (int)s.th - 1);
    float dx = px - (float)x0, dy = py - (float)y0;
    float a = (1.f - dx) * (1.f - dy), b = dx * (1.f - dy), c = (1.f - dx) * dy, e = dx * dy;
    if (s.tex_mono) {
        // the bands of every texel are equal: one fetch per texel, the same per-band arithmetic
        const float t00 = __ldg(&s.tex[(size_t)y0 * s.tw + x0]), t10 = __ldg(&s.tex[(size_t)y0 * s.tw + x1]);
        const float t01 = __ldg(&s.tex[(size_t)y1 * s.tw + x0]), t11 = __ldg(&s.tex[(size_t)y1 * s.tw + x1]);
        const float val = ((a * t00 + b * t10) + c * t01) + e * t11;
#pragma unroll
        for (int k = 0; k < NB; ++k) out[k] = val;
        return;
    }
    const float* p00 = &s.tex[((size_t)y0 * s.tw + x0) * nb];
    const float* p10 = &s.tex[((size_t)y0 * s.tw + x1) * nb];
    const float* p01 = &s.tex[((size_t)y1 * s.tw + x0) * nb];
    const float* p11 = &s.tex[((size_t)y1 * s.tw + x1) * nb];
#pragma unroll
    for (int k = 0; k < NB; ++k)
        if (k < (int)nb) out[k] = ((a * __ldg(p00 + k) + b * __ldg(p10 + k)) + c * __ldg(p01 + k)) + e * __ldg(p11 + k);
}

// Image<Normal>::sampleUVs of the normal map (wrap + bilinear, image.ipp:589-671).
__device__ __forceinline__ F3 sample_normal_map(const DevScene& s, float u, float v) {
    const float rx = (float)s.nw, ry = (float)s.nh;
    float px = fmodf(u * rx, rx), py = fmodf(v * ry, ry);
    if (px < 0) px += rx;
    if (py < 0) py += ry;
    int x0 = (int)floorf(px), y0 = (int)floorf(py);
    x0 = min(x0, (int)s.nw - 1); y0 = min(y0, (int)s.nh - 1);
    const int x1 = min(x0 + 1, (int)s.nw - 1), y1 = min(y0 + 1, (int)s.nh - 1);
    const float dx = px - (float)x0, dy = py - (float)y0;
    const float* p00 = &s.nmap[((size_t)y0 * s.nw + x0) * 3];
    const float* p10 = &s.nmap[((size_t)y0 * s.nw + x1) * 3];
    const float* p01 = &s.nmap[((size_t)y1 * s.nw + x0) * 3];
    const float* p11 = &s.nmap[((size_t)y1 * s.nw + x1) * 3];
    const F3 a{__ldg(p00), __ldg(p00 + 1), __ldg(p00 + 2)}, b{__ldg(p10), __ldg(p10 + 1), __ldg(p10 + 2)};
    const F3 c{__ldg(p01), __ldg(p01 + 1), __ldg(p01 + 2)}, e{__ldg(p11), __ldg(p11 + 1), __ldg(p11 + 2)};
    return (((1.f - dx) * (1.f - dy) * a + dx * (1.f - dy) * b) + (1.f - dx) * dy * c) + dx * dy * e;
}

// Material::getNormal (materials/material.ipp:129-143): the tangent-space normal map sample taken
// to the scene frame by [tangent | bitangent | N] and normalised; N itself without a map.
// Out of line: a scene without a normal map never runs it, and the kernels that shade keep a
// smaller instruction footprint.
__device__ __noinline__ F3 normal_from_map(const DevScene& s, float u, float v, F3 N, F3 tg, F3 bt) {
    const F3 t = sample_normal_map(s, u, v);
    return normalize(F3{(tg.x * t.x + bt.x * t.y) + N.x * t.z, (tg.y * t.x + bt.y * t.y) + N.y * t.z,
                        (tg.z * t.x + bt.z * t.y) + N.z * t.z});
}
__device__ __forceinline__ F3 mapped_normal(const DevScene& s, float u, float v, F3 N, F3 tg, F3 bt) {
    if (!s.nmap) return N;
    return normal_from_map(s, u, v, N, tg, bt);
}

// The tangent frame of the shading normal (cpu_path_tracer.ipp:318-321).
__device__ __forceinline__ void tangent_frame(F3 N, F3& tg, F3& bt) {
    F3 arb = (fabsf(N.x) < 0.9f) ? F3{1, 0, 0} : F3{0, 1, 0};
    tg = normalize(cross(arb, N));
    bt = cross(N, tg);
}

// processIntersection up to the shading point (cpu_path_tracer.ipp:295-346): uv, face and
// shading normals, tangent frame, the normal map, albedo (vertex albedo x texture), interpolated
// position and computeShadingPoint (:494-511).  The normal matrix is the identity in the
// flattened frame.  N: the shading normal after the normal map (NEE, MIS and the film's normal);
// (tg, bt, nf): the tangent frame built before the map, which the continuation samples in;
// FRAME = false for callers that sample no continuation (tg and bt are then left unset unless
// the scene has a normal map, which needs them).
template <int NB, bool FRAME = true>
__device__ __forceinline__ void surface_at(const DevScene& s, uint32_t nb, bool smooth, uint32_t t, float w0f,
                                           float w1f, F3& Pp, F3& N, F3& fnrm, F3& tg, F3& bt, F3& nf, float* alb,
                                           float* va_out = nullptr, float* tex_out = nullptr, float* uv_out = nullptr) {
    float w[3];
    w[0] = w0f;
    w[1] = w1f;
    w[2] = 1.0f - w[0] - w[1];
    const uint32_t i0 = __ldg(&s.idx[3 * t]), i1 = __ldg(&s.idx[3 * t + 1]), i2 = __ldg(&s.idx[3 * t + 2]);
    const uint32_t vi[3] = {i1, i2, i0};
    F3 vp[3], vn[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) { vp[k] = ld3(__ldg(&s.vpos[vi[k]])); vn[k] = ld3(__ldg(&s.vnrm[vi[k]])); }
    const float2 uva = __ldg(&s.vuv[vi[0]]), uvb = __ldg(&s.vuv[vi[1]]), uvc = __ldg(&s.vuv[vi[2]]);
    const float uvx = (w[0] * uva.x + w[1] * uvb.x) + w[2] * uvc.x;
    const float uvy = (w[0] * uva.y + w[1] * uvb.y) + w[2] * uvc.y;
    // Triangle::init face normal from the caller's vertex order (v0, v1, v2) = (vp[2], vp[0], vp[1])
    F3 fnn = normalize(cross(vp[2] - vp[0], vp[1] - vp[2]));
    fnrm = F3{-fnn.x, -fnn.y, -fnn.z};
    F3 Nl = fnrm;
    if (smooth) Nl = normalize((w[0] * vn[0] + w[1] * vn[1]) + w[2] * vn[2]);
    nf = Nl;
    N = Nl;
    if (FRAME || s.nmap) {
        tangent_frame(Nl, tg, bt);
        N = mapped_normal(s, uvx, uvy, Nl, tg, bt);
    }
    float texv[NB];
    sample_uvs<NB>(s, nb, uvx, uvy, texv);
#pragma unroll
    for (int k = 0; k < NB; ++k) {
        if (k < (int)nb) {
            float va;
            if (s.albedo_uniform) {
                const float c = s.albedo_value[k];
                va = (w[0] * c + w[1] * c) + w[2] * c;
            } else {
                va = (w[0] * __ldg(&s.valb[(size_t)vi[0] * nb + k]) + w[1] * __ldg(&s.valb[(size_t)vi[1] * nb + k])) +
                     w[2] * __ldg(&s.valb[(size_t)vi[2] * nb + k]);
            }
            alb[k] = va * texv[k];
            if (va_out) va_out[k] = va;
            if (tex_out) tex_out[k] = texv[k];
        } else {
            alb[k] = 0.f;
        }
    }
    if (uv_out) { uv_out[0] = uvx; uv_out[1] = uvy; }
    Pp = (w[0] * vp[0] + w[1] * vp[1]) + w[2] * vp[2];
    F3 q[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) q[k] = Pp - dot(Pp - vp[k], vn[k]) * vn[k];
    F3 sp = (q[0] * w[0] + q[1] * w[1]) + q[2] * w[2];
    if (dot(sp - Pp, Nl) > 0) Pp = sp;
}

// Direct lighting from one light (cpu_path_tracer.ipp:399-428): samples the light and returns
// whether a shadow ray is needed, its direction and length, and the contribution per band if
// the shadow ray is unoccluded.
template <int NB>
__device__ __forceinline__ bool nee_light(const vgb_light& L, F3 Pp, F3 N, const float* alb, const float* thr,
                                          uint32_t nb, bool det, float ru1, float ru2, F3& Ld, float& dist,
                                          float* con) {
    float lpdf = 0.f;
    light_sample(L, Pp, det, ru1, ru2, Ld, dist, lpdf);
    if (!(lpdf > 0)) return false;
    const float nl = dot(N, Ld);
    const float cos_t = smax(0.0f, dot(Ld, N));
    const float mpdf = (nl <= 0.f) ? 0.f : nl * kInvPi;
    const float wgt = power_heuristic(lpdf, mpdf);
#pragma unroll
    for (int k = 0; k < NB; ++k) {
        const float bsdf = alb[k] * kInvPi * smax(nl, 0.f);
        con[k] = (k < (int)nb) ? thr[k] * bsdf * L.radiance[k] * cos_t * wgt / lpdf : 0.f;
    }
    return true;
}

// BSDF-sampled continuation (cpu_path_tracer.ipp:431-461) with optional Russian roulette.
// Returns whether the path continues; new_ray is false when the sampled pdf is 0 (the reference
// then keeps the incoming ray and throughput).
template <int NB>
__device__ __forceinline__ bool continue_path(const vgb_light* lights, uint32_t nlights, const vgb_pt_options& opt,
                                              uint32_t nb, F3 Pp, F3 N, F3 tg, F3 bt, F3 nf, const float* alb,
                                              float* thr, U4 r0, uint32_t slot, uint32_t sample, uint32_t frame,
                                              uint32_t bounce, F3& nd, bool& new_ray) {
    new_ray = false;
    F3 ls = cosine_sample(u01(r0.z), u01(r0.w));
    const float mpdf = ls.z * kInvPi;
    nd = F3{(tg.x * ls.x + bt.x * ls.y) + nf.x * ls.z, (tg.y * ls.x + bt.y * ls.y) + nf.y * ls.z,
            (tg.z * ls.x + bt.z * ls.y) + nf.z * ls.z};
    if (!(mpdf > 0)) return true;
    const float nl = dot(N, nd);
    const float cos_t = smax(0.0f, dot(nd, N));
    float lp = 0;
    for (uint32_t l = 0; l < nlights; ++l) lp += light_pdf(lights[l], Pp, nd);
    lp /= (float)nlights;
    const float wgt = power_heuristic(mpdf, lp);
#pragma unroll
    for (int k = 0; k < NB; ++k) {
        const float bsdf = alb[k] * kInvPi * smax(nl, 0.f);
        if (k < (int)nb) thr[k] *= bsdf * cos_t * wgt / mpdf;
    }
    new_ray = true;
    if (opt.rr_depth != 0 && bounce + 1 >= opt.rr_depth) {
        float q = 0.f;
#pragma unroll
        for (int k = 0; k < NB; ++k) if (k < (int)nb) q = smax(q, thr[k]);
        q = smin(q, 1.0f);
        const U4 rr = philox(U4{slot, sample, frame, (bounce << 8) | kSlotRR}, (uint32_t)opt.seed,
                             (uint32_t)(opt.seed >> 32));
        if (u01(rr.x) >= q) return false;
#pragma unroll
        for (int k = 0; k < NB; ++k) if (k < (int)nb) thr[k] = thr[k] / q;
    }
    return true;
}

// ------------------------------------------------------------------ camera rays
// Lens distortion models, FP32 in the reference's operation order:
// BrownDistortion::computeDelta (cameras/distortions/brown_distortion.ipp:24-44),
// OpenCVDistortion::distort (opencv_distortion.ipp:28-54), OwenDistortion::computeDelta
// (owen_distortion.ipp:24-46).  `h` is the normalised image point K^-1 (x, y, 1).
__device__ __forceinline__ void brown_delta(const float* k, float x, float y, float& dx, float& dy) {
    const float r = sqrtf(x * x + y * y);
    const float r2 = r * r, r4 = r2 * r2, r6 = r2 * r2 * r2;
    const float s = (k[0] * r2 + k[1] * r4) + k[2] * r6;
    dx = s * x + ((2.f * k[3] * x * y) + (k[4] * (r2 + 2.f * x * x)));
    dy = s * y + ((k[3] * (r2 + 2.f * y * y)) + (2.f * k[4] * x * y));
}
__device__ __forceinline__ void opencv_distort(const float* k, float x, float y, float& ox, float& oy) {
    const float r = sqrtf(x * x + y * y);
    const float r2 = r * r, r4 = r2 * r2, r6 = r2 * r2 * r2;
    const float num = 1.f + k[0] * r2 + k[1] * r4 + k[2] * r6;
    const float den = 1.f + k[3] * r2 + k[4] * r4 + k[5] * r6;
    const float f = num / den;
    const float tx = (2.f * k[6] * x * y) + (k[7] * (r2 + 2.f * x * x)) + (k[8] * r2) + (k[9] * r4);
    const float ty = (k[6] * (r2 + 2.f * y * y)) + (2.f * k[7] * x * y) + (k[10] * r2) + (k[11] * r4);
    ox = f * x + tx;
    oy = f * y + ty;
}
__device__ __forceinline__ void owen_delta(const float* e, float x, float y, float& dx, float& dy) {
    const float r = sqrtf(x * x + y * y);
    const float r2 = r * r, r3 = r * r * r;
    const float rf = (e[1] * r2) + (e[3] * r2 * r2) + (e[4] * y) + (e[5] * x);
    const float of = (e[0] * r) + (e[2] * r3);
    dx = rf * x + of * -y;
    dy = rf * y + of * x;
}
// Distortion::undistort: u = h - delta(u), 20 times from u = h.  OpenCV's delta is u - distort(u)
// (opencv_distortion.ipp:20-23), the opposite sign of the other models', so its iteration settles
// where u - h = distort(u) - u rather than inverting the model; kept as the reference has it.
__device__ __noinline__ float2 undistort(const vgb_camera& c, float hx, float hy) {
    float ux = hx, uy = hy;
    for (int it = 0; it < 20; ++it) {
        float dx, dy;
        if (c.distortion == VGB_DISTORTION_OPENCV) {
            float ox, oy;
            opencv_distort(c.distortion_coeffs, ux, uy, ox, oy);
            dx = ux - ox;
            dy = uy - oy;
        } else if (c.distortion == VGB_DISTORTION_BROWN) {
            brown_delta(c.distortion_coeffs, ux, uy, dx, dy);
        } else {
            owen_delta(c.distortion_coeffs, ux, uy, dx, dy);
        }
        ux = hx - dx;
        uy = hy - dy;
    }
    return make_float2(ux, uy);
}
// Distortion::distort (the rasterizer's projection): h + delta(h), OpenCV's formula directly.
__device__ __forceinline__ void distort(const vgb_camera& c, float& hx, float& hy) {
    float dx, dy;
    if (c.distortion == VGB_DISTORTION_OPENCV) {
        opencv_distort(c.distortion_coeffs, hx, hy, dx, dy);
        hx = dx;
        hy = dy;
        return;
    }
    if (c.distortion == VGB_DISTORTION_BROWN) brown_delta(c.distortion_coeffs, hx, hy, dx, dy);
    else owen_delta(c.distortion_coeffs, hx, hy, dx, dy);
    hx = hx + dx;
    hy = hy + dy;
}

// Camera::pixelToDirectionHelper (camera.ipp:1738-1749): K^-1 (x, y, 1), undistorted, in the
// camera frame.
__device__ __forceinline__ F3 direction_helper(const vgb_camera& cam, float X, float Y) {
    const float* K = cam.kinv;
    float hx = (K[0] * X + K[2] * Y) + K[4] * 1.0f;
    float hy = (K[1] * X + K[3] * Y) + K[5] * 1.0f;
    if (cam.distortion) {
        const float2 u = undistort(cam, hx, hy);
        hx = u.x;
        hy = u.y;
    }
    return F3{hx, cam.z_dir * hy, cam.z_dir};
}

// Camera::pixelToDirection (camera.ipp:1105-1117): with a distortion and direction interpolation,
// Image::interpolatePixel (image.ipp:619-671) of the table precomputePixelDirections fills with
// normalize(pixelToDirectionHelper(i, j)) -- evaluated here at the four corners on the fly.
__device__ __noinline__ F3 interpolated_direction(const vgb_camera& cam, float X, float Y) {
    int x0 = (int)floorf(X), y0 = (int)floorf(Y);
    x0 = min(x0, (int)cam.width - 1);
    y0 = min(y0, (int)cam.height - 1);
    const int x1 = min(x0 + 1, (int)cam.width - 1), y1 = min(y0 + 1, (int)cam.height - 1);
    const F3 p00 = normalize(direction_helper(cam, (float)x0, (float)y0));
    const F3 p10 = normalize(direction_helper(cam, (float)x1, (float)y0));
    const F3 p01 = normalize(direction_helper(cam, (float)x0, (float)y1));
    const F3 p11 = normalize(direction_helper(cam, (float)x1, (float)y1));
    const float dx = X - (float)x0, dy = Y - (float)y0;
    return (((1.f - dx) * (1.f - dy) * p00 + dx * (1.f - dy) * p10) + (1.f - dx) * dy * p01) + dx * dy * p11;
}

__device__ __forceinline__ F3 camera_direction(const vgb_camera& cam, float X, float Y) {
    if (cam.distortion && cam.interpolate_directions) return interpolated_direction(cam, X, Y);
    return direction_helper(cam, X, Y);
}

// Camera::pixelToRay for pixel (pi, pj) = slot: sample 0 through the pixel corner with the
// pinhole overload, later samples jittered and, with depth of field, through a point of the
// aperture (camera.ipp:1126-1163, cpu_path_tracer.ipp:182-192).  Random numbers: the jitter
// draw's first two words move the pixel coordinate, its last two sample the aperture disc
// (UniformDiskSample, sampling.ipp:43-52).
__device__ __forceinline__ void pixel_ray(const vgb_camera& cam, uint32_t pi, uint32_t pj, uint32_t slot,
                                          uint32_t sample, uint32_t frame, uint32_t k0, uint32_t k1, F3& ro, F3& rd) {
    float X = (float)pi, Y = (float)pj;
    U4 jr{0, 0, 0, 0};
    if (sample != 0) {
        jr = philox(U4{slot, sample, frame, kSlotJitter}, k0, k1);
        X = X + u01(jr.x);
        Y = Y + u01(jr.y);
    }
    F3 dc = camera_direction(cam, X, Y);
    const float* R = cam.rotation;
    ro = F3{cam.origin[0], cam.origin[1], cam.origin[2]};
    if (sample != 0 && cam.depth_of_field) {
        const float r = sqrtf(u01(jr.z));
        const float theta = 2.f * kPi * u01(jr.w);
        const F3 off{cam.aperture_radius * (r * cosf(theta)), cam.aperture_radius * (r * sinf(theta)), cam.focal_length};
        ro = ro + F3{(R[0] * off.x + R[3] * off.y) + R[6] * off.z, (R[1] * off.x + R[4] * off.y) + R[7] * off.z,
                     (R[2] * off.x + R[5] * off.y) + R[8] * off.z};
        if (!isinf(cam.focus_distance)) dc = cam.focus_distance * normalize(dc) - off;
    }
    F3 dw{(R[0] * dc.x + R[3] * dc.y) + R[6] * dc.z, (R[1] * dc.x + R[4] * dc.y) + R[7] * dc.z,
          (R[2] * dc.x + R[5] * dc.y) + R[8] * dc.z};
    rd = normalize(dw);
}

__device__ __forceinline__ bool camera_ray(const FrameParams& fp, uint32_t item, uint32_t sample, uint32_t& slot,
                                           F3& ro, F3& rd) {
    const uint32_t tile = item >> 5, ln = item & 31u;
    const uint32_t tx = tile % fp.tiles_x, ty = tile / fp.tiles_x;
    const uint32_t pi = tx * 8u + (ln & 7u), pj = ty * 4u + (ln >> 3);
    if (pi >= fp.cam.width || pj >= fp.cam.height) return false;
    slot = pj * fp.cam.width + pi;
    pixel_ray(fp.cam, pi, pj, slot, sample, fp.opt.frame, (uint32_t)fp.opt.seed, (uint32_t)(fp.opt.seed >> 32), ro, rd);
    return true;
}

// ------------------------------------------------------------------ first-hit passes
// renderPasses.save_triangle_size / save_velocity at a pixel's first hit (cpu_path_tracer.ipp:
// 356-372).  Pp: the shading point before offsetIntersection; vert = {v1, v2, v0}; the triangle
// size is the longest edge over Camera::calculateGSD (camera.ipp:1408-1414) at the hit distance;
// the velocity is the instance's point velocity at Pp (reference_frame.ipp:367-373) and, in the
// camera frame, relative to the camera's point velocity evaluated at rotation * p_global.
__device__ __noinline__ void first_hit_passes(const DevScene& s, const vgb_camera& cam, uint32_t t, F3 Pp,
                                              float* vel_g, float* vel_c, float* tsz, size_t FP, uint32_t slot) {
    if (tsz) {
        const F3 a = ld3(__ldg(&s.vpos[__ldg(&s.idx[3 * (size_t)t + 1])]));
        const F3 b = ld3(__ldg(&s.vpos[__ldg(&s.idx[3 * (size_t)t + 2])]));
        const F3 c = ld3(__ldg(&s.vpos[__ldg(&s.idx[3 * (size_t)t])]));
        const float e01 = length(b - a), e02 = length(c - a), e12 = length(c - b);
        const float edge = smax(e01, smax(e02, e12));
        const float distance = length(Pp - F3{cam.origin[0], cam.origin[1], cam.origin[2]});
        const float gx = distance * cam.sensor_size[0] / (cam.focal_length * (float)cam.width);
        const float gy = distance * cam.sensor_size[1] / (cam.focal_length * (float)cam.height);
        tsz[slot] = edge / smin(gx, gy);
    }
    if (vel_g || vel_c) {
        F3 v{0.f, 0.f, 0.f}, w{0.f, 0.f, 0.f}, o{0.f, 0.f, 0.f};
        if (s.nmotion) {
            uint32_t lo = 0, hi = s.nmotion - 1;   // the last instance whose first triangle is <= t
            while (lo < hi) {
                const uint32_t mid = (lo + hi + 1) >> 1;
                if (s.motion[mid].first_triangle <= t) lo = mid; else hi = mid - 1;
            }
            const vgb_instance_motion& m = s.motion[lo];
            v = F3{m.velocity[0], m.velocity[1], m.velocity[2]};
            w = F3{m.angular_rate[0], m.angular_rate[1], m.angular_rate[2]};
            o = F3{m.position[0], m.position[1], m.position[2]};
        }
        const F3 vg = v + cross(w, Pp - o);
        if (vel_g) { vel_g[slot] = vg.x; vel_g[FP + slot] = vg.y; vel_g[2 * FP + slot] = vg.z; }
        if (vel_c) {
            const float* R = cam.rotation;
            const F3 rp{((R[0] * Pp.x + R[3] * Pp.y) + R[6] * Pp.z) + cam.rot_origin[0],
                        ((R[1] * Pp.x + R[4] * Pp.y) + R[7] * Pp.z) + cam.rot_origin[1],
                        ((R[2] * Pp.x + R[5] * Pp.y) + R[8] * Pp.z) + cam.rot_origin[2]};
            const F3 cv = F3{cam.velocity[0], cam.velocity[1], cam.velocity[2]} +
                          cross(F3{cam.angular_rate[0], cam.angular_rate[1], cam.angular_rate[2]}, rp);
            const F3 rv = vg - cv;
            // globalDirectionToLocal: the inverse (transpose) of the camera rotation
            vel_c[slot] = (R[0] * rv.x + R[1] * rv.y) + R[2] * rv.z;
            vel_c[FP + slot] = (R[3] * rv.x + R[4] * rv.y) + R[5] * rv.z;
            vel_c[2 * FP + slot] = (R[6] * rv.x + R[7] * rv.y) + R[8] * rv.z;
        }
    }
}

// ------------------------------------------------------------------ k_trace (closest hit)
// Scene::intersect for every live path: camera rays at bounce 0, queued continuation rays
// after.  Writes one 16-byte hit record per queue item; kept lean so that enough warps are
// resident to hide the latency of the node and triangle fetches.
// B0: the launch traces bounce 0 (camera rays generated in place); later bounces read the queue.
template <int L, bool COUNT, bool B0>
__global__ void __launch_bounds__(VGB_TRACE_BLOCK, (L == 8 ? VGB_TRACE8_MINB : VGB_TRACE_MINB) * 256 / VGB_TRACE_BLOCK) k_trace(const DevScene s, DevState st, const __grid_constant__ FrameParams fp,
                                               uint32_t bounce, uint32_t sample, uint32_t in_q, uint32_t n_items_bounce0) {
    const size_t P = st.P;
    const uint32_t n_items = (B0) ? n_items_bounce0 : st.counters[in_q];
    const uint32_t* in_queue = st.pq[in_q];
    uint32_t err = 0, nclosest = 0;
    Counters cnt{0, 0};
    for (uint32_t item = blockIdx.x * blockDim.x + threadIdx.x; item < n_items; item += gridDim.x * blockDim.x) {
        uint32_t slot = 0;
        F3 ro, rd;
        if (B0) {
            if (!camera_ray(fp, item, sample, slot, ro, rd)) continue;
            if (fp.opt.adaptive_sampling && sample != 0 && st.anum[slot]) continue;  // pixel has stopped
        }
        uint32_t qi = item;  // the queue position this ray's hit record goes to
        if (!B0) {
#if VGB_TRACE_BINS > 0
            if (st.binq) {
                uint32_t first = 0;
#pragma unroll
                for (int b = 0; b < VGB_TRACE_BINS; ++b) {
                    const uint32_t c = st.counters[C_BIN + b];
                    if (item >= first && item - first < c) qi = st.binq[b * P + (item - first)];
                    first += c;
                }
            }
#endif
            slot = in_queue[qi];
            ro = F3{st.org[slot], st.org[P + slot], st.org[2 * P + slot]};
            rd = F3{st.dir[slot], st.dir[P + slot], st.dir[2 * P + slot]};
        }
        HitOut h;
        h.U = h.V = h.W = 0.f; h.det = 1.f;
        const WRay wr = make_wray(ro, rd);
        traverse_any_layout<L, false, COUNT>(s.nodes, s.tris, wr, 0.f, h, err, cnt, s.iter_cap);
        nclosest++;
        float w0 = 0.f, w1 = 0.f;
        if (h.id != VGB_NO_HIT) {
            const float rcp = 1.0f / h.det;
            w0 = h.V * rcp;
            w1 = h.W * rcp;
        }
        st.hit[qi] = make_float4(h.t, __uint_as_float(h.id), w0, w1);
    }
    if (err) atomicOr(&st.counters[C_ERR], err);
    warp_reduce_add(&st.stats[2], nclosest);
    if (COUNT) {
        warp_reduce_add(&st.stats[0], cnt.nodes);
        warp_reduce_add(&st.stats[1], cnt.tris);
        warp_reduce_add(&st.stats[4], cnt.nodes);
        warp_reduce_add(&st.stats[5], cnt.tris);
    }
}

#if VGB_TRACE_BINS > 0
// The live-path queue `in_q` binned by the vertical component of each ray's direction (bins of
// equal width over [-1, 1]), so that a warp of k_trace takes rays of similar traversal length:
// on terrain the near-horizontal rays cross far more of the tree than the steep ones.  Each bin
// lists queue positions; the appends are warp-aggregated per bin.  Sum of the bins = the queue.
__global__ void __launch_bounds__(256) k_bin_rays(DevState st, uint32_t in_q) {
    const size_t P = st.P;
    const uint32_t n = st.counters[in_q];
    const uint32_t* in_queue = st.pq[in_q];
    const int lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n; base += stride) {
        const uint32_t item = base + lane;
        const bool valid = item < n;
        const unsigned vmask = __ballot_sync(0xffffffffu, valid);
        if (!valid) continue;
        const float dz = st.dir[2 * P + in_queue[item]];
        const float x = fminf(fmaxf((dz + 1.0f) * (0.5f * VGB_TRACE_BINS), 0.0f), (float)(VGB_TRACE_BINS - 1));
        const uint32_t b = (uint32_t)x;
        const unsigned grp = __match_any_sync(vmask, b);
        const int leader = __ffs(grp) - 1;
        uint32_t pos = 0;
        if (lane == leader) pos = atomicAdd(&st.counters[C_BIN + b], (uint32_t)__popc(grp));
        pos = __shfl_sync(grp, pos, leader) + (uint32_t)__popc(grp & ((1u << lane) - 1u));
        st.binq[b * P + pos] = item;
    }
}
#endif

// ------------------------------------------------------------------ persistent traversal (binary layout)
// k_trace_p / k_shadow_p replace the grid-stride loops of k_trace / k_shadow for the binary BVH.
// They launch one wave of resident blocks; each warp claims chunks of kWarpChunk consecutive queue
// items from a launch-wide counter and hands them to its lanes as lanes become free, and every
// lane advances its ray by at most `budget` inner-node visits between hand-outs (traverse_resume).
// A lane whose ray finished thus starts the next ray while its neighbours are still traversing,
// instead of idling until the warp's slowest ray is done, which is what left bounce-1 rays at
// half-empty warps.  Rays, their order within a warp and every test are those of the grid-stride
// kernels, so the hit records are identical.
constexpr uint32_t kWarpChunk = 64;
constexpr unsigned kFullMask = 0xffffffffu;

// The items a warp holds and has not handed out: [base, base + left), all below the launch's item
// count; `done` once the launch-wide counter has passed it.  Warp-uniform.
struct WarpItems {
    uint32_t base, left;
    bool done;
};

// Hands one item to every lane set in `idle` (the lanes' rank in `idle` orders them); returns this
// lane's item, or n when there is none.  Claims a new chunk when the held items do not suffice.
__device__ __forceinline__ uint32_t warp_take(WarpItems& wi, uint32_t* counter, uint32_t n, unsigned idle, int lane) {
    const uint32_t k = __popc(idle);
    const uint32_t r = __popc(idle & ((1u << lane) - 1u));
    const bool mine = (idle >> lane) & 1u;
    uint32_t item = n;
    if (wi.left < k && !wi.done) {
        uint32_t nb = 0;
        if (lane == 0) nb = atomicAdd(counter, kWarpChunk);
        nb = __shfl_sync(kFullMask, nb, 0);
        const uint32_t fresh = nb < n ? min(kWarpChunk, n - nb) : 0u;
        if (nb + kWarpChunk >= n) wi.done = true;
        if (mine) {
            if (r < wi.left) item = wi.base + r;
            else if (r - wi.left < fresh) item = nb + (r - wi.left);
        }
        const uint32_t used = min(k - wi.left, fresh);
        wi.base = nb + used;
        wi.left = fresh - used;
    } else {
        const uint32_t take = min(k, wi.left);
        if (mine && r < take) item = wi.base + r;
        wi.base += take;
        wi.left -= take;
    }
    return item;
}

template <bool COUNT>
__global__ void __launch_bounds__(256, VGB_TRACEP_MINB) k_trace_p(const DevScene s, DevState st, const __grid_constant__ FrameParams fp,
                                                 uint32_t bounce, uint32_t sample, uint32_t in_q,
                                                 uint32_t n_items_bounce0, int budget, uint32_t refill) {
    const size_t P = st.P;
    const uint32_t n_items = (bounce == 0) ? n_items_bounce0 : st.counters[in_q];
    const uint32_t* in_queue = st.pq[in_q];
    const float4* nodes = reinterpret_cast<const float4*>(s.nodes);
    const int lane = threadIdx.x & 31;
    uint32_t err = 0, nclosest = 0;
    Counters cnt{0, 0};
    WarpItems wi{0, 0, false};
    bool live = false;
    uint32_t item = 0;
    WRay wr;
    SlabRay q;
    TravState ts;
    HitOut h;
    int stack[kStackSize];
    while (true) {
        const unsigned idle = __ballot_sync(kFullMask, !live);
        if ((wi.left || !wi.done) && (__popc(idle) >= refill || idle == kFullMask)) {
            const uint32_t it = warp_take(wi, &st.counters[C_FTRACE], n_items, idle, lane);
            if (it < n_items) {
                uint32_t slot = 0;
                F3 ro, rd;
                bool ok = true;
                if (bounce == 0) {
                    ok = camera_ray(fp, it, sample, slot, ro, rd);
                    if (ok && fp.opt.adaptive_sampling && sample != 0 && st.anum[slot]) ok = false;  // stopped
                } else {
                    slot = in_queue[it];
                    ro = F3{st.org[slot], st.org[P + slot], st.org[2 * P + slot]};
                    rd = F3{st.dir[slot], st.dir[P + slot], st.dir[2 * P + slot]};
                }
                if (ok) {
                    item = it;
                    wr = make_wray(ro, rd);
                    q = make_slab(wr);
                    ts = trav_start(0.f, false, h);
                    live = true;
                    nclosest++;
                }
            }
        }
        if (__ballot_sync(kFullMask, live) == 0) {
            if (wi.done && wi.left == 0) break;
            continue;
        }
        if (live && traverse_resume<COUNT>(nodes, s.tris, wr, q, 0.f, false, stack, ts, h, err, cnt, s.iter_cap, budget)) {
            float w0 = 0.f, w1 = 0.f;
            if (h.id != VGB_NO_HIT) {
                const float rcp = 1.0f / h.det;
                w0 = h.V * rcp;
                w1 = h.W * rcp;
            }
            st.hit[item] = make_float4(h.t, __uint_as_float(h.id), w0, w1);
            live = false;
        }
    }
    if (err) atomicOr(&st.counters[C_ERR], err);
    warp_reduce_add(&st.stats[2], nclosest);
    if (COUNT) {
        warp_reduce_add(&st.stats[0], cnt.nodes);
        warp_reduce_add(&st.stats[1], cnt.tris);
        warp_reduce_add(&st.stats[4], cnt.nodes);
        warp_reduce_add(&st.stats[5], cnt.tris);
    }
}

template <int NB, bool COUNT>
__global__ void __launch_bounds__(256, VGB_SHADOWP_MINB) k_shadow_p(const DevScene s, DevState st, uint32_t light, uint32_t nb,
                                                   int budget, uint32_t refill) {
    const size_t P = st.P;
    const uint32_t n = st.counters[C_SQ + light];
    const float4* nodes = reinterpret_cast<const float4*>(s.nodes);
    const int lane = threadIdx.x & 31;
    uint32_t err = 0, nsh = 0;
    Counters cnt{0, 0};
    WarpItems wi{0, 0, false};
    bool live = false;
    uint32_t item = 0;
    float tmax = 0.f;
    WRay wr;
    SlabRay q;
    TravState ts;
    HitOut h;
    int stack[kStackSize];
    while (true) {
        const unsigned idle = __ballot_sync(kFullMask, !live);
        if ((wi.left || !wi.done) && (__popc(idle) >= refill || idle == kFullMask)) {
            const uint32_t it = warp_take(wi, &st.counters[C_FSHADOW + light], n, idle, lane);
            if (it < n) {
                item = it;
                const F3 o{st.sq_org[light][it], st.sq_org[light][P + it], st.sq_org[light][2 * P + it]};
                const F3 d{st.sq_dir[light][it], st.sq_dir[light][P + it], st.sq_dir[light][2 * P + it]};
                tmax = st.sq_tmax[light][it];
                wr = make_wray(o, d);
                q = make_slab(wr);
                ts = trav_start(tmax, true, h);
                live = true;
                nsh++;
            }
        }
        if (__ballot_sync(kFullMask, live) == 0) {
            if (wi.done && wi.left == 0) break;
            continue;
        }
        if (live && traverse_resume<COUNT>(nodes, s.tris, wr, q, tmax, true, stack, ts, h, err, cnt, s.iter_cap, budget)) {
            if (h.id == VGB_NO_HIT) {
                const uint32_t slot = st.sq_slot[light][item];
#pragma unroll
                for (int k = 0; k < NB; ++k)
                    if (k < (int)nb) st.brad[k * P + slot] += st.sq_con[light][k * P + item];
            }
            live = false;
        }
    }
    if (err) atomicOr(&st.counters[C_ERR], err);
    warp_reduce_add(&st.stats[3], nsh);
    if (COUNT) {
        warp_reduce_add(&st.stats[0], cnt.nodes);
        warp_reduce_add(&st.stats[1], cnt.tris);
    }
}

// ------------------------------------------------------------------ k_shade
// processIntersection for every item of k_trace: AOVs, shading point, NEE shadow-ray enqueue,
// BSDF-sampled continuation and live-path enqueue (warp-aggregated appends).
// The bilinear weights of the background lookup of a missed ray (cpu_path_tracer.ipp:256-270),
// out of line: a cold path of the shading kernels, kept out of their instruction footprint.
__device__ __noinline__ float4 background_weights(F3 rd) {
    float x = rd.x, y = rd.y, z = rd.z;
    float u = atan2f(y, x) / (2 * kPi);
    float v = atan2f(sqrtf(x * x + y * y), z) / kPi;
    float px = fmodf(u * 1.f, 1.f), py = fmodf(v * 1.f, 1.f);
    if (px < 0) px += 1.f;
    if (py < 0) py += 1.f;
    float ddx = px - 0.f, ddy = py - 0.f;
    return make_float4((1.f - ddx) * (1.f - ddy), ddx * (1.f - ddy), (1.f - ddx) * ddy, ddx * ddy);
}

// B0: the launch shades bounce 0 (camera hits); the bounce-0-only and later-bounce-only code
// paths are compiled into separate instantiations.
template <int NB, bool B0>
__global__ void __launch_bounds__(VGB_SHADE_BLOCK, VGB_SHADE_MINB * 256 / VGB_SHADE_BLOCK) k_shade(const DevScene s, DevState st, const __grid_constant__ FrameParams fp, uint32_t bounce,
                                               uint32_t sample, uint32_t in_q, uint32_t n_items_bounce0) {
    const uint32_t nb = fp.nb;
    const size_t P = st.P;
    const int lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t n_items = (B0) ? n_items_bounce0 : st.counters[in_q];
    uint32_t* out_count = &st.counters[(in_q ^ 1u)];
    uint32_t* out_q = st.pq[in_q ^ 1u];
    const uint32_t* in_queue = st.pq[in_q];
    uint32_t nhits = 0;
    for (uint32_t base = blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < n_items; base += stride) {
        const uint32_t item = base + lane;
        bool active = item < n_items;
        uint32_t slot = 0;
        F3 ro{0, 0, 0}, rd{0, 0, 1};
        float thr[NB];
#pragma unroll
        for (int k = 0; k < NB; ++k) thr[k] = 1.f;
        const uint32_t aux = fp.aux;
        uint32_t pendv = 0u;  // this item's fold state, written once below
        if (active) {
            if (B0) {
                active = camera_ray(fp, item, sample, slot, ro, rd);
                if (active && fp.opt.adaptive_sampling) {
                    if (sample == 0) { st.as1[slot] = 0.f; st.as2[slot] = 0.f; st.anum[slot] = 0u; }
                    else if (st.anum[slot]) active = false;  // the pixel has stopped sampling
                }
                if (active) {
                    if (sample == 0) {
#pragma unroll
                        for (int k = 0; k < NB; ++k) {
                            if (k < (int)nb) {
                                st.arad[k * P + slot] = 0.f;
                                if (aux & AUX_DIR) st.adir[k * P + slot] = 0.f;
                                if (aux & AUX_ALB) st.aalb[k * P + slot] = 0.f;
                            }
                        }
                        if (aux & AUX_NRM) { st.anrm[slot] = 0.f; st.anrm[P + slot] = 0.f; st.anrm[2 * P + slot] = 0.f; }
                        if (aux & AUX_DEP) { st.adep[slot] = 0.f; st.acnt[slot] = 0u; }
                        if (aux & AUX_TRI) st.atri[slot] = VGB_NO_HIT;
                        const size_t FP = (size_t)fp.cam.width * fp.cam.height;
                        if (fp.tsz) fp.tsz[slot] = __int_as_float(0x7f800000);
                        if (fp.vel_g) { fp.vel_g[slot] = 0.f; fp.vel_g[FP + slot] = 0.f; fp.vel_g[2 * FP + slot] = 0.f; }
                        if (fp.vel_c) { fp.vel_c[slot] = 0.f; fp.vel_c[FP + slot] = 0.f; fp.vel_c[2 * FP + slot] = 0.f; }
                    }
                    pendv = kPradEmpty;  // the path radiance starts at 0 without being written
                }
            } else {
                slot = in_queue[item];
                // the incoming ray stays in the path state; it is read below only for a miss.
                // Fold the previous bounce's radiance into the path now, so that the path
                // radiance is not live through the shading.
                const uint32_t pend = st.pend[slot];
                if (pend & kPendMask) {
#pragma unroll
                    for (int k = 0; k < NB; ++k) {
                        if (k < (int)nb) {
                            const float br = st.brad[k * P + slot];
                            const float pr = (pend & kPradEmpty) ? 0.f : st.prad[k * P + slot];
                            st.prad[k * P + slot] = pr + br;
                            if ((pend & kPendMask) == 1u && (aux & AUX_DIR)) st.adir[k * P + slot] += br;
                        }
                    }
                    pendv = 0u;
                } else {
                    pendv = pend & kPradEmpty;
                }
            }
        }
        // ---- closest hit, from k_trace
        float4 hr = make_float4(__int_as_float(0x7f800000), __uint_as_float(VGB_NO_HIT), 0.f, 0.f);
        if (active) hr = st.hit[item];
        const uint32_t hid = __float_as_uint(hr.y);
        bool hit = active && hid != VGB_NO_HIT;
        nhits += hit ? 1u : 0u;
        bool cont = false;
        bool lit = false;  // hit and simulate_lighting: NEE runs for this lane
        F3 Pp{0, 0, 0}, N{0, 0, 1};
        float alb[NB];
#pragma unroll
        for (int k = 0; k < NB; ++k) alb[k] = 0.f;
        U4 r0{0, 0, 0, 0};
        const uint32_t k0 = (uint32_t)fp.opt.seed, k1 = (uint32_t)(fp.opt.seed >> 32);
        if (active && !hit) {
            if (fp.opt.simulate_lighting && fp.opt.show_background) {
                if (!B0) rd = F3{st.dir[slot], st.dir[P + slot], st.dir[2 * P + slot]};
                const float4 bw = background_weights(rd);
                const float a = bw.x, b = bw.y, c = bw.z, e = bw.w;
#pragma unroll
                for (int k = 0; k < NB; ++k) {
                    if (k < (int)nb) {
                        const float bgv = fp.opt.background[k];
                        float bg = ((a * bgv + b * bgv) + c * bgv) + e * bgv;
                        const float tk = (B0) ? 1.f : st.thr[k * P + slot];
                        const float pr = (pendv & kPradEmpty) ? 0.f : st.prad[k * P + slot];
                        st.prad[k * P + slot] = pr + tk * (bg * 1.f);
                    }
                }
                pendv = 0u;
            }
        }
        F3 tg{1, 0, 0}, bt{0, 1, 0}, nf{0, 0, 1};
        if (hit) {
            // ---- processIntersection (cpu_path_tracer.ipp:280-469)
            const uint32_t t = hid;
            F3 fnrm;
            surface_at<NB>(s, nb, fp.opt.smooth_shading != 0, t, hr.z, hr.w, Pp, N, fnrm, tg, bt, nf, alb);
            if (B0) {
                if ((aux & AUX_TRI) && st.atri[slot] == VGB_NO_HIT) {
                    st.atri[slot] = t;
                    if (fp.tsz || fp.vel_g || fp.vel_c)
                        first_hit_passes(s, fp.cam, t, Pp, fp.vel_g, fp.vel_c, fp.tsz,
                                         (size_t)fp.cam.width * fp.cam.height, slot);
                }
                if (aux & AUX_ALB) {
#pragma unroll
                    for (int k = 0; k < NB; ++k)
                        if (k < (int)nb) st.aalb[k * P + slot] += alb[k];
                }
                if (aux & AUX_NRM) { st.anrm[slot] += N.x; st.anrm[P + slot] += N.y; st.anrm[2 * P + slot] += N.z; }
                if (aux & AUX_DEP) { st.adep[slot] += hr.x; st.acnt[slot] += 1u; }
            }
            if (fp.opt.simulate_lighting) {
                lit = true;
                if (!B0) {
#pragma unroll
                    for (int k = 0; k < NB; ++k)
                        if (k < (int)nb) thr[k] = st.thr[k * P + slot];
                }
                Pp = F3{offset1(Pp.x, fnrm.x), offset1(Pp.y, fnrm.y), offset1(Pp.z, fnrm.z)};
#pragma unroll
                for (int k = 0; k < NB; ++k) {
                    if (k < (int)nb)
                        st.brad[k * P + slot] = (B0 && fp.opt.has_ambient) ? 0.f + thr[k] * (fp.opt.ambient[k] * alb[k]) : 0.f;
                }
                pendv = (pendv & kPradEmpty) | ((B0) ? 1u : 2u);
                r0 = philox(U4{slot, sample, fp.opt.frame, (bounce << 8) | kSlotMain}, k0, k1);
            }
        }
        // ---- NEE: one shadow ray per light, appended to that light's queue (warp ballot)
        for (uint32_t l = 0; l < fp.nlights; ++l) {
            bool pred = false;
            F3 Ld{0, 0, 1};
            float dist = 0.f;
            float con[NB];
            if (lit) {
                float ru1, ru2;
                if (l == 0) { ru1 = u01(r0.x); ru2 = u01(r0.y); }
                else {
                    U4 rl = philox(U4{slot, sample, fp.opt.frame, (bounce << 8) | (1u + l)}, k0, k1);
                    ru1 = u01(rl.x); ru2 = u01(rl.y);
                }
                pred = nee_light<NB>(fp.lights[l], Pp, N, alb, thr, nb, fp.opt.deterministic_light != 0, ru1, ru2, Ld,
                                     dist, con);
            }
            const uint32_t qi = warp_append(&st.counters[C_SQ + l], pred);
            if (pred) {
                st.sq_org[l][qi] = Pp.x; st.sq_org[l][P + qi] = Pp.y; st.sq_org[l][2 * P + qi] = Pp.z;
                st.sq_dir[l][qi] = Ld.x; st.sq_dir[l][P + qi] = Ld.y; st.sq_dir[l][2 * P + qi] = Ld.z;
                st.sq_tmax[l][qi] = dist;
                st.sq_slot[l][qi] = slot;
#pragma unroll
                for (int k = 0; k < NB; ++k)
                    if (k < (int)nb) st.sq_con[l][k * P + qi] = con[k];
            }
        }
        // ---- BSDF-sampled continuation
        bool new_ray = false;
        if (lit && bounce < fp.opt.bounces) {
            F3 nd;
            cont = continue_path<NB>(fp.lights, fp.nlights, fp.opt, nb, Pp, N, tg, bt, nf, alb, thr, r0, slot, sample,
                                     fp.opt.frame, bounce, nd, new_ray);
            if (new_ray) { ro = Pp; rd = nd; }
            // pdf 0: the reference keeps the incoming ray and throughput
        }
        // ---- write path state and append live paths
        if (active) {
            st.pend[slot] = pendv;
            if (cont) {
#pragma unroll
                for (int k = 0; k < NB; ++k)
                    if (k < (int)nb) st.thr[k * P + slot] = thr[k];
            }
            // a path that keeps its incoming ray (sampled pdf 0) already has it in the state,
            // except a camera ray
            if (cont && (new_ray || B0)) {
                st.org[slot] = ro.x; st.org[P + slot] = ro.y; st.org[2 * P + slot] = ro.z;
                st.dir[slot] = rd.x; st.dir[P + slot] = rd.y; st.dir[2 * P + slot] = rd.z;
            }
        }
        const uint32_t pqi = warp_append(out_count, cont);
        if (cont) out_q[pqi] = slot;
    }
    warp_reduce_add(&st.stats[6], nhits);
}

// ------------------------------------------------------------------ k_shadow
template <int NB, int L, bool COUNT>
__global__ void __launch_bounds__(VGB_SHADOW_BLOCK, (L == 8 ? VGB_SHADOW8_MINB : VGB_SHADOW_MINB) * 256 / VGB_SHADOW_BLOCK) k_shadow(const DevScene s, DevState st, uint32_t light, uint32_t nb) {
    const size_t P = st.P;
    const uint32_t n = st.counters[C_SQ + light];
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t err = 0, nsh = 0;
    Counters cnt{0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        F3 o{st.sq_org[light][i], st.sq_org[light][P + i], st.sq_org[light][2 * P + i]};
        F3 d{st.sq_dir[light][i], st.sq_dir[light][P + i], st.sq_dir[light][2 * P + i]};
        const float tmax = st.sq_tmax[light][i];
        WRay wr = make_wray(o, d);
        HitOut h;
        traverse_any_layout<L, true, COUNT>(s.nodes, s.tris, wr, tmax, h, err, cnt, s.iter_cap);
        nsh++;
        if (h.id == VGB_NO_HIT) {
            const uint32_t slot = st.sq_slot[light][i];
#pragma unroll
            for (int k = 0; k < NB; ++k)
                if (k < (int)nb) st.brad[k * P + slot] += st.sq_con[light][k * P + i];
        }
    }
    if (err) atomicOr(&st.counters[C_ERR], err);
    warp_reduce_add(&st.stats[3], nsh);
    if (COUNT) {
        warp_reduce_add(&st.stats[0], cnt.nodes);
        warp_reduce_add(&st.stats[1], cnt.tris);
    }
}

// ------------------------------------------------------------------ k_end_sample
template <int NB, bool ADAPTIVE>
__global__ void __launch_bounds__(256) k_end_sample(DevState st, const __grid_constant__ FrameParams fp, uint32_t smp,
                                                    uint32_t last, FilmOut f) {
    const size_t P = st.P;                       // plane stride of the scratch state
    const uint32_t nb = fp.nb;
    const uint32_t npix = fp.cam.width * fp.cam.height;
    const size_t FP = npix;                      // plane stride of the caller's film
    const float sf_all = (float)fp.opt.samples;
    const bool adaptive = ADAPTIVE;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < npix; p += gridDim.x * blockDim.x) {
        const bool want_dir = (fp.aux & AUX_DIR) != 0;
        uint32_t stopped = adaptive ? st.anum[p] : 0u;
        float tot[NB];
        if (!stopped) {
            const uint32_t pend = st.pend[p];
            float prs[NB];
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                prs[k] = 0.f;
                if (k < (int)nb) {
                    float pr = (pend & kPradEmpty) ? 0.f : st.prad[k * P + p];
                    if (pend & kPendMask) {
                        const float br = st.brad[k * P + p];
                        pr += br;
                        if ((pend & kPendMask) == 1u && want_dir) st.adir[k * P + p] += br;
                    }
                    prs[k] = pr;
                    tot[k] = st.arad[k * P + p] + pr;
                    st.arad[k * P + p] = tot[k];
                }
            }
            // (the fold state is rewritten for every pixel by the next sample's camera rays)
            if (adaptive) {
                // unidirectional's stopping rule (cpu_path_tracer.ipp:198-226)
                float sq = 0.f;
#pragma unroll
                for (int k = 0; k < NB; ++k) if (k < (int)nb) sq += prs[k] * prs[k];
                const float illum = sqrtf(sq);
                const float s1 = st.as1[p] + illum, s2 = st.as2[p] + illum * illum;
                st.as1[p] = s1;
                st.as2[p] = s2;
                bool stop = false;
                if (smp != 0 && smp % fp.opt.samples_to_detect_miss == 0 && st.adep[p] == 0.f) {
                    stop = true;
                } else if (smp != 0 && smp % fp.opt.samples_per_batch == 0) {
                    if (s1 == 0.f) {
                        stop = true;
                    } else {
                        const float n = (float)smp + 1.f;
                        const float mu = s1 / n;
                        const float variance = (1.f / (n - 1.f)) * (s2 - (s1 * s1) / n);
                        const float I = 1.96f * sqrtf(variance / n);
                        stop = I <= fp.opt.sampling_tolerance * mu;
                    }
                }
                if (stop) { st.anum[p] = smp; stopped = smp; }
            }
        } else {
#pragma unroll
            for (int k = 0; k < NB; ++k) tot[k] = (k < (int)nb) ? st.arad[k * P + p] : 0.f;
        }
        if (!last) continue;
        // unidirectional (cpu_path_tracer.ipp:229-240) + RenderPasses::updateImages (passes.ipp:82-128);
        // a pixel that stopped early divides by the index of its last sample, as the reference does
        const float sf = stopped ? (float)stopped : sf_all;
        const uint32_t count = (fp.aux & AUX_DEP) ? st.acnt[p] : 0u;
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            if (k < (int)nb) {
                const float total = tot[k] / sf;
                const float direct = want_dir ? st.adir[k * P + p] / sf : 0.f;
                if (f.total) f.total[k * FP + p] = total;
                if (f.direct) f.direct[k * FP + p] = direct;
                if (f.indirect) f.indirect[k * FP + p] = total - direct;
                if (f.albedo) f.albedo[k * FP + p] = st.aalb[k * P + p] / sf;
                if (f.power) f.power[k * FP + p] = (fp.cam.power_scale[k] * f.omega[p]) * total;
            }
        }
        if (f.normal) {
            F3 n = normalize(F3{st.anrm[p], st.anrm[P + p], st.anrm[2 * P + p]});
            f.normal[p] = n.x; f.normal[FP + p] = n.y; f.normal[2 * FP + p] = n.z;
        }
        if (f.depth) f.depth[p] = (count == 0) ? __int_as_float(0x7f800000) : st.adep[p] / (float)count;
        if (f.alpha) f.alpha[p] = (float)count / sf;
        if (f.tri) f.tri[p] = st.atri[p];
    }
}

// ------------------------------------------------------------------ pixel solid angle (FP64)
// pixelToDirectionHelper_d (camera.ipp:1759-1771): the distortion models take and return FP32
// points, so with a distortion the FP64 point is rounded to FP32, undistorted and widened back.
__device__ double3 corner_dir(const vgb_camera& c, double x, double y) {
    const float* K = c.kinv;
    double hx = ((double)K[0] * x + (double)K[2] * y) + (double)K[4] * 1.0;
    double hy = ((double)K[1] * x + (double)K[3] * y) + (double)K[5] * 1.0;
    if (c.distortion) {
        const float2 u = undistort(c, (float)hx, (float)hy);
        hx = (double)u.x;
        hy = (double)u.y;
    }
    double zd = (double)c.z_dir;
    double vx = hx, vy = zd * hy, vz = zd;
    double s = 1.0 / sqrt((vx * vx + vy * vy) + vz * vz);
    return make_double3(vx * s, vy * s, vz * s);
}
__device__ double3 dcross(double3 a, double3 b) {
    return make_double3(a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y);
}
__device__ double ddot(double3 a, double3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ double3 dtangent(double3 p0, double3 p1) {
    double3 p = make_double3(p1.x - p0.x, p1.y - p0.y, p1.z - p0.z);
    double3 t = dcross(dcross(p0, p), p0);
    double s = 1.0 / sqrt(ddot(t, t));
    return make_double3(t.x * s, t.y * s, t.z * s);
}
__device__ double tri_omega(double3 c0, double3 c1, double3 c2) {
    double a0 = acos(ddot(dtangent(c0, c1), dtangent(c0, c2)));
    double a1 = acos(ddot(dtangent(c1, c0), dtangent(c1, c2)));
    double a2 = acos(ddot(dtangent(c2, c0), dtangent(c2, c1)));
    return ((a0 + a1) + a2) - 3.141592653589793238462;
}
__global__ void k_pixel_solid_angle(const __grid_constant__ vgb_camera cam, float* out) {
    const uint32_t W = cam.width, H = cam.height;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < W * H; p += gridDim.x * blockDim.x) {
        const uint32_t i = p % W, j = p / W;
        double3 c0 = corner_dir(cam, i, j), c1 = corner_dir(cam, i + 1, j);
        double3 c2 = corner_dir(cam, i + 1, j + 1), c3 = corner_dir(cam, i, j + 1);
        out[p] = (float)(tri_omega(c0, c1, c2) + tri_omega(c0, c2, c3));
    }
}

// ------------------------------------------------------------------ batch trace (TLAS::intersect seam)
template <int L, bool ANY, bool COUNT>
__global__ void __launch_bounds__(VGB_RAYS_BLOCK) k_trace_batch(const DevScene s, const float* org, const float* dir, const float* tmax,
                                               uint32_t n, uint32_t* tri, float* tout, float* bary,
                                               uint32_t* counters, uint64_t* stats) {
    uint32_t err = 0;
    Counters cnt{0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        F3 o{org[3 * i], org[3 * i + 1], org[3 * i + 2]};
        F3 d{dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]};
        WRay wr = make_wray(o, d);
        HitOut h;
        h.U = h.V = h.W = 0.f; h.det = 1.f;
        traverse_any_layout<L, ANY, COUNT>(s.nodes, s.tris, wr, tmax ? tmax[i] : __int_as_float(0x7f800000), h, err, cnt, s.iter_cap);
        tri[i] = h.id;
        if (tout) tout[i] = h.t;
        if (bary) {
            float w0 = 0.f, w1 = 0.f, w2 = 0.f;
            if (h.id != VGB_NO_HIT && !ANY) {
                const float rcp = 1.0f / h.det;
                w0 = h.V * rcp; w1 = h.W * rcp; w2 = 1.0f - w0 - w1;
            }
            bary[3 * i] = w0; bary[3 * i + 1] = w1; bary[3 * i + 2] = w2;
        }
    }
    if (err) atomicOr(&counters[C_ERR], err);
    if (COUNT) {
        warp_reduce_add(&stats[0], cnt.nodes);
        warp_reduce_add(&stats[1], cnt.tris);
        if (!ANY) {
            warp_reduce_add(&stats[4], cnt.nodes);
            warp_reduce_add(&stats[5], cnt.tris);
        }
    }
}

}  // namespace

// ====================================================================== context
struct vgb_context {
    int device = 0;
    int num_sms = 1;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::string err;
    // scene
    uint32_t nverts = 0, ntris = 0, nbands = 0;
    float4* d_vpos = nullptr;
    float4* d_vnrm = nullptr;
    float2* d_vuv = nullptr;
    float* d_valb = nullptr;
    uint32_t* d_idx = nullptr;
    float* d_tex = nullptr;
    uint32_t tw = 1, th = 1;
    float* d_nmap = nullptr;        // tangent-space normal map [nh][nw][3], or null
    uint32_t nw = 0, nh = 0;
    vgb_instance_motion* d_motion = nullptr;   // instance motion table, or null (all at rest)
    uint32_t nmotion = 0;
    uint32_t albedo_uniform = 0, tex_mono = 0;
    float albedo_value[VGB_MAX_BANDS] = {0};
    std::vector<float> h_pos;   // kept for the BVH build
    std::vector<uint32_t> h_idx;
    // BVH
    uint4* d_nodes = nullptr;
    float4* d_tris = nullptr;
    uint32_t nnodes = 0;
    uint32_t bvh_layout = 2;
    bool bvh_ready = false;
    uint32_t* d_parent = nullptr;   // binary layout: (parent << 1 | side) per node, for refits
    uint32_t* d_refit = nullptr;    // nnodes + 1 words: arrival counters and the walk-bound flag
    uint32_t bvh_leaf = 0, bvh_threads = 0;
    bool h_pos_stale = false;       // device positions moved by a device-side update
    uint32_t* d_vnl = nullptr;      // per-vertex corner lists of the uploaded mesh (vertex-normal updates)
    // render scratch
    size_t cap_P = 0, cap_items = 0;
    uint32_t cap_B = 0, cap_L = 0;
    std::vector<void*> scratch;
    DevState st{};
    uint32_t* d_counters = nullptr;
    uint64_t* d_stats = nullptr;
    // staging for host films / host rays
    std::vector<void*> staging;
    size_t staging_bytes = 0;
    void* staging_base = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    vgb_stats stats{};
    bool count_pass = false;
    bool profiling = false;
    std::vector<cudaEvent_t> prof_events;   // pairs around each launch
    std::vector<int> prof_family;           // 0 closest-hit trace, 1 shadow, 2 film, 3 shade
    size_t prof_used = 0;
    // batched rendering
    void* d_frames = nullptr;                // DevFrame table
    size_t cap_frames = 0;
    void* h_frames = nullptr;                // pinned staging of the table
    uint32_t tuned_threads = 0, tuned_bps = 0, tuned_grab = 0;
    cudaGraphExec_t graph_exec = nullptr;
    uint64_t graph_key = 0;
    unsigned char graph_params_probe[1024] = {0};   // kernel parameters the graph was captured with
    // adjoint
    float* d_adj = nullptr;                  // [nverts][3] vertex-normal gradients, [nverts][3] normal sums,
    size_t cap_adj = 0;                      //   [nverts][3] position gradients (z-only callers)
    void* d_views = nullptr;                 // DevView table of vgb_render_adjoint_batch
    size_t cap_views = 0;
    double* d_loss = nullptr;
    // denoiser scratch: ping-pong illumination planes and the render's internal passes
    float* d_dn = nullptr;
    size_t cap_dn = 0;
    // pinned host staging of file payloads (Quipu LoDs)
    void* h_pin = nullptr;
    size_t cap_pin = 0;
    // device address of vgb_render_noalloc's fixed array, looked up by its first call
    unsigned char* noalloc_base = nullptr;
    // traversal steps per ray before the ray gives up (vgb_set_traversal_limit)
    uint32_t iter_cap = vgbd::kIterCap;
    // wavefront traversal (vgb_set_wavefront_tuning): persistent kernels, node visits per ray
    // between hand-outs, free lanes that trigger a hand-out
    uint32_t trav_persistent = 0, trav_budget = VGB_TRAV_BUDGET, trav_refill = VGB_TRAV_REFILL;
};

namespace {

vgb_status fail(vgb_context* c, vgb_status s, const std::string& msg) {
    if (c) c->err = msg;
    return s;
}

#define CK(call)                                                                                  \
    do {                                                                                          \
        cudaError_t e_ = (call);                                                                  \
        if (e_ != cudaSuccess) {                                                                  \
            return fail(ctx, e_ == cudaErrorMemoryAllocation ? VGB_ERR_OUT_OF_MEMORY : VGB_ERR_CUDA, \
                        std::string(#call) + ": " + cudaGetErrorString(e_));                     \
        }                                                                                         \
    } while (0)

template <typename T>
vgb_status dalloc(vgb_context* ctx, T** p, size_t bytes) {
    *p = nullptr;
    if (bytes == 0) bytes = 16;
    cudaError_t e = cudaMalloc((void**)p, bytes);
    if (e != cudaSuccess) return fail(ctx, VGB_ERR_OUT_OF_MEMORY, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    return VGB_OK;
}

void dfree(void* p) { if (p) cudaFree(p); }

void free_scene(vgb_context* ctx) {
    dfree(ctx->d_vpos); dfree(ctx->d_vnrm); dfree(ctx->d_vuv); dfree(ctx->d_valb); dfree(ctx->d_idx); dfree(ctx->d_tex);
    ctx->d_vpos = nullptr; ctx->d_vnrm = nullptr; ctx->d_vuv = nullptr; ctx->d_valb = nullptr; ctx->d_idx = nullptr; ctx->d_tex = nullptr;
    dfree(ctx->d_vnl);
    ctx->d_vnl = nullptr;
    dfree(ctx->d_nmap);
    ctx->d_nmap = nullptr;
    ctx->nw = ctx->nh = 0;
    dfree(ctx->d_motion);
    ctx->d_motion = nullptr;
    ctx->nmotion = 0;
}
void free_bvh(vgb_context* ctx) {
    dfree(ctx->d_nodes); dfree(ctx->d_tris); dfree(ctx->d_parent); dfree(ctx->d_refit);
    ctx->d_nodes = nullptr; ctx->d_tris = nullptr; ctx->d_parent = nullptr; ctx->d_refit = nullptr;
    ctx->bvh_ready = false; ctx->nnodes = 0;
}
void free_scratch(vgb_context* ctx) {
    for (void* p : ctx->scratch) dfree(p);
    ctx->scratch.clear();
    ctx->cap_P = 0; ctx->cap_items = 0; ctx->cap_B = 0; ctx->cap_L = 0;
}
void free_staging(vgb_context* ctx) {
    dfree(ctx->staging_base);
    ctx->staging_base = nullptr;
    ctx->staging_bytes = 0;
}

// The device address of a pinned, mapped host allocation (cudaHostAlloc, cudaHostRegister) on the
// current device, or null for device memory, pageable memory and null pointers.
void* mapped_host(const void* p) {
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? a.devicePointer : nullptr;
}

vgb_status ensure_staging(vgb_context* ctx, size_t bytes) {
    if (bytes <= ctx->staging_bytes) return VGB_OK;
    free_staging(ctx);
    vgb_status s = dalloc(ctx, &ctx->staging_base, bytes);
    if (s != VGB_OK) return s;
    ctx->staging_bytes = bytes;
    return VGB_OK;
}

// Scratch for a frame of P pixels whose bounce-0 launch covers n_items queue items (the frame
// rounded up to whole 8x4-pixel tiles, so n_items >= P): the hit records of bounce 0 are indexed
// by item, every other plane by pixel or by a queue position below P.
vgb_status ensure_scratch(vgb_context* ctx, size_t P, size_t n_items, uint32_t B, uint32_t L) {
    if (P <= ctx->cap_P && n_items <= ctx->cap_items && B <= ctx->cap_B && L <= ctx->cap_L) return VGB_OK;
    P = std::max(P, ctx->cap_P);
    n_items = std::max(std::max(n_items, P), ctx->cap_items);
    B = std::max(B, ctx->cap_B);
    L = std::max(L, ctx->cap_L);
    free_scratch(ctx);
    DevState& st = ctx->st;
    auto A = [&](auto** p, size_t n) -> vgb_status {
        vgb_status s = dalloc(ctx, p, n);
        if (s == VGB_OK) ctx->scratch.push_back((void*)*p);
        return s;
    };
    vgb_status s = VGB_OK;
    const size_t f = sizeof(float), u = sizeof(uint32_t);
#define AL(ptr, n) do { s = A(&(ptr), (n)); if (s != VGB_OK) { free_scratch(ctx); return s; } } while (0)
    AL(st.org, 3 * P * f); AL(st.dir, 3 * P * f); AL(st.thr, B * P * f); AL(st.prad, B * P * f);
    AL(st.brad, B * P * f); AL(st.pend, P * u);
    AL(st.arad, B * P * f); AL(st.adir, B * P * f); AL(st.aalb, B * P * f); AL(st.anrm, 3 * P * f);
    AL(st.adep, P * f); AL(st.acnt, P * u); AL(st.atri, P * u);
    AL(st.pq[0], P * u); AL(st.pq[1], P * u);
    AL(st.hit, n_items * sizeof(float4));
    AL(st.as1, P * f); AL(st.as2, P * f); AL(st.anum, P * u);
    st.binq = nullptr;
    if (VGB_TRACE_BINS > 0) AL(st.binq, VGB_TRACE_BINS * P * u);
    for (uint32_t l = 0; l < VGB_MAX_LIGHTS; ++l) {
        if (l < L) {
            AL(st.sq_org[l], 3 * P * f); AL(st.sq_dir[l], 3 * P * f); AL(st.sq_tmax[l], P * f);
            AL(st.sq_slot[l], P * u); AL(st.sq_con[l], B * P * f);
        } else {
            st.sq_org[l] = st.sq_dir[l] = st.sq_tmax[l] = st.sq_con[l] = nullptr; st.sq_slot[l] = nullptr;
        }
    }
#undef AL
    st.counters = ctx->d_counters;
    st.stats = ctx->d_stats;
    st.P = P;
    ctx->cap_P = P; ctx->cap_items = n_items; ctx->cap_B = B; ctx->cap_L = L;
    return VGB_OK;
}

DevScene dev_scene(const vgb_context* ctx) {
    DevScene s;
    s.nodes = ctx->d_nodes; s.tris = ctx->d_tris; s.idx = ctx->d_idx; s.vpos = ctx->d_vpos; s.vnrm = ctx->d_vnrm;
    s.vuv = ctx->d_vuv; s.valb = ctx->d_valb; s.tex = ctx->d_tex; s.tw = ctx->tw; s.th = ctx->th;
    s.nmap = ctx->d_nmap; s.nw = ctx->nw; s.nh = ctx->nh;
    s.motion = ctx->d_motion; s.nmotion = ctx->nmotion;
    s.albedo_uniform = ctx->albedo_uniform; s.tex_mono = ctx->tex_mono;
    s.iter_cap = ctx->iter_cap;
    for (int k = 0; k < VGB_MAX_BANDS; ++k) s.albedo_value[k] = ctx->albedo_value[k];
    return s;
}

// Blocks for n items at `items` items per block, capped at per_sm blocks per SM (0: no cap).
int grid_for(const vgb_context* ctx, size_t n, int per_sm = 8, size_t items = 256) {
    size_t blocks = (n + items - 1) / items;
    size_t cap = per_sm > 0 ? (size_t)ctx->num_sms * per_sm : blocks;
    return (int)std::max<size_t>(1, std::min(blocks, cap));
}

// CUDA events around one launch when `on` and the context's profiling switch are both set.
struct Prof {
    vgb_context* ctx;
    int family;
    size_t slot;
    bool on;
    Prof(vgb_context* c, int fam, bool enable) : ctx(c), family(fam), slot(0), on(enable && c->profiling) {
        if (!on) return;
        if (ctx->prof_used + 2 > ctx->prof_events.size()) {
            for (int k = 0; k < 64; ++k) {
                cudaEvent_t e;
                cudaEventCreate(&e);
                ctx->prof_events.push_back(e);
            }
            ctx->prof_family.resize(ctx->prof_events.size() / 2);
        }
        slot = ctx->prof_used;
        ctx->prof_used += 2;
        ctx->prof_family[slot / 2] = family;
        cudaEventRecord(ctx->prof_events[slot], ctx->stream);
    }
    ~Prof() {
        if (on) cudaEventRecord(ctx->prof_events[slot + 1], ctx->stream);
    }
};

// Queue items of a frame's bounce-0 launch: the frame rounded up to whole 8x4-pixel tiles.
inline uint64_t tile_items(uint32_t W, uint32_t H) {
    return (((uint64_t)W + 7u) / 8u) * (((uint64_t)H + 3u) / 4u) * 32u;
}

// A frame the kernels can index: non-empty, pixel indices and tile items within 2^31 (32-bit
// slots and grid-stride loops that cannot wrap).
inline bool frame_fits(uint32_t W, uint32_t H) {
    return W != 0 && H != 0 && (uint64_t)W * H <= (1ull << 31) && tile_items(W, H) <= (1ull << 31);
}

// The render's launch sequence (per sample: per bounce k_trace, k_shade, k_shadow per light;
// then k_end_sample) over the scratch `st`.  vgb_render passes the context's scratch,
// vgb_render_noalloc the fixed array; `prof` allows CUDA-event profiling of the launches.
// Resident blocks of a 256-thread kernel on the whole GPU (one wave of a persistent launch).
template <typename K>
int resident_grid(const vgb_context* ctx, K kernel) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, 256, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
    return per_sm * ctx->num_sms;
}

template <int NB, int L, bool COUNT>
void launch_render(vgb_context* ctx, const FrameParams& fp, const FilmOut& film, const DevState& st, bool prof,
                   uint32_t& launches) {
    const DevScene s = dev_scene(ctx);
    const uint32_t n0 = (uint32_t)tile_items(fp.cam.width, fp.cam.height);
    const int gt = grid_for(ctx, n0, VGB_TRACE_GRID * 256 / VGB_TRACE_BLOCK, VGB_TRACE_BLOCK);
    const int gs = grid_for(ctx, n0, VGB_SHADE_GRID * 256 / VGB_SHADE_BLOCK, VGB_SHADE_BLOCK);
    const int go = grid_for(ctx, n0, VGB_SHADOW_GRID * 256 / VGB_SHADOW_BLOCK, VGB_SHADOW_BLOCK);
    const int gp = grid_for(ctx, (size_t)fp.cam.width * fp.cam.height, VGB_END_GRID);
    // persistent traversal (binary layout): one resident wave, lanes refilled from the queue
    const bool persist = L == 2 && ctx->trav_persistent;
    const int gtp = persist ? resident_grid(ctx, k_trace_p<COUNT>) : 0;
    const int gop = persist ? resident_grid(ctx, k_shadow_p<NB, COUNT>) : 0;
    const int budget = (int)ctx->trav_budget;
    const uint32_t refill = ctx->trav_refill;
#if VGB_L1_CARVEOUT >= 0
    static bool carved = false;   // once per instantiation (the attribute is the function's)
    if (!carved) {
        cudaFuncSetAttribute(k_trace<L, COUNT, true>, cudaFuncAttributePreferredSharedMemoryCarveout, VGB_L1_CARVEOUT);
        cudaFuncSetAttribute(k_trace<L, COUNT, false>, cudaFuncAttributePreferredSharedMemoryCarveout, VGB_L1_CARVEOUT);
        cudaFuncSetAttribute(k_shadow<NB, L, COUNT>, cudaFuncAttributePreferredSharedMemoryCarveout, VGB_L1_CARVEOUT);
        cudaFuncSetAttribute(k_shade<NB, true>, cudaFuncAttributePreferredSharedMemoryCarveout, VGB_L1_CARVEOUT);
        cudaFuncSetAttribute(k_shade<NB, false>, cudaFuncAttributePreferredSharedMemoryCarveout, VGB_L1_CARVEOUT);
        carved = true;
    }
#endif
    for (uint32_t smp = 0; smp < fp.opt.samples; ++smp) {
        uint32_t q = 0;
        for (uint32_t b = 0; b <= fp.opt.bounces; ++b) {
            // reset the output path queue, the shadow queues and the persistent item counters
            cudaMemsetAsync(&st.counters[(q ^ 1u)], 0, sizeof(uint32_t), ctx->stream);
            cudaMemsetAsync(&st.counters[C_SQ], 0, sizeof(uint32_t) * kBounceResetWords, ctx->stream);
#if VGB_TRACE_BINS > 0
            if (b != 0 && st.binq && !persist) {
                cudaMemsetAsync(&st.counters[C_BIN], 0, sizeof(uint32_t) * VGB_TRACE_BINS, ctx->stream);
                k_bin_rays<<<gs, 256, 0, ctx->stream>>>(st, q);
                launches++;
            }
#endif
            {
                Prof p(ctx, 0, prof);
                if (persist) k_trace_p<COUNT><<<gtp, 256, 0, ctx->stream>>>(s, st, fp, b, smp, q, n0, budget, refill);
                else if (b == 0) k_trace<L, COUNT, true><<<gt, VGB_TRACE_BLOCK, 0, ctx->stream>>>(s, st, fp, b, smp, q, n0);
                else k_trace<L, COUNT, false><<<gt, VGB_TRACE_BLOCK, 0, ctx->stream>>>(s, st, fp, b, smp, q, n0);
            }
            {
                Prof p(ctx, 3, prof);
                if (b == 0) k_shade<NB, true><<<gs, VGB_SHADE_BLOCK, 0, ctx->stream>>>(s, st, fp, b, smp, q, n0);
                else k_shade<NB, false><<<gs, VGB_SHADE_BLOCK, 0, ctx->stream>>>(s, st, fp, b, smp, q, n0);
            }
            launches += 2;
            for (uint32_t l = 0; l < fp.nlights; ++l) {
                Prof p(ctx, 1, prof);
                if (persist) k_shadow_p<NB, COUNT><<<gop, 256, 0, ctx->stream>>>(s, st, l, fp.nb, budget, refill);
                else k_shadow<NB, L, COUNT><<<go, VGB_SHADOW_BLOCK, 0, ctx->stream>>>(s, st, l, fp.nb);
                launches++;
            }
            q ^= 1u;
        }
        {
            Prof p(ctx, 2, prof);
            const uint32_t last = smp + 1 == fp.opt.samples ? 1u : 0u;
            if (fp.opt.adaptive_sampling) k_end_sample<NB, true><<<gp, 256, 0, ctx->stream>>>(st, fp, smp, last, film);
            else k_end_sample<NB, false><<<gp, 256, 0, ctx->stream>>>(st, fp, smp, last, film);
        }
        launches++;
    }
}

template <int L, bool COUNT>
void dispatch_render_l(vgb_context* ctx, const FrameParams& fp, const FilmOut& film, const DevState& st, bool prof,
                       uint32_t& launches) {
    if (fp.nb <= 1) launch_render<1, L, COUNT>(ctx, fp, film, st, prof, launches);
    else if (fp.nb <= 4) launch_render<4, L, COUNT>(ctx, fp, film, st, prof, launches);
    else launch_render<8, L, COUNT>(ctx, fp, film, st, prof, launches);
}

template <bool COUNT>
void dispatch_render(vgb_context* ctx, const FrameParams& fp, const FilmOut& film, const DevState& st, bool prof,
                     uint32_t& launches) {
    if (ctx->bvh_layout == 8) dispatch_render_l<8, COUNT>(ctx, fp, film, st, prof, launches);
    else dispatch_render_l<2, COUNT>(ctx, fp, film, st, prof, launches);
}

}  // namespace

// ====================================================================== C ABI
// ====================================================================== EATWT denoiser
// denoiseSpectralRadianceEATWT (rendering/cpu_denoise.ipp:9-214): the direct and indirect
// radiance are divided by the albedo (clamped below by epsilon), filtered level by level with
// the 5-tap binomial kernel at a stride of 2^level, each tap weighted by a depth-ratio and a
// normal-similarity term, and multiplied back by the albedo.  The reference indexes its images
// (y, x), i.e. transposed: its first ("horizontal") pass of a level runs along image columns and
// its second along rows, which is the order used here (exactly the reference's on square images).
namespace {

__constant__ float kEatwtTaps[5] = {1.0f / 16.0f, 4.0f / 16.0f, 6.0f / 16.0f, 4.0f / 16.0f, 1.0f / 16.0f};

struct DnOpts {
    uint32_t levels_direct, levels_indirect;
    float depth_threshold, normal_threshold, min_normal_weight, eps;
};

DnOpts dn_opts(const vgb_denoise_options* o) {
    DnOpts d{5u, 5u, 0.2f, 0.5f, 0.3f, 1e-6f};  // EATWTOptions defaults (cpu_denoise.hpp:10-19)
    if (!o) return d;
    if (o->levels_direct) d.levels_direct = o->levels_direct;
    if (o->levels_indirect) d.levels_indirect = o->levels_indirect;
    if (o->depth_threshold != 0.f) d.depth_threshold = o->depth_threshold;
    if (o->normal_threshold != 0.f) d.normal_threshold = o->normal_threshold;
    if (o->min_normal_weight != 0.f) d.min_normal_weight = o->min_normal_weight;
    if (o->epsilon != 0.f) d.eps = o->epsilon;
    return d;
}

// Working layout of the filter: each illumination image interleaved per pixel ([P][NB], so a
// tap is one or two float4 loads) and the guide packed as one float4 per pixel (depth, normal).
template <int NB>
__global__ void k_dn_split(const float* __restrict__ direct, const float* __restrict__ indirect,
                           const float* __restrict__ albedo, const float* __restrict__ depth,
                           const float* __restrict__ normal, float* __restrict__ D, float* __restrict__ I,
                           float4* __restrict__ guide, size_t P, uint32_t nb, float eps) {
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            float d = 0.f, i = 0.f;
            if (k < (int)nb) {
                const float a = smax(albedo[k * P + p], eps);
                d = direct[k * P + p] / a;
                i = indirect[k * P + p] / a;
            }
            D[p * NB + k] = d;
            I[p * NB + k] = i;
        }
        guide[p] = make_float4(depth[p], normal[p], normal[P + p], normal[2 * P + p]);
    }
}

template <int NB>
__device__ __forceinline__ void dn_load(const float* __restrict__ src, size_t q, float* v) {
    if (NB % 4 == 0) {
        const float4* s4 = reinterpret_cast<const float4*>(src + q * NB);
#pragma unroll
        for (int j = 0; j < NB / 4; ++j) {
            const float4 t = s4[j];
            v[4 * j] = t.x; v[4 * j + 1] = t.y; v[4 * j + 2] = t.z; v[4 * j + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int k = 0; k < NB; ++k) v[k] = src[q * NB + k];
    }
}

template <int NB>
__device__ __forceinline__ void dn_store(float* __restrict__ dst, size_t q, const float* v) {
    if (NB % 4 == 0) {
        float4* d4 = reinterpret_cast<float4*>(dst + q * NB);
#pragma unroll
        for (int j = 0; j < NB / 4; ++j) d4[j] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
    } else {
#pragma unroll
        for (int k = 0; k < NB; ++k) dst[q * NB + k] = v[k];
    }
}

// One pass of one level over both illumination images (either may be null: its level count is
// exhausted).  The tap weights depend only on depth and normal, so they are formed once.
template <int NB>
__global__ void k_dn_pass(const float* __restrict__ Din, float* __restrict__ Dout, const float* __restrict__ Iin,
                          float* __restrict__ Iout, const float4* __restrict__ guide, uint32_t W, uint32_t H,
                          uint32_t nb, int step, int along_columns, const DnOpts o) {
    const size_t P = (size_t)W * H;
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(p % W), y = (int)(p / W);
        const float4 cg = guide[p];
        const float cd = cg.x;
        float w[5];
        size_t q[5];
        float wsum = 0.f;
#pragma unroll
        for (int t = 0; t < 5; ++t) {
            const int k = t - 2;
            int sx = along_columns ? x : x + k * step;
            int sy = along_columns ? y + k * step : y;
            sx = min(max(sx, 0), (int)W - 1);
            sy = min(max(sy, 0), (int)H - 1);
            q[t] = (size_t)sy * W + sx;
            const float4 sg = guide[q[t]];
            const float sd = sg.x;
            const float ratio = smax(cd, sd) / (smin(cd, sd) + o.eps);
            const float dw = ratio < (1.0f + o.depth_threshold) ? 1.0f : expf(-(ratio - 1.0f) / o.depth_threshold);
            const float nd = (cg.y * sg.y + cg.z * sg.z) + cg.w * sg.w;
            const float sim = smax(0.0f, nd);
            const float om = 1.0f - sim;
            const float nw = smax(o.min_normal_weight, expf(-(om * om) / o.normal_threshold));
            w[t] = (kEatwtTaps[t] * dw) * nw;
            wsum += w[t];
        }
        const bool norm = wsum > o.eps;
#pragma unroll
        for (int img = 0; img < 2; ++img) {
            const float* in = img ? Iin : Din;
            float* out = img ? Iout : Dout;
            if (!in) continue;
            float sum[NB], v[NB];
#pragma unroll
            for (int k = 0; k < NB; ++k) sum[k] = 0.f;
#pragma unroll
            for (int t = 0; t < 5; ++t) {
                dn_load<NB>(in, q[t], v);
#pragma unroll
                for (int k = 0; k < NB; ++k) sum[k] += v[k] * w[t];
            }
            if (norm) {
#pragma unroll
                for (int k = 0; k < NB; ++k) sum[k] = sum[k] / wsum;
            } else {
                dn_load<NB>(in, p, sum);
            }
            dn_store<NB>(out, p, sum);
        }
    }
}

struct PowerScale { float v[VGB_MAX_BANDS]; };

template <int NB>
__global__ void k_dn_merge(const float* __restrict__ D, const float* __restrict__ I, const float* __restrict__ albedo,
                           float* direct, float* indirect, float* __restrict__ total, float* __restrict__ power,
                           const float* __restrict__ omega, const PowerScale ps, size_t P, uint32_t nb) {
    for (size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (size_t)gridDim.x * blockDim.x) {
        float dv[NB], iv[NB];
        dn_load<NB>(D, p, dv);
        dn_load<NB>(I, p, iv);
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            if (k >= (int)nb) break;
            const float a = albedo[k * P + p];
            const float d = dv[k] * a, i = iv[k] * a;
            if (direct) direct[k * P + p] = d;
            if (indirect) indirect[k * P + p] = i;
            const float t = d + i;  // renderPasses.total_radiance = direct + indirect
            if (total) total[k * P + p] = t;
            if (power) power[k * P + p] = (ps.v[k] * omega[p]) * t;
        }
    }
}

// Floats of the filter's working buffers: two ping-pong pairs of interleaved images (bands
// rounded up to the kernel instance, 1, 4 or 8) and the packed guide.
size_t dn_work_floats(uint32_t nb, size_t P) {
    const size_t nbs = nb <= 1 ? 1 : (nb <= 4 ? 4 : 8);
    return 4 * nbs * P + 4 * P;
}

vgb_status ensure_dn_scratch(vgb_context* ctx, size_t floats) {
    const size_t need = floats * sizeof(float);
    if (need <= ctx->cap_dn) return VGB_OK;
    dfree(ctx->d_dn);
    ctx->d_dn = nullptr;
    ctx->cap_dn = 0;
    vgb_status s = dalloc(ctx, &ctx->d_dn, need);
    if (s != VGB_OK) return s;
    ctx->cap_dn = need;
    return VGB_OK;
}

template <int NB>
void launch_denoise_t(vgb_context* ctx, const float* in_d, const float* in_i, const float* albedo, const float* depth,
                      const float* normal, uint32_t W, uint32_t H, uint32_t nb, const DnOpts& o, float* scratch,
                      float* out_d, float* out_i, float* total, float* power, const float* omega, const PowerScale& ps) {
    const size_t P = (size_t)W * H;
    const int g = grid_for(ctx, P);
    float* Db[2] = {scratch, scratch + NB * P};
    float* Ib[2] = {scratch + 2 * NB * P, scratch + 3 * NB * P};
    float4* guide = reinterpret_cast<float4*>(scratch + 4 * NB * P);
    k_dn_split<NB><<<g, 256, 0, ctx->stream>>>(in_d, in_i, albedo, depth, normal, Db[0], Ib[0], guide, P, nb, o.eps);
    int cd = 0, ci = 0;  // buffer holding the current image
    const uint32_t levels = std::max(o.levels_direct, o.levels_indirect);
    for (uint32_t level = 0; level < levels; ++level) {
        const int step = 1 << std::min<uint32_t>(level, 30u);
        const bool fd = level < o.levels_direct, fi = level < o.levels_indirect;
        for (int pass = 0; pass < 2; ++pass) {
            k_dn_pass<NB><<<g, 256, 0, ctx->stream>>>(fd ? Db[cd] : nullptr, fd ? Db[cd ^ 1] : nullptr,
                                                      fi ? Ib[ci] : nullptr, fi ? Ib[ci ^ 1] : nullptr, guide, W, H,
                                                      nb, step, pass == 0 ? 1 : 0, o);
            if (fd) cd ^= 1;
            if (fi) ci ^= 1;
        }
    }
    k_dn_merge<NB><<<g, 256, 0, ctx->stream>>>(Db[cd], Ib[ci], albedo, out_d, out_i, total, power, omega, ps, P, nb);
}

void launch_denoise(vgb_context* ctx, const float* in_d, const float* in_i, const float* albedo, const float* depth,
                    const float* normal, uint32_t W, uint32_t H, uint32_t nb, const DnOpts& o, float* scratch,
                    float* out_d, float* out_i, float* total, float* power, const float* omega, const PowerScale& ps) {
    if (nb <= 1) launch_denoise_t<1>(ctx, in_d, in_i, albedo, depth, normal, W, H, nb, o, scratch, out_d, out_i, total, power, omega, ps);
    else if (nb <= 4) launch_denoise_t<4>(ctx, in_d, in_i, albedo, depth, normal, W, H, nb, o, scratch, out_d, out_i, total, power, omega, ps);
    else launch_denoise_t<8>(ctx, in_d, in_i, albedo, depth, normal, W, H, nb, o, scratch, out_d, out_i, total, power, omega, ps);
}

}  // namespace

extern "C" {

VGB_API const char* vgb_version(void) { return "vira_gb300 0.1 (sm_103a)"; }

VGB_API vgb_status vgb_context_create(vgb_context** out, int device) try {
    if (!out) return VGB_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    vgb_context* ctx = new (std::nothrow) vgb_context();
    if (!ctx) return VGB_ERR_OUT_OF_MEMORY;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || device < 0 || device >= n) {
        delete ctx;
        return VGB_ERR_CUDA;
    }
    ctx->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete ctx; return VGB_ERR_CUDA; }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return VGB_ERR_CUDA; }
    ctx->own_stream = true;
    if (cudaMalloc(&ctx->d_counters, sizeof(uint32_t) * C_COUNT) != cudaSuccess ||
        cudaMalloc(&ctx->d_stats, sizeof(uint64_t) * 8) != cudaSuccess) {
        cudaStreamDestroy(ctx->stream);
        delete ctx;
        return VGB_ERR_OUT_OF_MEMORY;
    }
    cudaMemset(ctx->d_counters, 0, sizeof(uint32_t) * C_COUNT);
    cudaMemset(ctx->d_stats, 0, sizeof(uint64_t) * 8);
    cudaEventCreate(&ctx->ev0);
    cudaEventCreate(&ctx->ev1);
    *out = ctx;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(nullptr);
}

VGB_API vgb_status vgb_context_destroy(vgb_context* ctx) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    free_scene(ctx); free_bvh(ctx); free_scratch(ctx); free_staging(ctx);
    dfree(ctx->d_counters); dfree(ctx->d_stats);
    for (cudaEvent_t e : ctx->prof_events) cudaEventDestroy(e);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    dfree(ctx->d_frames);
    if (ctx->h_frames) cudaFreeHost(ctx->h_frames);
    dfree(ctx->d_adj); dfree(ctx->d_views); dfree(ctx->d_loss); dfree(ctx->d_dn);
    if (ctx->h_pin) cudaFreeHost(ctx->h_pin);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->own_stream && ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API const char* vgb_last_error(const vgb_context* ctx) { return ctx ? ctx->err.c_str() : "null context"; }

VGB_API vgb_status vgb_set_stream(vgb_context* ctx, void* stream) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream));
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    if (stream) { ctx->stream = (cudaStream_t)stream; ctx->own_stream = false; }
    else { CK(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking)); ctx->own_stream = true; }
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_synchronize(vgb_context* ctx) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream));
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_scene_motion(vgb_context* ctx, const vgb_instance_motion* motion, uint32_t n) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (ctx->nverts == 0) return fail(ctx, VGB_ERR_NOT_READY, "scene_motion: upload the scene first");
    if (motion && n) {
        if (motion[0].first_triangle != 0) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "scene_motion: the first entry must start at triangle 0");
        for (uint32_t k = 1; k < n; ++k)
            if (motion[k].first_triangle <= motion[k - 1].first_triangle || motion[k].first_triangle >= ctx->ntris)
                return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "scene_motion: first_triangle must ascend within the mesh");
    }
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream));
    dfree(ctx->d_motion);
    ctx->d_motion = nullptr;
    ctx->nmotion = 0;
    if (!motion || n == 0) return VGB_OK;
    vgb_status s = dalloc(ctx, &ctx->d_motion, sizeof(vgb_instance_motion) * n);
    if (s != VGB_OK) return s;
    CK(cudaMemcpy(ctx->d_motion, motion, sizeof(vgb_instance_motion) * n, cudaMemcpyHostToDevice));
    ctx->nmotion = n;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_scene_normal_map(vgb_context* ctx, const float* nmap, uint32_t w, uint32_t h) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (ctx->nverts == 0) return fail(ctx, VGB_ERR_NOT_READY, "scene_normal_map: upload the scene first");
    if (nmap && (uint64_t)w * h > (1ull << 31)) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "scene_normal_map: map too large");
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream));
    dfree(ctx->d_nmap);
    ctx->d_nmap = nullptr;
    ctx->nw = ctx->nh = 0;
    if (!nmap || w == 0 || h == 0) return VGB_OK;
    vgb_status s = dalloc(ctx, &ctx->d_nmap, (size_t)w * h * 3 * sizeof(float));
    if (s != VGB_OK) return s;
    CK(cudaMemcpy(ctx->d_nmap, nmap, (size_t)w * h * 3 * sizeof(float), cudaMemcpyHostToDevice));
    ctx->nw = w;
    ctx->nh = h;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_scene_upload(vgb_context* ctx, const float* pos, uint32_t nverts, const uint32_t* idx,
                                    uint32_t ntris, uint32_t nbands, const float* valb, const float* vnrm,
                                    const float* vuv, const float* tex, uint32_t tw, uint32_t th) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!pos || !idx || nverts == 0 || ntris == 0)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "scene_upload: empty mesh or null buffer");
    if (nbands == 0 || nbands > VGB_MAX_BANDS)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "scene_upload: nbands must be 1..8");
    if (tex && (tw == 0 || th == 0)) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "scene_upload: empty texture");
    for (size_t k = 0; k < (size_t)3 * ntris; ++k)
        if (idx[k] >= nverts) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "scene_upload: index out of range");
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream));
    free_scene(ctx);
    free_bvh(ctx);
    ctx->nverts = nverts; ctx->ntris = ntris; ctx->nbands = nbands;
    std::vector<float> nrm;
    if (!vnrm) {
        nrm.resize(3 * (size_t)nverts);
        vgb_status s = vgb_compute_vertex_normals(pos, nverts, idx, ntris, nrm.data());
        if (s != VGB_OK) return fail(ctx, s, "scene_upload: normals");
        vnrm = nrm.data();
    }
    std::vector<float4> p4(nverts), n4(nverts);
    for (uint32_t v = 0; v < nverts; ++v) {
        p4[v] = make_float4(pos[3 * v], pos[3 * v + 1], pos[3 * v + 2], 0.f);
        n4[v] = make_float4(vnrm[3 * v], vnrm[3 * v + 1], vnrm[3 * v + 2], 0.f);
    }
    std::vector<float2> uv2(nverts, make_float2(0.f, 0.f));
    if (vuv) for (uint32_t v = 0; v < nverts; ++v) uv2[v] = make_float2(vuv[2 * v], vuv[2 * v + 1]);
    std::vector<float> alb;
    if (!valb) { alb.assign((size_t)nverts * nbands, 1.f); valb = alb.data(); }
    std::vector<float> one;
    if (!tex) { one.assign(nbands, 1.f); tex = one.data(); tw = th = 1; }
    // Uniform inputs are folded into constants: same expressions, fewer gathers.
    bool uniform = true;
    for (size_t v = 1; v < nverts && uniform; ++v)
        for (uint32_t k = 0; k < nbands; ++k)
            if (std::memcmp(&valb[v * nbands + k], &valb[k], 4) != 0) { uniform = false; break; }
    bool mono = true;
    const size_t ntex = (size_t)tw * th;
    for (size_t t = 0; t < ntex && mono; ++t)
        for (uint32_t k = 1; k < nbands; ++k)
            if (std::memcmp(&tex[t * nbands + k], &tex[t * nbands], 4) != 0) { mono = false; break; }
    ctx->albedo_uniform = uniform ? 1u : 0u;
    ctx->tex_mono = mono ? 1u : 0u;
    for (uint32_t k = 0; k < VGB_MAX_BANDS; ++k) ctx->albedo_value[k] = k < nbands ? valb[k] : 0.f;
    std::vector<float> mono_tex;
    if (mono) {
        mono_tex.resize(ntex);
        for (size_t t = 0; t < ntex; ++t) mono_tex[t] = tex[t * nbands];
    }
    vgb_status s;
    if ((s = dalloc(ctx, &ctx->d_vpos, sizeof(float4) * nverts)) != VGB_OK) return s;
    if ((s = dalloc(ctx, &ctx->d_vnrm, sizeof(float4) * nverts)) != VGB_OK) return s;
    if ((s = dalloc(ctx, &ctx->d_vuv, sizeof(float2) * nverts)) != VGB_OK) return s;
    if ((s = dalloc(ctx, &ctx->d_valb, sizeof(float) * nverts * (size_t)nbands)) != VGB_OK) return s;
    if ((s = dalloc(ctx, &ctx->d_idx, sizeof(uint32_t) * 3 * (size_t)ntris)) != VGB_OK) return s;
    const size_t tex_floats = mono ? ntex : ntex * nbands;
    if ((s = dalloc(ctx, &ctx->d_tex, sizeof(float) * tex_floats)) != VGB_OK) return s;
    CK(cudaMemcpy(ctx->d_vpos, p4.data(), sizeof(float4) * nverts, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_vnrm, n4.data(), sizeof(float4) * nverts, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_vuv, uv2.data(), sizeof(float2) * nverts, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_valb, valb, sizeof(float) * nverts * (size_t)nbands, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_idx, idx, sizeof(uint32_t) * 3 * (size_t)ntris, cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_tex, mono ? mono_tex.data() : tex, sizeof(float) * tex_floats, cudaMemcpyHostToDevice));
    ctx->tw = tw; ctx->th = th;
    ctx->h_pos.assign(pos, pos + 3 * (size_t)nverts);
    ctx->h_idx.assign(idx, idx + 3 * (size_t)ntris);
    ctx->h_pos_stale = false;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_bvh_build(vgb_context* ctx, const vgb_bvh_options* opts) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (ctx->ntris == 0) return fail(ctx, VGB_ERR_NOT_READY, "bvh_build: no scene uploaded");
    uint32_t leaf = opts ? opts->max_leaf_size : 0, threads = opts ? opts->threads : 0;
    uint32_t layout = (opts && opts->layout) ? opts->layout : 2;
    if (opts && opts->builder > 1) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "bvh_build: unknown builder");
    if (layout != 2 && layout != 8) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "bvh_build: layout must be 2 or 8");
    if (opts && opts->builder == 1 && layout != 2)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "bvh_build: the GPU builder writes the binary layout");
    if (leaf > (layout == 8 ? vgb::kMaxLeaf8 : vgb::kMaxLeaf))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "bvh_build: max_leaf_size must be <= 8 (binary) or <= 3 (8-wide)");
    if (opts && opts->builder == 1 && ctx->ntris > (leaf ? leaf : 4u)) {
        // GPU linear BVH (binary layout), from the device vertices; a scene that fits one leaf
        // takes the host path below
        if (leaf == 0) leaf = 4;
        const uint32_t n = ctx->ntris;
        if ((uint64_t)n >= (1ull << (31 - vgb::kLeafShift)))
            return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "bvh_build: too many triangles for the leaf encoding");
        cudaSetDevice(ctx->device);
        CK(cudaStreamSynchronize(ctx->stream));
        free_bvh(ctx);
        vgb_status s;
        uint32_t nn = 0;
        if ((s = ensure_dn_scratch(ctx, vgb::lbvh_work_words(n))) != VGB_OK) return s;
        CK((cudaError_t)vgb::launch_lbvh_sort_and_link(ctx->stream, ctx->num_sms, ctx->d_vpos, ctx->d_idx, n, leaf,
                                                       reinterpret_cast<uint32_t*>(ctx->d_dn), &nn));
        if ((s = dalloc(ctx, &ctx->d_nodes, (size_t)nn * 64)) != VGB_OK) return s;
        if ((s = dalloc(ctx, &ctx->d_tris, (size_t)n * 48)) != VGB_OK) return s;
        if ((s = dalloc(ctx, &ctx->d_parent, (size_t)nn * 4)) != VGB_OK) return s;
        if ((s = dalloc(ctx, &ctx->d_refit, ((size_t)nn + 1) * 4)) != VGB_OK) return s;
        const int rc = vgb::launch_lbvh_emit(ctx->stream, ctx->num_sms, ctx->d_vpos, ctx->d_idx, n, leaf,
                                             reinterpret_cast<const uint32_t*>(ctx->d_dn),
                                             reinterpret_cast<uint32_t*>(ctx->d_nodes), nn, ctx->d_tris, ctx->d_parent,
                                             ctx->d_refit);
        if (rc == -2) return fail(ctx, VGB_ERR_INTERNAL, "bvh_build: GPU build walk exceeded the tree depth");
        CK((cudaError_t)rc);
        ctx->nnodes = nn;
        ctx->bvh_layout = 2;
        ctx->bvh_leaf = leaf; ctx->bvh_threads = 0;
        ctx->bvh_ready = true;
        ctx->stats.bvh_nodes = nn;
        ctx->stats.bvh_node_bytes = 64;
        ctx->stats.tri_record_bytes = 48;
        return VGB_OK;
    }
    if (leaf > (layout == 8 ? vgb::kMaxLeaf8 : vgb::kMaxLeaf))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "bvh_build: max_leaf_size must be <= 8 (binary) or <= 3 (8-wide)");
    cudaSetDevice(ctx->device);
    if (ctx->h_pos_stale) {
        // positions were last updated on the device: bring them back for the host builder
        std::vector<float4> p4(ctx->nverts);
        CK(cudaStreamSynchronize(ctx->stream));
        CK(cudaMemcpy(p4.data(), ctx->d_vpos, sizeof(float4) * ctx->nverts, cudaMemcpyDeviceToHost));
        for (uint32_t v = 0; v < ctx->nverts; ++v) {
            ctx->h_pos[3 * (size_t)v] = p4[v].x; ctx->h_pos[3 * (size_t)v + 1] = p4[v].y; ctx->h_pos[3 * (size_t)v + 2] = p4[v].z;
        }
        ctx->h_pos_stale = false;
    }
    vgb::BvhHost bvh;
    const char* why = "";
    if (!vgb::build_bvh(ctx->h_pos.data(), ctx->nverts, ctx->h_idx.data(), ctx->ntris, leaf, threads, layout, bvh, &why))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, std::string("bvh_build: ") + why);
    CK(cudaStreamSynchronize(ctx->stream));
    free_bvh(ctx);
    vgb_status s;
    if ((s = dalloc(ctx, &ctx->d_nodes, bvh.nodes.size() * sizeof(uint32_t))) != VGB_OK) return s;
    if ((s = dalloc(ctx, &ctx->d_tris, bvh.tris.size() * sizeof(float))) != VGB_OK) return s;
    CK(cudaMemcpy(ctx->d_nodes, bvh.nodes.data(), bvh.nodes.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(ctx->d_tris, bvh.tris.data(), bvh.tris.size() * sizeof(float), cudaMemcpyHostToDevice));
    if (layout == 2) {
        if ((s = dalloc(ctx, &ctx->d_parent, bvh.parent.size() * sizeof(uint32_t))) != VGB_OK) return s;
        if ((s = dalloc(ctx, &ctx->d_refit, (bvh.parent.size() + 1) * sizeof(uint32_t))) != VGB_OK) return s;
        CK(cudaMemcpy(ctx->d_parent, bvh.parent.data(), bvh.parent.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
    }
    ctx->nnodes = bvh.num_nodes;
    ctx->bvh_layout = layout;
    ctx->bvh_leaf = leaf; ctx->bvh_threads = threads;
    ctx->bvh_ready = true;
    ctx->stats.bvh_nodes = bvh.num_nodes;
    ctx->stats.bvh_node_bytes = layout == 8 ? 80 : 64;
    ctx->stats.tri_record_bytes = 48;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_pixel_solid_angle(vgb_context* ctx, const vgb_camera* cam, float* out, int on_device) try {
    if (!ctx || !cam || !out) return VGB_ERR_INVALID_ARGUMENT;
    if (cam->width == 0 || cam->height == 0) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "pixel_solid_angle: empty image");
    cudaSetDevice(ctx->device);
    const size_t n = (size_t)cam->width * cam->height;
    float* d = out;
    if (!on_device) {
        vgb_status s = ensure_staging(ctx, n * sizeof(float));
        if (s != VGB_OK) return s;
        d = (float*)ctx->staging_base;
    }
    k_pixel_solid_angle<<<grid_for(ctx, n, 16), 256, 0, ctx->stream>>>(*cam, d);
    CK(cudaGetLastError());
    if (!on_device) CK(cudaMemcpyAsync(out, d, n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_set_count_pass(vgb_context* ctx, int enable) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    ctx->count_pass = enable != 0;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_set_profiling(vgb_context* ctx, int enable) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    ctx->profiling = enable != 0;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_measure_l2_read(vgb_context* ctx, uint64_t bytes, uint32_t passes, uint32_t repeats,
                                       double* gbps) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!gbps || bytes < (1u << 20) || bytes > (uint64_t(1) << 34) || bytes % 16 != 0 || passes == 0 || repeats == 0)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "measure_l2_read: bytes in [1 MiB, 16 GiB], a multiple of 16; passes, repeats >= 1");
    CK(cudaSetDevice(ctx->device));
    void* buf = nullptr;
    vgb_status s = dalloc(ctx, &buf, bytes + 256);
    if (s != VGB_OK) return s;
    struct Free { void* p; ~Free() { dfree(p); } } guard{buf};
    uint32_t* sink = reinterpret_cast<uint32_t*>(static_cast<unsigned char*>(buf) + bytes);
    CK(cudaMemsetAsync(buf, 0x5A, bytes, ctx->stream));
    // warm-up: one pass brings the buffer into L2 (when it fits)
    if (vgb::launch_l2_read(ctx->stream, buf, bytes, 1, sink, ctx->num_sms)) CK(cudaGetLastError());
    double best = 0.0;
    for (uint32_t r = 0; r < repeats; ++r) {
        CK(cudaEventRecord(ctx->ev0, ctx->stream));
        if (vgb::launch_l2_read(ctx->stream, buf, bytes, passes, sink, ctx->num_sms)) CK(cudaGetLastError());
        CK(cudaEventRecord(ctx->ev1, ctx->stream));
        CK(cudaEventSynchronize(ctx->ev1));
        float ms = 0.f;
        CK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
        if (ms > 0.f) best = std::max(best, (double)bytes * passes / (ms * 1e-3) / 1e9);
    }
    *gbps = best;
    ctx->stats.ms_last = (float)((double)bytes * passes / (best * 1e9) * 1e3);
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_set_wavefront_tuning(vgb_context* ctx, uint32_t persistent, uint32_t budget,
                                            uint32_t refill) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (refill > 32) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "wavefront_tuning: refill is a lane count, 0..32");
    ctx->trav_persistent = persistent ? 1u : 0u;
    ctx->trav_budget = budget ? budget : VGB_TRAV_BUDGET;
    ctx->trav_refill = refill ? refill : VGB_TRAV_REFILL;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_set_traversal_limit(vgb_context* ctx, uint32_t max_steps) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    ctx->iter_cap = max_steps ? max_steps : vgbd::kIterCap;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_dem_triangulate_gpu(vgb_context* ctx, const float* heights, uint32_t W, uint32_t H, double sx,
                                           double sy, float* pos, uint32_t* idx, uint32_t* nt_out, int on_device) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!heights || !pos || !idx || !nt_out || W < 2 || H < 2 || (uint64_t)W * H >= (1ull << 31))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "dem_triangulate_gpu: null array or grid outside 2..2^31 posts");
    cudaSetDevice(ctx->device);
    const size_t nv = (size_t)W * H, nq = (size_t)(W - 1) * (H - 1);
    const size_t work = vgb::dem_work_words(W, H);
    const size_t stage = on_device ? 0 : nv + 3 * nv + 6 * nq;
    vgb_status s;
    if ((s = ensure_dn_scratch(ctx, work + stage)) != VGB_OK) return s;
    uint32_t* w = reinterpret_cast<uint32_t*>(ctx->d_dn);
    const float* h = heights;
    float* p = pos;
    uint32_t* ix = idx;
    if (!on_device) {
        float* cur = ctx->d_dn + work;
        CK(cudaMemcpyAsync(cur, heights, nv * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        h = cur; cur += nv;
        p = cur; cur += 3 * nv;
        ix = reinterpret_cast<uint32_t*>(cur);
    }
    uint32_t nt = 0;
    CK((cudaError_t)vgb::launch_dem_triangulate(ctx->stream, ctx->num_sms, h, W, H,
                                                vgb::dem_pose_of(1.0 * sx, 1.0 * sy, 0.0, 0.0, W, H), p, ix, w, &nt));
    if (!on_device) {
        CK(cudaMemcpyAsync(pos, p, 3 * nv * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(idx, ix, 3 * (size_t)nt * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    *nt_out = nt;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_compute_vertex_normals_gpu(vgb_context* ctx, const float* pos, uint32_t nverts,
                                                  const uint32_t* idx, uint32_t ntris, float* normals,
                                                  int on_device) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!pos || !idx || !normals || nverts == 0)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "compute_vertex_normals_gpu: null array or no vertices");
    cudaSetDevice(ctx->device);
    const size_t work = vgb::normals_work_words(nverts, ntris);
    const size_t stage = on_device ? 0 : 6 * (size_t)nverts + 3 * (size_t)ntris;
    vgb_status s;
    if ((s = ensure_dn_scratch(ctx, work + stage)) != VGB_OK) return s;
    uint32_t* w = reinterpret_cast<uint32_t*>(ctx->d_dn);
    const float* p = pos;
    const uint32_t* ix = idx;
    float* out = normals;
    if (!on_device) {
        float* cur = ctx->d_dn + work;
        CK(cudaMemcpyAsync(cur, pos, 3 * (size_t)nverts * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        p = cur; cur += 3 * (size_t)nverts;
        out = cur; cur += 3 * (size_t)nverts;
        CK(cudaMemcpyAsync(cur, idx, 3 * (size_t)ntris * sizeof(uint32_t), cudaMemcpyHostToDevice, ctx->stream));
        ix = reinterpret_cast<const uint32_t*>(cur);
    }
    const int rc = vgb::launch_vertex_normals(ctx->stream, ctx->num_sms, p, nverts, ix, ntris, out, w);
    if (rc == -1) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "compute_vertex_normals_gpu: an index is >= nverts");
    CK((cudaError_t)rc);
    if (!on_device) {
        CK(cudaMemcpyAsync(normals, out, 3 * (size_t)nverts * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaStreamSynchronize(ctx->stream));
    }
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

namespace {
__global__ void k_pack_vertices(const float* __restrict__ p3, const float* __restrict__ n3, uint32_t nv,
                                float4* __restrict__ p4, float4* __restrict__ n4) {
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
        p4[v] = make_float4(p3[3 * v], p3[3 * v + 1], p3[3 * v + 2], 0.f);
        n4[v] = make_float4(n3[3 * v], n3[3 * v + 1], n3[3 * v + 2], 0.f);
    }
}
}  // namespace

VGB_API vgb_status vgb_scene_update_positions(vgb_context* ctx, const float* pos, const float* normals, int on_device) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (ctx->nverts == 0) return fail(ctx, VGB_ERR_NOT_READY, "scene_update_positions: no scene uploaded");
    if (!pos) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "scene_update_positions: null positions");
    cudaSetDevice(ctx->device);
    const size_t nv = ctx->nverts, nt = ctx->ntris;
    vgb_status s;
    if (!normals && !ctx->d_vnl) {
        // the corner lists of this topology, once per upload
        if ((s = dalloc(ctx, &ctx->d_vnl, vgb::vertex_normal_list_words((uint32_t)nv, (uint32_t)nt) * 4)) != VGB_OK)
            return s;
        if ((s = ensure_dn_scratch(ctx, nv + vgb::scan_temp_words(nv + 1))) != VGB_OK) return s;
        const int rc = vgb::launch_vertex_normal_lists(ctx->stream, ctx->num_sms, ctx->d_idx, (uint32_t)nv, (uint32_t)nt,
                                                       ctx->d_vnl, reinterpret_cast<uint32_t*>(ctx->d_dn));
        if (rc != 0) { dfree(ctx->d_vnl); ctx->d_vnl = nullptr; }
        CK((cudaError_t)(rc == -1 ? (int)cudaErrorInvalidValue : rc));
    }
    const size_t work = normals ? 0 : (3 * nt + 3) & ~(size_t)3;   // face normals
    const size_t stage = (on_device ? 0 : 3 * nv) + (normals && on_device ? 0 : 3 * nv);
    if ((s = ensure_dn_scratch(ctx, work + stage)) != VGB_OK) return s;
    float* cur = ctx->d_dn + work;
    const float* p = pos;
    if (!on_device) {
        CK(cudaMemcpyAsync(cur, pos, 3 * nv * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        p = cur; cur += 3 * nv;
    }
    const float* n = normals;
    if (normals && !on_device) {
        CK(cudaMemcpyAsync(cur, normals, 3 * nv * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        n = cur;
    } else if (!normals) {
        CK((cudaError_t)vgb::launch_vertex_normals_listed(ctx->stream, ctx->num_sms, p, (uint32_t)nv, ctx->d_idx,
                                                          (uint32_t)nt, ctx->d_vnl, ctx->d_dn, cur));
        n = cur;
    }
    k_pack_vertices<<<grid_for(ctx, nv, 8), 256, 0, ctx->stream>>>(p, n, (uint32_t)nv, ctx->d_vpos, ctx->d_vnrm);
    CK(cudaGetLastError());
    if (on_device) {
        ctx->h_pos_stale = true;
    } else {
        ctx->h_pos.assign(pos, pos + 3 * nv);
        ctx->h_pos_stale = false;
    }
    if (ctx->bvh_ready) {
        if (ctx->bvh_layout == 2) {
            const int rc = vgb::launch_refit(ctx->stream, ctx->num_sms, ctx->d_vpos, ctx->d_idx, (uint32_t)nt, ctx->d_tris,
                                             reinterpret_cast<uint32_t*>(ctx->d_nodes), ctx->nnodes, ctx->d_parent,
                                             ctx->d_refit);
            if (rc == -2) return fail(ctx, VGB_ERR_CUDA, "scene_update_positions: refit walk exceeded the tree depth");
            CK((cudaError_t)rc);
        } else {
            vgb_bvh_options o{};
            o.max_leaf_size = ctx->bvh_leaf; o.threads = ctx->bvh_threads; o.layout = ctx->bvh_layout;
            if ((s = vgb_bvh_build(ctx, &o)) != VGB_OK) return s;
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

// ---------------------------------------------------------------- rasterizer
namespace {

// static_cast<int>(float) as x86-64 performs it (cvttss2si): values outside int's range and NaN
// become INT_MIN.  The reference's bounding boxes go through this cast.
__device__ __forceinline__ int x86_int(float x) {
    return (x >= -2147483648.f && x < 2147483648.f) ? (int)x : (int)0x80000000;
}

struct RasterParams {
    vgb_camera cam;
    float K[6];
    vgb_light lights[VGB_MAX_LIGHTS];
    uint32_t nlights, nb, smooth, lighting;
};

struct RTri {
    F3 vc[3];            // corners in the camera frame
    float px[3], py[3];  // projected corners
    float d[3];          // distances to the camera
    float area;
    int x0, x1, y0, y1;  // clamped pixel box [x0, x1) x [y0, y1)
};

// Camera frame, behind test, projection and pixel box of triangle t (cpu_rasterizer.ipp:73-120).
__device__ __forceinline__ bool raster_setup(const DevScene& s, const RasterParams& rp, uint32_t t, RTri& r) {
    const vgb_camera& c = rp.cam;
    F3 p[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) p[k] = ld3(__ldg(&s.vpos[__ldg(&s.idx[3 * (size_t)t + k])]));
    if (isinf(p[0].x) || isinf(p[1].x) || isinf(p[2].x)) return false;
    const F3 O{c.origin[0], c.origin[1], c.origin[2]};
    const F3 ax{c.rotation[0], c.rotation[1], c.rotation[2]}, ay{c.rotation[3], c.rotation[4], c.rotation[5]},
             az{c.rotation[6], c.rotation[7], c.rotation[8]};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const F3 d = p[k] - O;
        r.vc[k] = F3{dot(ax, d), dot(ay, d), dot(az, d)};
    }
#pragma unroll
    for (int k = 0; k < 3; ++k)
        if ((-c.z_dir * r.vc[k].z) >= 0) return false;   // Camera::behind (camera.ipp:1394-1397)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        float hx = r.vc[k].x / r.vc[k].z, hy = r.vc[k].y / r.vc[k].z;
        if (c.distortion) distort(c, hx, hy);   // Camera::projectCameraPoint (camera.ipp:1060-1080)
        float X = (rp.K[0] * hx + rp.K[1] * hy) + rp.K[2];
        const float Y = (rp.K[3] * hx + rp.K[4] * hy) + rp.K[5];
        if (c.z_dir < 0) X = (float)(c.width - 1) - X;   // Blender frame (camera.ipp:1062-1080)
        r.px[k] = X;
        r.py[k] = Y;
    }
    const int sx = x86_int(floorf(smin(r.px[0], smin(r.px[1], r.px[2]))));
    const int sy = x86_int(floorf(smin(r.py[0], smin(r.py[1], r.py[2]))));
    const int ex = x86_int(ceilf(smax(r.px[0], smax(r.px[1], r.px[2]))));
    const int ey = x86_int(ceilf(smax(r.py[0], smax(r.py[1], r.py[2]))));
    const int W = (int)c.width, H = (int)c.height;
    if (ex < 0 || sx > W || ey < 0 || sy > H) return false;
    r.x0 = min(max(sx, 0), W); r.y0 = min(max(sy, 0), H);
    r.x1 = min(max(ex, 0), W); r.y1 = min(max(ey, 0), H);
#pragma unroll
    for (int k = 0; k < 3; ++k) r.d[k] = length(r.vc[k]);
    // edgeFunction(p0, p1, p2) (triangle.ipp:90-93)
    r.area = (r.px[2] - r.px[0]) * (r.py[1] - r.py[0]) - (r.py[2] - r.py[0]) * (r.px[1] - r.px[0]);
    return true;
}

// Barycentric weights at the pixel corner (X, Y), the inside test and the interpolated distance
// (cpu_rasterizer.ipp:132-146).
__device__ __forceinline__ bool raster_w(const RTri& r, int X, int Y, float* w, float& depth) {
    const float fx = (float)X, fy = (float)Y;
    w[0] = ((fx - r.px[1]) * (r.py[2] - r.py[1]) - (fy - r.py[1]) * (r.px[2] - r.px[1])) / r.area;
    w[1] = ((fx - r.px[2]) * (r.py[0] - r.py[2]) - (fy - r.py[2]) * (r.px[0] - r.px[2])) / r.area;
    w[2] = ((fx - r.px[0]) * (r.py[1] - r.py[0]) - (fy - r.py[0]) * (r.px[1] - r.px[0])) / r.area;
    if (!(w[0] >= 0 && w[1] >= 0 && w[2] >= 0)) return false;
    depth = ((w[0] * r.d[0]) + (w[1] * r.d[1])) + (w[2] * r.d[2]);
    return true;
}

// Closest fragment per pixel: the smallest (distance, triangle) pair, which is what the
// reference's in-order `current < previous` leaves (only finite distances ever pass it).
__device__ __forceinline__ void raster_fragment(unsigned long long* keys, uint32_t W, int X, int Y, float depth,
                                                uint32_t t) {
    if (!(depth < __int_as_float(0x7f800000))) return;
    const uint32_t bits = depth == 0.f ? 0u : __float_as_uint(depth);
    atomicMin(&keys[(size_t)Y * W + X], ((unsigned long long)bits << 32) | t);
}

constexpr uint32_t kRasterSmall = 256;   // box pixels a thread walks by itself

__global__ void k_raster_cover(DevScene s, RasterParams rp, uint32_t ntris, unsigned long long* __restrict__ keys,
                               uint32_t* __restrict__ bigq, uint32_t* __restrict__ nbig) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < ntris; t += (size_t)gridDim.x * blockDim.x) {
        RTri r;
        if (!raster_setup(s, rp, (uint32_t)t, r)) continue;
        const uint64_t npix = (uint64_t)(r.x1 - r.x0) * (uint64_t)(r.y1 - r.y0);
        if (npix == 0) continue;
        if (npix > kRasterSmall) { bigq[atomicAdd(nbig, 1u)] = (uint32_t)t; continue; }
        for (int X = r.x0; X < r.x1; ++X)
            for (int Y = r.y0; Y < r.y1; ++Y) {
                float w[3], depth;
                if (raster_w(r, X, Y, w, depth)) raster_fragment(keys, rp.cam.width, X, Y, depth, (uint32_t)t);
            }
    }
}

// Triangles with large boxes: one block per triangle, the box's pixels spread over its threads.
__global__ void k_raster_big(DevScene s, RasterParams rp, const uint32_t* __restrict__ bigq,
                             const uint32_t* __restrict__ nbig, unsigned long long* __restrict__ keys) {
    const uint32_t n = *nbig;
    for (uint32_t q = blockIdx.x; q < n; q += gridDim.x) {
        const uint32_t t = bigq[q];
        RTri r;
        if (!raster_setup(s, rp, t, r)) continue;
        const uint64_t ww = (uint64_t)(r.x1 - r.x0), npix = ww * (uint64_t)(r.y1 - r.y0);
        for (uint64_t k = threadIdx.x; k < npix; k += blockDim.x) {
            const int X = r.x0 + (int)(k % ww), Y = r.y0 + (int)(k / ww);
            float w[3], depth;
            if (raster_w(r, X, Y, w, depth)) raster_fragment(keys, rp.cam.width, X, Y, depth, t);
        }
    }
}

struct RasterOut {
    float *depth, *alpha, *albedo, *normal, *total, *direct, *indirect, *power;
    uint32_t* tri;
    const float* omega;
    float *tsz, *vel_g, *vel_c;   // first-fragment passes (null when not requested)
};

// The winner's passes (cpu_rasterizer.ipp:148-250, passes.ipp:80-128): the fragment is
// recomputed from its triangle with the same arithmetic as the coverage pass.
__global__ void k_raster_resolve(DevScene s, RasterParams rp, const unsigned long long* __restrict__ keys,
                                 RasterOut o) {
    const uint32_t W = rp.cam.width, H = rp.cam.height, nb = rp.nb;
    const size_t P = (size_t)W * H;
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < P; v += (size_t)gridDim.x * blockDim.x) {
        const unsigned long long key = keys[v];
        float depth = __int_as_float(0x7f800000), alpha = 0.f;
        float alb[VGB_MAX_BANDS], rad[VGB_MAX_BANDS];
#pragma unroll
        for (int k = 0; k < VGB_MAX_BANDS; ++k) { alb[k] = 0.f; rad[k] = 0.f; }
        F3 N{0.f, 0.f, 0.f};
        uint32_t tri = VGB_NO_HIT;
        RTri r;
        float w[3];
        const uint32_t t = (uint32_t)(key & 0xFFFFFFFFull);
        if (key != ~0ull && raster_setup(s, rp, t, r) && raster_w(r, (int)(v % W), (int)(v / W), w, depth)) {
            const uint32_t vi[3] = {__ldg(&s.idx[3 * (size_t)t]), __ldg(&s.idx[3 * (size_t)t + 1]),
                                    __ldg(&s.idx[3 * (size_t)t + 2])};
            F3 vp[3];
#pragma unroll
            for (int k = 0; k < 3; ++k) vp[k] = ld3(__ldg(&s.vpos[vi[k]]));
            const float2 u0 = __ldg(&s.vuv[vi[0]]), u1 = __ldg(&s.vuv[vi[1]]), u2 = __ldg(&s.vuv[vi[2]]);
            const float uvx = (w[0] * u0.x + w[1] * u1.x) + w[2] * u2.x;
            const float uvy = (w[0] * u0.y + w[1] * u1.y) + w[2] * u2.y;
            float texv[VGB_MAX_BANDS];
            sample_uvs<VGB_MAX_BANDS>(s, nb, uvx, uvy, texv);
#pragma unroll
            for (int k = 0; k < VGB_MAX_BANDS; ++k) {
                if (k >= (int)nb) break;
                float va;
                if (s.albedo_uniform) {
                    const float cst = s.albedo_value[k];
                    va = (w[0] * cst + w[1] * cst) + w[2] * cst;
                } else {
                    va = (w[0] * __ldg(&s.valb[(size_t)vi[0] * nb + k]) + w[1] * __ldg(&s.valb[(size_t)vi[1] * nb + k])) +
                         w[2] * __ldg(&s.valb[(size_t)vi[2] * nb + k]);
                }
                alb[k] = va * texv[k];
            }
            // Triangle::init's face normal -normalize((v0 - v1) x (v2 - v0)), or the smooth normal
            const F3 fn = normalize(cross(vp[0] - vp[1], vp[2] - vp[0]));
            N = F3{-fn.x, -fn.y, -fn.z};
            if (rp.smooth) {
                F3 vn[3];
#pragma unroll
                for (int k = 0; k < 3; ++k) vn[k] = ld3(__ldg(&s.vnrm[vi[k]]));
                N = normalize((w[0] * vn[0] + w[1] * vn[1]) + w[2] * vn[2]);
            }
            if (s.nmap) {   // the tangent frame and Material::getNormal (cpu_rasterizer.ipp:177-191)
                F3 tg, bt;
                tangent_frame(N, tg, bt);
                N = mapped_normal(s, uvx, uvy, N, tg, bt);
            }
            // the fragment's scene position: camera-frame corners interpolated with the screen-space
            // weights, then R p + origin (camera.localToGlobal)
            const F3 fc = (w[0] * r.vc[0] + w[1] * r.vc[1]) + w[2] * r.vc[2];
            const vgb_camera& c = rp.cam;
            const F3 fg{((c.rotation[0] * fc.x + c.rotation[3] * fc.y) + c.rotation[6] * fc.z) + c.origin[0],
                        ((c.rotation[1] * fc.x + c.rotation[4] * fc.y) + c.rotation[7] * fc.z) + c.origin[1],
                        ((c.rotation[2] * fc.x + c.rotation[5] * fc.y) + c.rotation[8] * fc.z) + c.origin[2]};
            if (o.tsz) {
                // the longest projected edge in pixels (cpu_rasterizer.ipp:123-129)
                const float e01 = sqrtf((r.px[1] - r.px[0]) * (r.px[1] - r.px[0]) + (r.py[1] - r.py[0]) * (r.py[1] - r.py[0]));
                const float e02 = sqrtf((r.px[2] - r.px[0]) * (r.px[2] - r.px[0]) + (r.py[2] - r.py[0]) * (r.py[2] - r.py[0]));
                const float e12 = sqrtf((r.px[2] - r.px[1]) * (r.px[2] - r.px[1]) + (r.py[2] - r.py[1]) * (r.py[2] - r.py[1]));
                o.tsz[v] = smax(e01, smax(e02, e12));
            }
            // the instance's and the camera's point velocities at the fragment (:211-218), as the
            // path tracer's first hit computes them
            if (o.vel_g || o.vel_c) first_hit_passes(s, c, t, fg, o.vel_g, o.vel_c, nullptr, P, (uint32_t)v);
            if (rp.lighting) {
                for (uint32_t l = 0; l < rp.nlights; ++l) {
                    F3 L;
                    float dist, pdf;
                    light_sample(rp.lights[l], fg, true, 0.f, 0.f, L, dist, pdf);
                    const float nl = smax(dot(N, L), 0.f);
#pragma unroll
                    for (int k = 0; k < VGB_MAX_BANDS; ++k) {
                        if (k >= (int)nb) break;
                        const float bsdf = ((alb[k] * kInvPi) * nl) / pdf;   // Lambertian::evaluateBSDF / pdf
                        rad[k] = rad[k] + rp.lights[l].radiance[k] * bsdf;
                    }
                }
            }
            alpha = __int_as_float(0x7f800000);   // count / sample with sample = 0: 1/0
            tri = t + 1u;
        } else {
            depth = __int_as_float(0x7f800000);
            // DataPayload's defaults where no fragment was drawn
            if (o.tsz) o.tsz[v] = __int_as_float(0x7f800000);
            if (o.vel_g) { o.vel_g[v] = 0.f; o.vel_g[P + v] = 0.f; o.vel_g[2 * P + v] = 0.f; }
            if (o.vel_c) { o.vel_c[v] = 0.f; o.vel_c[P + v] = 0.f; o.vel_c[2 * P + v] = 0.f; }
        }
        if (o.depth) o.depth[v] = depth;
        if (o.alpha) o.alpha[v] = alpha;
        if (o.tri) o.tri[v] = tri;
        if (o.normal) { o.normal[v] = N.x; o.normal[P + v] = N.y; o.normal[2 * P + v] = N.z; }
        for (uint32_t k = 0; k < nb; ++k) {
            if (o.albedo) o.albedo[k * P + v] = alb[k];
            if (o.total) o.total[k * P + v] = rad[k];
            if (o.direct) o.direct[k * P + v] = 0.f;
            if (o.indirect) o.indirect[k * P + v] = 0.f;
            if (o.power) o.power[k * P + v] = (rp.cam.power_scale[k] * o.omega[v]) * rad[k];
        }
    }
}

}  // namespace

VGB_API vgb_status vgb_rasterize(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights, uint32_t nlights,
                                 const vgb_raster_options* opts, vgb_film* film) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!cam || !opts || !film) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "rasterize: null argument");
    if (ctx->ntris == 0) return fail(ctx, VGB_ERR_NOT_READY, "rasterize: no scene uploaded");
    if (cam->width == 0 || cam->height == 0) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "rasterize: empty image");
    if ((uint64_t)cam->width * cam->height >= (1ull << 32))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "rasterize: image larger than 2^32 pixels");
    if (opts->nbands != ctx->nbands) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "rasterize: nbands differs from the scene's");
    if (nlights > VGB_MAX_LIGHTS || (nlights && !lights))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "rasterize: 0..8 lights");
    if (film->received_power && !film->pixel_solid_angle)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "rasterize: received_power needs pixel_solid_angle");
    cudaSetDevice(ctx->device);
    const size_t P = (size_t)cam->width * cam->height, B = ctx->nbands;
    RasterParams rp{};
    rp.cam = *cam;
    for (int k = 0; k < 6; ++k) rp.K[k] = opts->intrinsic[k];
    for (uint32_t l = 0; l < nlights; ++l) rp.lights[l] = lights[l];
    rp.nlights = opts->simulate_lighting ? nlights : 0;
    rp.nb = (uint32_t)B;
    rp.smooth = opts->smooth_shading ? 1u : 0u;
    rp.lighting = opts->simulate_lighting ? 1u : 0u;
    // scratch: keys (P x 8 B), big-triangle queue and its count
    const size_t key_floats = 2 * P, q_floats = (size_t)ctx->ntris + 4;
    // host film: every plane staged on the device (albedo and the four radiance planes of B bands;
    // depth, alpha, triangle id, triangle size, the pixel solid angle and three 3-vector planes),
    // each rounded up to 4 floats
    const size_t host_planes = film->on_device ? 0 : (size_t)(5 * B + 14) * P + 4 * 13;
    vgb_status s;
    if ((s = ensure_dn_scratch(ctx, key_floats + q_floats + host_planes)) != VGB_OK) return s;
    unsigned long long* keys = reinterpret_cast<unsigned long long*>(ctx->d_dn);
    uint32_t* bigq = reinterpret_cast<uint32_t*>(ctx->d_dn + key_floats);
    uint32_t* nbig = bigq + ctx->ntris;
    RasterOut o{film->depth, film->alpha, film->albedo, film->normal_global, film->total_radiance,
                film->direct_radiance, film->indirect_radiance, film->received_power, film->triangle_id,
                film->pixel_solid_angle, film->triangle_size, film->velocity_global, film->velocity_camera};
    if (!rp.lighting) o.total = o.direct = o.indirect = o.power = nullptr;
    float* stage = ctx->d_dn + key_floats + q_floats;
    if (!film->on_device) {
        // host film: device planes in scratch, copied back below
        auto take = [&](float* hp, size_t n) -> float* { if (!hp) return nullptr; float* d = stage; stage += (n + 3) & ~(size_t)3; return d; };
        o.depth = take(film->depth, P); o.alpha = take(film->alpha, P); o.albedo = take(film->albedo, B * P);
        o.normal = take(film->normal_global, 3 * P);
        o.tri = reinterpret_cast<uint32_t*>(take(reinterpret_cast<float*>(film->triangle_id), P));
        o.tsz = take(film->triangle_size, P);
        o.vel_g = take(film->velocity_global, 3 * P);
        o.vel_c = take(film->velocity_camera, 3 * P);
        if (rp.lighting) {
            o.total = take(film->total_radiance, B * P); o.direct = take(film->direct_radiance, B * P);
            o.indirect = take(film->indirect_radiance, B * P); o.power = take(film->received_power, B * P);
            float* om = take(const_cast<float*>(film->pixel_solid_angle), P);
            if (om) {
                CK(cudaMemcpyAsync(om, film->pixel_solid_angle, P * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
                o.omega = om;
            }
        }
    }
    const DevScene sc = dev_scene(ctx);
    CK(cudaMemsetAsync(keys, 0xFF, P * sizeof(unsigned long long), ctx->stream));
    CK(cudaMemsetAsync(nbig, 0, sizeof(uint32_t), ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    k_raster_cover<<<grid_for(ctx, ctx->ntris, 8), 256, 0, ctx->stream>>>(sc, rp, ctx->ntris, keys, bigq, nbig);
    k_raster_big<<<ctx->num_sms * 4, 256, 0, ctx->stream>>>(sc, rp, bigq, nbig, keys);
    k_raster_resolve<<<grid_for(ctx, P, 8), 256, 0, ctx->stream>>>(sc, rp, keys, o);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    if (!film->on_device) {
        auto back = [&](void* hp, const void* dp, size_t bytes) -> cudaError_t {
            return (hp && dp) ? cudaMemcpyAsync(hp, dp, bytes, cudaMemcpyDeviceToHost, ctx->stream) : cudaSuccess;
        };
        CK(back(film->depth, o.depth, P * 4)); CK(back(film->alpha, o.alpha, P * 4));
        CK(back(film->albedo, o.albedo, B * P * 4)); CK(back(film->normal_global, o.normal, 3 * P * 4));
        CK(back(film->triangle_id, o.tri, P * 4));
        CK(back(film->triangle_size, o.tsz, P * 4));
        CK(back(film->velocity_global, o.vel_g, 3 * P * 4));
        CK(back(film->velocity_camera, o.vel_c, 3 * P * 4));
        if (rp.lighting) {
            CK(back(film->total_radiance, o.total, B * P * 4)); CK(back(film->direct_radiance, o.direct, B * P * 4));
            CK(back(film->indirect_radiance, o.indirect, B * P * 4)); CK(back(film->received_power, o.power, B * P * 4));
        }
    }
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.ms_last = ms;
    ctx->stats.kernel_launches = 3;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

// DEMQuipu::readBuffers (dem_quipu.ipp:124-221): the file's stored codes are read and LZ4-decoded
// on the host into pinned memory, copied to the device as stored (1-4 bytes per post), and
// decoded, posed (DEM::makeVertexBuffer), triangulated (imageToIndexBuffer) and given vertex
// normals (Mesh::calculateNormals) there.
VGB_API vgb_status vgb_quipu_read_mesh(vgb_context* ctx, vgb_quipu_dem* q, uint32_t lod,
                                       const vgb_quipu_read_options* opts, float* positions, float* vert_albedo,
                                       float* normals, uint32_t* indices, uint32_t* ntris, int on_device) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!q || !opts || !positions || !indices || !ntris)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "quipu_read_mesh: null argument");
    if (vert_albedo && (opts->nbands == 0 || opts->nbands > VGB_MAX_BANDS))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "quipu_read_mesh: nbands must be 1..8");
    vgb::QuipuPayload pl;
    if (vgb::quipu_lod_payload(q, lod, &pl) != VGB_OK)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, std::string("quipu_read_mesh: ") + vgb_quipu_last_error());
    if (pl.proj.is_ogr)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "quipu_read_mesh: map-projected (OGR) LoDs need GDAL, which is absent");
    const uint32_t W = pl.heights.w, H = pl.heights.h;
    if (W < 2 || H < 2) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "quipu_read_mesh: fewer than 2x2 posts");
    // triangle ids and vertex indices are 32-bit, and VGB_NO_HIT (2^32 - 1) marks a miss
    if ((uint64_t)W * H >= (1ull << 31))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "quipu_read_mesh: LoD of 2^31 posts or more (32-bit triangle ids)");
    const size_t nv = (size_t)W * H, nq = (size_t)(W - 1) * (H - 1);
    const uint32_t nb = vert_albedo ? opts->nbands : 0;
    const bool use_albedo = vert_albedo && opts->read_albedos && pl.albedo_type != VGB_QUIPU_NO_ALBEDO;
    if (use_albedo && pl.albedo_type == 2 && pl.planes.size() != nb)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "quipu_read_mesh: the file's albedo has " +
                    std::to_string(pl.planes.size()) + " channels, the reader " + std::to_string(nb) + " bands");
    // host: stored codes and albedo planes into pinned staging
    const size_t code_bytes = (pl.heights.raw_bytes + 15) & ~(size_t)15;
    const size_t plane_bytes = use_albedo && pl.albedo_type != 0 ? pl.planes.size() * nv : 0;
    const size_t pin_need = code_bytes + ((plane_bytes + 15) & ~(size_t)15);
    cudaSetDevice(ctx->device);
    CK(cudaStreamSynchronize(ctx->stream));
    if (pin_need > ctx->cap_pin) {
        if (ctx->h_pin) cudaFreeHost(ctx->h_pin);
        ctx->h_pin = nullptr;
        ctx->cap_pin = 0;
        CK(cudaMallocHost(&ctx->h_pin, pin_need));
        ctx->cap_pin = pin_need;
    }
    uint8_t* hp = (uint8_t*)ctx->h_pin;
    {
        // every image is its own LZ4 block: the heights and the albedo planes decode in parallel
        const size_t nimg = 1 + (plane_bytes ? pl.planes.size() : 0);
        std::vector<std::string> errs(nimg);
        vgb::parallel_for_each((uint32_t)nimg, [&](uint32_t k) {
            const vgb::ImageRefView& img = k == 0 ? pl.heights : pl.planes[k - 1].img;
            uint8_t* dst = k == 0 ? hp : hp + code_bytes + (k - 1) * nv;
            if (vgb::quipu_read_pixels(pl.path, img, dst) != VGB_OK) errs[k] = vgb_quipu_last_error();
        });
        for (const std::string& e : errs)
            if (!e.empty()) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "quipu_read_mesh: " + e);
    }
    vgb::QuipuDecode d{};
    d.W = W; d.H = H; d.precision = pl.precision; d.nbands = nb;
    d.hmin = pl.hmin; d.hmax = pl.hmax;
    d.albedo_type = use_albedo ? pl.albedo_type : VGB_QUIPU_NO_ALBEDO;
    d.nplanes = (uint32_t)(plane_bytes ? pl.planes.size() : 0);
    for (uint32_t b = 0; b < VGB_MAX_BANDS; ++b) {
        d.constant[b] = opts->default_albedo;
        d.profile[b] = opts->albedo_profile[b];
    }
    for (uint32_t c = 0; c < d.nplanes && c < VGB_MAX_BANDS; ++c) { d.pmin[c] = pl.planes[c].mn; d.pmax[c] = pl.planes[c].mx; }
    if (use_albedo && pl.albedo_type == 0 && nb) {
        float cst[VGB_MAX_BANDS];
        if (vgb::quipu_read_constant(pl.path, pl.constant_pos, nb, cst) != VGB_OK)
            return fail(ctx, VGB_ERR_INVALID_ARGUMENT, std::string("quipu_read_mesh: ") + vgb_quipu_last_error());
        for (uint32_t b = 0; b < nb; ++b) d.constant[b] = cst[b];
    }
    // device scratch (floats): codes | planes | heights | triangulation work | normals work |
    // output staging when the caller's arrays are on the host
    // every section starts on a 16-byte boundary (4 floats)
    auto al4 = [](size_t f) { return (f + 3) & ~(size_t)3; };
    const size_t f_codes = code_bytes / 4, f_planes = ((plane_bytes + 15) & ~(size_t)15) / 4;
    const size_t f_work = al4(vgb::dem_work_words(W, H));
    const size_t f_out = on_device ? 0 : al4(3 * nv) + al4((size_t)nb * nv) + (normals ? al4(3 * nv) : 0) + 6 * nq;
    vgb_status s;
    if ((s = ensure_dn_scratch(ctx, f_codes + f_planes + al4(nv) + f_work + f_out)) != VGB_OK) return s;
    float* cur = ctx->d_dn;
    void* d_codes = cur; cur += f_codes;
    uint8_t* d_planes = (uint8_t*)cur; cur += f_planes;
    float* d_h = cur; cur += al4(nv);
    uint32_t* d_work = (uint32_t*)cur; cur += f_work;
    float* p = positions;
    float* a = vert_albedo;
    float* nr = normals;
    uint32_t* ix = indices;
    if (!on_device) {
        p = cur; cur += al4(3 * nv);
        if (nb) { a = cur; cur += al4((size_t)nb * nv); }
        if (normals) { nr = cur; cur += al4(3 * nv); }
        ix = (uint32_t*)cur;
    }
    CK(cudaMemcpyAsync(d_codes, hp, pl.heights.raw_bytes, cudaMemcpyHostToDevice, ctx->stream));
    if (plane_bytes) CK(cudaMemcpyAsync(d_planes, hp + code_bytes, plane_bytes, cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    CK((cudaError_t)vgb::launch_quipu_decode(ctx->stream, ctx->num_sms, d, d_codes, d_planes, d_h, nb ? a : nullptr));
    uint32_t nt = 0;
    // normals from the grid's structure (the same sums launch_vertex_normals forms on these arrays)
    CK((cudaError_t)vgb::launch_dem_triangulate(ctx->stream, ctx->num_sms, d_h, W, H, vgb::dem_pose(pl.proj), p, ix,
                                                d_work, &nt, normals ? nr : nullptr));
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    if (!on_device) {
        CK(cudaMemcpyAsync(positions, p, 3 * nv * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        if (nb) CK(cudaMemcpyAsync(vert_albedo, a, (size_t)nb * nv * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        if (normals) CK(cudaMemcpyAsync(normals, nr, 3 * nv * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(indices, ix, 3 * (size_t)nt * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    ctx->stats.ms_last = ms;   // device decode + triangulation + normals
    *ntris = nt;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_sensor_simulate(vgb_context* ctx, const float* received_power, uint32_t width,
                                       uint32_t height, uint32_t nbands, const vgb_sensor* sensor, float* image,
                                       int on_device) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!received_power || !sensor || !image || width == 0 || height == 0 || nbands == 0 || nbands > VGB_MAX_BANDS)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "sensor_simulate: null plane or sensor, empty image or bands outside 1..8");
    if (!(sensor->max_adu > 0.f)) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "sensor_simulate: max_adu must be > 0");
    for (uint32_t k = 0; k < nbands; ++k)
        if (!(sensor->photon_energy[k] > 0.f))
            return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "sensor_simulate: photon energies must be > 0");
    cudaSetDevice(ctx->device);
    const size_t P = (size_t)width * height, BP = (size_t)nbands * P;
    vgb::SensorParams sp{};
    sp.exposure_time = sensor->exposure_time;
    for (int k = 0; k < 8; ++k) { sp.photon_energy[k] = sensor->photon_energy[k]; sp.quantum_efficiency[k] = sensor->quantum_efficiency[k]; }
    sp.gain = sensor->gain; sp.max_adu = sensor->max_adu;
    sp.photon_noise = sensor->simulate_photon_noise; sp.noise_model = sensor->noise_model;
    sp.dark_current = sensor->dark_current; sp.readout_mean = sensor->readout_noise_mean; sp.readout_std = sensor->readout_noise_std;
    sp.hscale = sensor->horizontal_scale; sp.vscale = sensor->vertical_scale;
    sp.hperiod = sensor->horizontal_pattern_period; sp.vperiod = sensor->vertical_pattern_period;
    sp.frame = sensor->frame; sp.seed = sensor->seed; sp.mosaic = sensor->filter_mosaic;
    const float* pw = received_power;
    float* img = image;
    vgb_status s;
    if (!on_device) {
        if ((s = ensure_staging(ctx, (BP * (sensor->filter_mosaic ? 2 : 1) + P) * sizeof(float))) != VGB_OK) return s;
        float* cur = (float*)ctx->staging_base;
        CK(cudaMemcpyAsync(cur, received_power, BP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); pw = cur; cur += BP;
        if (sensor->filter_mosaic) {
            CK(cudaMemcpyAsync(cur, sensor->filter_mosaic, BP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
            sp.mosaic = cur; cur += BP;
        }
        img = cur;
    }
    CK((cudaError_t)vgb::launch_sensor(ctx->stream, pw, width, height, nbands, sp, img, ctx->num_sms));
    if (!on_device) CK(cudaMemcpyAsync(image, img, P * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_sensor_simulate_rgb(vgb_context* ctx, const float* received_power, uint32_t width,
                                           uint32_t height, uint32_t nbands, const vgb_sensor* sensor,
                                           const vgb_rgb_conversion* rgb, float* image_rgb, int on_device) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!received_power || !sensor || !rgb || !image_rgb || width == 0 || height == 0 || nbands == 0 ||
        nbands > VGB_MAX_BANDS || (uint64_t)width * height > (1ull << 31))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "sensor_simulate_rgb: null plane, sensor or conversion, bad size or bands outside 1..8");
    if (!(sensor->max_adu > 0.f)) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "sensor_simulate_rgb: max_adu must be > 0");
    for (int c = 0; c < 3; ++c)
        if (!(rgb->rgb_photon_energy[c] > 0.f) || !(rgb->rgb_bandwidth[c] > 0.f))
            return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "sensor_simulate_rgb: RGB photon energies and bandwidths must be > 0");
    cudaSetDevice(ctx->device);
    const size_t P = (size_t)width * height, BP = (size_t)nbands * P;
    vgb::SensorParams sp{};
    sp.exposure_time = sensor->exposure_time;
    sp.gain = sensor->gain; sp.max_adu = sensor->max_adu;
    sp.photon_noise = sensor->simulate_photon_noise; sp.noise_model = sensor->noise_model;
    sp.dark_current = sensor->dark_current; sp.readout_mean = sensor->readout_noise_mean; sp.readout_std = sensor->readout_noise_std;
    sp.hscale = sensor->horizontal_scale; sp.vscale = sensor->vertical_scale;
    sp.hperiod = sensor->horizontal_pattern_period; sp.vperiod = sensor->vertical_pattern_period;
    sp.frame = sensor->frame; sp.seed = sensor->seed; sp.mosaic = sensor->filter_mosaic;
    vgb::RgbParams rp{};
    for (int k = 0; k < 8; ++k) { rp.band_min[k] = rgb->band_min[k]; rp.band_max[k] = rgb->band_max[k]; }
    for (int c = 0; c < 3; ++c) {
        rp.rgb_min[c] = rgb->rgb_min[c]; rp.rgb_max[c] = rgb->rgb_max[c]; rp.rgb_bw[c] = rgb->rgb_bandwidth[c];
        rp.rgb_pe[c] = rgb->rgb_photon_energy[c]; rp.rgb_qe[c] = rgb->rgb_quantum_efficiency[c];
    }
    const float* pw = received_power;
    float* img = image_rgb;
    vgb_status s;
    if (!on_device) {
        if ((s = ensure_staging(ctx, (BP * (sensor->filter_mosaic ? 2 : 1) + 3 * P) * sizeof(float))) != VGB_OK) return s;
        float* cur = (float*)ctx->staging_base;
        CK(cudaMemcpyAsync(cur, received_power, BP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); pw = cur; cur += BP;
        if (sensor->filter_mosaic) {
            CK(cudaMemcpyAsync(cur, sensor->filter_mosaic, BP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
            sp.mosaic = cur; cur += BP;
        }
        img = cur;
    }
    CK((cudaError_t)vgb::launch_sensor_rgb(ctx->stream, pw, width, height, nbands, sp, rp, img, ctx->num_sms));
    if (!on_device) CK(cudaMemcpyAsync(image_rgb, img, 3 * P * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_psf_convolve(vgb_context* ctx, float* received_power, uint32_t width, uint32_t height,
                                    uint32_t nbands, const float* kernel, uint32_t kernel_w, uint32_t kernel_h,
                                    int on_device) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!received_power || !kernel || width == 0 || height == 0 || nbands == 0 || nbands > VGB_MAX_BANDS)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "psf_convolve: null plane or kernel, empty image or bands outside 1..8");
    if (kernel_w == 0 || kernel_h == 0 || kernel_w > 127 || kernel_h > 127)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "psf_convolve: kernel sides must be 1..127");
    cudaSetDevice(ctx->device);
    const size_t P = (size_t)width * height, BP = (size_t)nbands * P, KN = (size_t)nbands * kernel_w * kernel_h;
    vgb_status s;
    if ((s = ensure_dn_scratch(ctx, BP + (on_device ? 0 : BP + KN))) != VGB_OK) return s;
    float* out = ctx->d_dn;
    float* io = received_power;
    const float* kr = kernel;
    if (!on_device) {
        float* cur = ctx->d_dn + BP;
        CK(cudaMemcpyAsync(cur, received_power, BP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); io = cur; cur += BP;
        CK(cudaMemcpyAsync(cur, kernel, KN * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); kr = cur;
    }
    CK((cudaError_t)vgb::launch_psf(ctx->stream, io, out, width, height, nbands, kr, kernel_w, kernel_h));
    CK(cudaMemcpyAsync(on_device ? received_power : io, out, BP * sizeof(float), cudaMemcpyDeviceToDevice, ctx->stream));
    if (!on_device) CK(cudaMemcpyAsync(received_power, io, BP * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_denoise(vgb_context* ctx, float* direct, float* indirect, const float* albedo,
                               const float* depth, const float* normal, uint32_t width, uint32_t height,
                               uint32_t nbands, const vgb_denoise_options* o, int on_device) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!direct || !indirect || !albedo || !depth || !normal || width == 0 || height == 0 || nbands == 0 ||
        nbands > VGB_MAX_BANDS)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "denoise: null plane, empty image or bands outside 1..8");
    cudaSetDevice(ctx->device);
    const size_t P = (size_t)width * height, BP = (size_t)nbands * P;
    vgb_status s;
    const size_t work = dn_work_floats(nbands, P);
    if ((s = ensure_dn_scratch(ctx, work + (on_device ? 0 : 3 * BP + 4 * P))) != VGB_OK) return s;
    float *d = direct, *i = indirect;
    const float *a = albedo, *z = depth, *n = normal;
    if (!on_device) {
        float* cur = ctx->d_dn + work;
        CK(cudaMemcpyAsync(cur, direct, BP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); d = cur; cur += BP;
        CK(cudaMemcpyAsync(cur, indirect, BP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); i = cur; cur += BP;
        CK(cudaMemcpyAsync(cur, albedo, BP * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); a = cur; cur += BP;
        CK(cudaMemcpyAsync(cur, depth, P * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); z = cur; cur += P;
        CK(cudaMemcpyAsync(cur, normal, 3 * P * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); n = cur;
    }
    launch_denoise(ctx, d, i, a, z, n, width, height, nbands, dn_opts(o), ctx->d_dn, d, i, nullptr, nullptr, nullptr,
                   PowerScale{});
    CK(cudaGetLastError());
    if (!on_device) {
        CK(cudaMemcpyAsync(direct, d, BP * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        CK(cudaMemcpyAsync(indirect, i, BP * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_get_stats(vgb_context* ctx, vgb_stats* out) try {
    if (!ctx || !out) return VGB_ERR_INVALID_ARGUMENT;
    *out = ctx->stats;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

static vgb_status check_device_error(vgb_context* ctx) {
    uint32_t e = 0;
    CK(cudaMemcpy(&e, &ctx->d_counters[C_ERR], sizeof(uint32_t), cudaMemcpyDeviceToHost));
    ctx->stats.device_error = e;
    if (e) {
        CK(cudaMemset(&ctx->d_counters[C_ERR], 0, sizeof(uint32_t)));
        return fail(ctx, VGB_ERR_DEVICE_LIMIT,
                    std::string("device traversal limit hit:") + ((e & kErrStack) ? " stack" : "") +
                        ((e & kErrIter) ? " iterations" : ""));
    }
    return VGB_OK;
}

VGB_API vgb_status vgb_render(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights, uint32_t nlights,
                              const vgb_pt_options* opts, vgb_film* film) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!cam || !opts || !film) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render: null camera/options/film");
    if (!ctx->bvh_ready) return fail(ctx, VGB_ERR_NOT_READY, "render: build the BVH first");
    if (opts->samples == 0) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render: options.samples must be >= 1");
    if (opts->adaptive_sampling && (opts->samples_per_batch == 0 || opts->samples_to_detect_miss == 0))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render: adaptive sampling needs samples_per_batch and samples_to_detect_miss >= 1");
    if (opts->nbands != ctx->nbands) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render: nbands differs from the scene");
    if (nlights > VGB_MAX_LIGHTS || (nlights && !lights))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render: at most 8 lights");
    if (!frame_fits(cam->width, cam->height))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render: bad resolution");
    if (film->received_power && !film->pixel_solid_angle)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render: received_power needs pixel_solid_angle");
    cudaSetDevice(ctx->device);
    const size_t P = (size_t)cam->width * cam->height;
    const uint32_t B = ctx->nbands;
    vgb_status s = ensure_scratch(ctx, P, tile_items(cam->width, cam->height), B, std::max<uint32_t>(1, nlights));
    if (s != VGB_OK) return s;
    FrameParams fp;
    std::memset(&fp, 0, sizeof(fp));
    fp.cam = *cam;
    fp.opt = *opts;
    for (uint32_t l = 0; l < nlights; ++l) fp.lights[l] = lights[l];
    fp.nlights = nlights;
    fp.nb = B;
    fp.tiles_x = (cam->width + 7) / 8;
    fp.tiles_y = (cam->height + 3) / 4;
    // film planes: device pointers as given, or staging buffers for host films
    FilmOut f{};
    struct Plane { float** host_f; uint32_t** host_u; size_t n; };
    constexpr int NPL = 11;
    float* hf[NPL] = {film->total_radiance, film->direct_radiance, film->indirect_radiance, film->received_power,
                      film->albedo, film->normal_global, film->depth, film->alpha, film->velocity_global,
                      film->velocity_camera, film->triangle_size};
    const size_t nplane[NPL] = {B * P, B * P, B * P, B * P, B * P, 3 * P, P, P, 3 * P, 3 * P, P};
    float* df[NPL];
    uint32_t* dtri = film->triangle_id;
    const float* domega = film->pixel_solid_angle;
    bool staged[NPL] = {false};
    bool tri_staged = false;
    if (film->on_device) {
        for (int k = 0; k < NPL; ++k) df[k] = hf[k];
    } else {
        // Host planes that the CUDA runtime reports as pinned and mapped (cudaHostAlloc or
        // cudaHostRegister memory) are written by the kernels through their device alias, across
        // the host link, with no device staging and no copy after the render; other host planes
        // are staged in device memory and copied back.
        float* mapped[NPL];
        size_t total = 0;
        for (int k = 0; k < NPL; ++k) {
            mapped[k] = static_cast<float*>(mapped_host(hf[k]));
            staged[k] = hf[k] && !mapped[k];
            if (staged[k]) total += nplane[k];
        }
        uint32_t* tri_mapped = static_cast<uint32_t*>(mapped_host(film->triangle_id));
        tri_staged = film->triangle_id && !tri_mapped;
        const float* omega_mapped = static_cast<const float*>(mapped_host(film->pixel_solid_angle));
        const bool omega_staged = film->pixel_solid_angle && !omega_mapped;
        total += (tri_staged ? P : 0) + (omega_staged ? P : 0);
        float* cur = nullptr;
        if (total) {
            if ((s = ensure_staging(ctx, total * sizeof(float))) != VGB_OK) return s;
            cur = (float*)ctx->staging_base;
        }
        for (int k = 0; k < NPL; ++k) {
            df[k] = staged[k] ? cur : mapped[k];
            if (staged[k]) cur += nplane[k];
        }
        dtri = tri_staged ? (uint32_t*)cur : tri_mapped;
        if (tri_staged) cur += P;
        domega = omega_mapped;
        if (omega_staged) {
            CK(cudaMemcpyAsync(cur, film->pixel_solid_angle, P * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
            domega = cur;
        }
    }
    f.total = df[0]; f.direct = df[1]; f.indirect = df[2]; f.power = df[3]; f.albedo = df[4];
    f.normal = df[5]; f.depth = df[6]; f.alpha = df[7]; f.tri = dtri; f.omega = domega;
    f.vel_g = df[8]; f.vel_c = df[9]; f.tsz = df[10];
    FilmOut fr = f;  // the planes the render itself writes
    float* dn_scratch = nullptr;
    if (opts->denoise) {
        // options.denoise (cpu_path_tracer.ipp:124-134): the render writes un-denoised direct and
        // indirect radiance (and albedo, depth and normal where the film has none) to scratch;
        // the denoiser then writes direct, indirect, total and received power to the film.
        const size_t work = dn_work_floats(B, P);
        if ((s = ensure_dn_scratch(ctx, work + (size_t)3 * B * P + 4 * P)) != VGB_OK) return s;
        dn_scratch = ctx->d_dn;
        float* extra = ctx->d_dn + work;
        fr.total = nullptr; fr.power = nullptr;
        fr.direct = extra; fr.indirect = extra + (size_t)B * P;
        if (!fr.albedo) fr.albedo = extra + (size_t)2 * B * P;
        if (!fr.normal) fr.normal = extra + (size_t)3 * B * P;
        if (!fr.depth) fr.depth = extra + (size_t)3 * B * P + 3 * P;
    }
    fp.aux = aux_for(fr) | (opts->adaptive_sampling ? AUX_DEP : 0u);  // the miss test reads the depth sum
    fp.vel_g = fr.vel_g; fp.vel_c = fr.vel_c; fp.tsz = fr.tsz;
    CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(uint64_t) * 8, ctx->stream));
    uint32_t launches = 0;
    ctx->prof_used = 0;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    dispatch_render<false>(ctx, fp, fr, ctx->st, true, launches);
    if (dn_scratch) {
        PowerScale ps{};
        for (uint32_t k = 0; k < B && k < VGB_MAX_BANDS; ++k) ps.v[k] = cam->power_scale[k];
        launch_denoise(ctx, fr.direct, fr.indirect, fr.albedo, fr.depth, fr.normal, cam->width, cam->height, B,
                       dn_opts(&opts->denoiser), dn_scratch, f.direct, f.indirect, f.total, f.power, f.omega, ps);
    }
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    if (!film->on_device) {
        for (int k = 0; k < NPL; ++k)
            if (staged[k]) CK(cudaMemcpyAsync(hf[k], df[k], nplane[k] * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        if (tri_staged) CK(cudaMemcpyAsync(film->triangle_id, dtri, P * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    uint64_t hs[8];
    CK(cudaMemcpy(hs, ctx->d_stats, sizeof(hs), cudaMemcpyDeviceToHost));
    ctx->stats.rays_closest = hs[2];
    ctx->stats.rays_shadow = hs[3];
    ctx->stats.hits_closest = hs[6];
    ctx->stats.kernel_launches = launches;
    ctx->stats.ms_last = ms;
    ctx->stats.nodes_visited = 0;
    ctx->stats.tris_tested = 0;
    ctx->stats.nodes_closest = 0;
    ctx->stats.tris_closest = 0;
    ctx->stats.ms_trace = ctx->stats.ms_shadow = ctx->stats.ms_film = ctx->stats.ms_shade = 0.f;
    ctx->stats.launches_trace = ctx->stats.launches_shadow = ctx->stats.launches_film = ctx->stats.launches_shade = 0;
    if (ctx->profiling) {
        float* fam_ms[4] = {&ctx->stats.ms_trace, &ctx->stats.ms_shadow, &ctx->stats.ms_film, &ctx->stats.ms_shade};
        uint32_t* fam_n[4] = {&ctx->stats.launches_trace, &ctx->stats.launches_shadow, &ctx->stats.launches_film,
                              &ctx->stats.launches_shade};
        for (size_t k = 0; k < ctx->prof_used; k += 2) {
            float e = 0.f;
            cudaEventElapsedTime(&e, ctx->prof_events[k], ctx->prof_events[k + 1]);
            const int fam = ctx->prof_family[k / 2];
            *fam_ms[fam] += e;
            *fam_n[fam] += 1;
        }
    }
    if ((s = check_device_error(ctx)) != VGB_OK) return s;
    if (ctx->count_pass) {
        // counting pass: same kernels with traversal counters, into scratch film planes
        FilmOut none{};
        none.omega = domega;
        none.power = nullptr;
        CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(uint64_t) * 8, ctx->stream));
        uint32_t l2 = 0;
        dispatch_render<true>(ctx, fp, none, ctx->st, false, l2);
        CK(cudaGetLastError());
        CK(cudaStreamSynchronize(ctx->stream));
        CK(cudaMemcpy(hs, ctx->d_stats, sizeof(hs), cudaMemcpyDeviceToHost));
        ctx->stats.nodes_visited = hs[0];
        ctx->stats.tris_tested = hs[1];
        ctx->stats.nodes_closest = hs[4];
        ctx->stats.tris_closest = hs[5];
        if ((s = check_device_error(ctx)) != VGB_OK) return s;
    }
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

VGB_API vgb_status vgb_trace_rays(vgb_context* ctx, const float* org, const float* dir, const float* tmax,
                                  uint32_t n, int any_hit, uint32_t* tri, float* tout, float* bary, int on_device) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!org || !dir || !tri) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "trace_rays: null buffer");
    if (!ctx->bvh_ready) return fail(ctx, VGB_ERR_NOT_READY, "trace_rays: build the BVH first");
    if (n == 0) return VGB_OK;
    cudaSetDevice(ctx->device);
    const float *dorg = org, *ddir = dir, *dtmax = tmax;
    uint32_t* dtri = tri;
    float *dt = tout, *db = bary;
    vgb_status s;
    // host buffers: pinned, mapped ones (cudaHostAlloc, cudaHostRegister) are read and written by
    // the kernel through their device address; the others are staged in device memory
    void* mp[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    if (!on_device) {
        const void* hb[6] = {org, dir, tmax, tri, tout, bary};
        const size_t words[6] = {3, 3, 1, 1, 1, 3};
        size_t need = 0;
        for (int k = 0; k < 6; ++k) {
            mp[k] = mapped_host(hb[k]);
            if (hb[k] && !mp[k]) need += words[k] * (size_t)n;
        }
        float* cur = nullptr;
        if (need) {
            if ((s = ensure_staging(ctx, need * 4)) != VGB_OK) return s;
            cur = (float*)ctx->staging_base;
        }
        void* dv[6];
        for (int k = 0; k < 6; ++k) {
            dv[k] = hb[k] ? (mp[k] ? mp[k] : (void*)cur) : nullptr;
            if (hb[k] && !mp[k]) cur += words[k] * (size_t)n;
        }
        for (int k = 0; k < 3; ++k)
            if (hb[k] && !mp[k])
                CK(cudaMemcpyAsync(dv[k], hb[k], 4 * words[k] * (size_t)n, cudaMemcpyHostToDevice, ctx->stream));
        dorg = (const float*)dv[0]; ddir = (const float*)dv[1]; dtmax = (const float*)dv[2];
        dtri = (uint32_t*)dv[3]; dt = (float*)dv[4]; db = (float*)dv[5];
    }
    const DevScene sc = dev_scene(ctx);
    CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(uint64_t) * 8, ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    const int g = grid_for(ctx, n, VGB_RAYS_GRID * 256 / VGB_RAYS_BLOCK, VGB_RAYS_BLOCK);
    auto launch = [&](auto lc) {
        constexpr int L = decltype(lc)::value;
        if (any_hit) {
            if (ctx->count_pass) k_trace_batch<L, true, true><<<g, VGB_RAYS_BLOCK, 0, ctx->stream>>>(sc, dorg, ddir, dtmax, n, dtri, dt, db, ctx->d_counters, ctx->d_stats);
            else k_trace_batch<L, true, false><<<g, VGB_RAYS_BLOCK, 0, ctx->stream>>>(sc, dorg, ddir, dtmax, n, dtri, dt, db, ctx->d_counters, ctx->d_stats);
        } else {
            if (ctx->count_pass) k_trace_batch<L, false, true><<<g, VGB_RAYS_BLOCK, 0, ctx->stream>>>(sc, dorg, ddir, dtmax, n, dtri, dt, db, ctx->d_counters, ctx->d_stats);
            else k_trace_batch<L, false, false><<<g, VGB_RAYS_BLOCK, 0, ctx->stream>>>(sc, dorg, ddir, dtmax, n, dtri, dt, db, ctx->d_counters, ctx->d_stats);
        }
    };
    if (ctx->bvh_layout == 8) launch(std::integral_constant<int, 8>{});
    else launch(std::integral_constant<int, 2>{});
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    if (!on_device) {
        if (!mp[3]) CK(cudaMemcpyAsync(tri, dtri, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
        if (tout && !mp[4]) CK(cudaMemcpyAsync(tout, dt, 4 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
        if (bary && !mp[5]) CK(cudaMemcpyAsync(bary, db, 12 * (size_t)n, cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    uint64_t hs[8];
    CK(cudaMemcpy(hs, ctx->d_stats, sizeof(hs), cudaMemcpyDeviceToHost));
    ctx->stats.ms_last = ms;
    ctx->stats.kernel_launches = 1;
    ctx->stats.nodes_visited = hs[0];
    ctx->stats.tris_tested = hs[1];
    ctx->stats.nodes_closest = hs[4];
    ctx->stats.tris_closest = hs[5];
    if (any_hit) { ctx->stats.rays_shadow = n; ctx->stats.rays_closest = 0; }
    else { ctx->stats.rays_closest = n; ctx->stats.rays_shadow = 0; }
    return check_device_error(ctx);
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

}  // extern "C"

// ====================================================================== render without allocation
// vgb_render_noalloc: the same launch sequence as vgb_render (launch_render), but every byte of
// its scratch (path state, live-path and shadow-ray queues, per-pixel accumulators, hit records,
// queue counters and the device error word) lives in one fixed device array that is part of this
// library image.  It exists for callers that must not allocate device memory once their scene is
// set up -- for example a frame loop with a fixed memory budget, or a host application whose own
// allocator owns the device, where a cudaMalloc inside a render call would synchronize the device
// or could fail.  The array is shared by every call on a device and keeps the previous call's
// contents.
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(8) << 20;  // 8 MiB per device
__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

inline size_t up256(size_t b) { return (b + 255) & ~size_t(255); }

// Bytes of the fixed array a frame of P pixels (n_items bounce-0 queue items), B bands and L
// lights needs.  With P and n_items at most 2^31 (frame_fits) and B, L at most 8, no term wraps.
size_t noalloc_bytes(size_t P, size_t n_items, size_t B, size_t L) {
    const size_t f = 4;
    size_t n = 2 * 256;  // counters, statistics
    const size_t planes[] = {3, 3, B, B, B, 1, B, B, B, 3, 1, 1, 1, 1, 1};
    for (size_t k : planes) n += up256(k * P * f);
    n += up256(n_items * sizeof(float4));  // hit records
    n += L * (up256(3 * P * f) + up256(3 * P * f) + up256(P * f) + up256(P * f) + up256(B * P * f));
    return n;
}

}  // namespace

extern "C" VGB_API vgb_status vgb_render_noalloc(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights,
                                                 uint32_t nlights, const vgb_pt_options* opts, vgb_film* film) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!cam || !opts || !film) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_noalloc: null camera/options/film");
    if (!ctx->bvh_ready) return fail(ctx, VGB_ERR_NOT_READY, "render_noalloc: build the BVH first");
    if (!film->on_device)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_noalloc: film planes must be device memory (on_device = 1)");
    if (opts->samples == 0) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_noalloc: options.samples must be >= 1");
    if (opts->adaptive_sampling || opts->denoise)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_noalloc: adaptive sampling and denoising keep per-pixel planes the fixed array has no room for; use vgb_render");
    if (opts->nbands != ctx->nbands)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_noalloc: nbands differs from the scene");
    if (nlights > VGB_MAX_LIGHTS || (nlights && !lights))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_noalloc: at most 8 lights");
    if (!frame_fits(cam->width, cam->height))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_noalloc: bad resolution");
    if (film->received_power && !film->pixel_solid_angle)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_noalloc: received_power needs pixel_solid_angle");
    const size_t P = (size_t)cam->width * cam->height;
    const size_t n_items = tile_items(cam->width, cam->height);
    const uint32_t B = ctx->nbands;
    const uint32_t nq = std::max<uint32_t>(1, nlights);
    const size_t need = noalloc_bytes(P, n_items, B, nq);
    if (need > kNoAllocScratchBytes) {
        char msg[256];
        std::snprintf(msg, sizeof(msg),
                      "render_noalloc: frame needs %zu bytes of scratch, the fixed array holds %zu "
                      "(%zu x %zu pixels, %u bands, %u lights); use vgb_render or a smaller frame",
                      need, kNoAllocScratchBytes, (size_t)cam->width, (size_t)cam->height, B, nlights);
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, msg);
    }
    CK(cudaSetDevice(ctx->device));
    if (!ctx->noalloc_base) {
        // Once per context, with its device current: the device address of the fixed array (in
        // host code the array's name stands for a host-side shadow, not for device memory).
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return fail(ctx, VGB_ERR_CUDA, std::string("render_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        ctx->noalloc_base = static_cast<unsigned char*>(p);
    }
    unsigned char* const base = ctx->noalloc_base;
    // Carve the frame's scratch out of the fixed array.
    DevState st{};
    size_t off = 0;
    auto take = [&](size_t bytes) { unsigned char* q = base + off; off += up256(bytes); return q; };
    const size_t f = sizeof(float);
    st.counters = reinterpret_cast<uint32_t*>(take(256));
    st.stats = reinterpret_cast<uint64_t*>(take(256));
    st.org = (float*)take(3 * P * f); st.dir = (float*)take(3 * P * f); st.thr = (float*)take(B * P * f);
    st.prad = (float*)take(B * P * f); st.brad = (float*)take(B * P * f); st.pend = (uint32_t*)take(P * f);
    st.arad = (float*)take(B * P * f); st.adir = (float*)take(B * P * f); st.aalb = (float*)take(B * P * f);
    st.anrm = (float*)take(3 * P * f); st.adep = (float*)take(P * f); st.acnt = (uint32_t*)take(P * f);
    st.atri = (uint32_t*)take(P * f); st.pq[0] = (uint32_t*)take(P * f); st.pq[1] = (uint32_t*)take(P * f);
    st.hit = (float4*)take(n_items * sizeof(float4));
    for (uint32_t l = 0; l < VGB_MAX_LIGHTS; ++l) {
        if (l < nq) {
            st.sq_org[l] = (float*)take(3 * P * f); st.sq_dir[l] = (float*)take(3 * P * f);
            st.sq_tmax[l] = (float*)take(P * f); st.sq_slot[l] = (uint32_t*)take(P * f);
            st.sq_con[l] = (float*)take(B * P * f);
        } else {
            st.sq_org[l] = st.sq_dir[l] = st.sq_tmax[l] = st.sq_con[l] = nullptr; st.sq_slot[l] = nullptr;
        }
    }
    if (off != need) return fail(ctx, VGB_ERR_INTERNAL, "render_noalloc: scratch layout differs from its size");
    st.P = P;
    FrameParams fp;
    std::memset(&fp, 0, sizeof(fp));
    fp.cam = *cam;
    fp.opt = *opts;
    for (uint32_t l = 0; l < nlights; ++l) fp.lights[l] = lights[l];
    fp.nlights = nlights;
    fp.nb = B;
    fp.tiles_x = (cam->width + 7) / 8;
    fp.tiles_y = (cam->height + 3) / 4;
    FilmOut fo{};
    fo.total = film->total_radiance; fo.direct = film->direct_radiance; fo.indirect = film->indirect_radiance;
    fo.power = film->received_power; fo.albedo = film->albedo; fo.normal = film->normal_global;
    fo.depth = film->depth; fo.alpha = film->alpha; fo.tri = film->triangle_id; fo.omega = film->pixel_solid_angle;
    fo.vel_g = film->velocity_global; fo.vel_c = film->velocity_camera; fo.tsz = film->triangle_size;
    fp.aux = aux_for(fo);
    fp.vel_g = fo.vel_g; fp.vel_c = fo.vel_c; fp.tsz = fo.tsz;
    // The array keeps the last call's contents: the counters, statistics and error word must
    // start at zero; every other region is written before it is read.
    CK(cudaMemsetAsync(st.counters, 0, 256, ctx->stream));
    CK(cudaMemsetAsync(st.stats, 0, 256, ctx->stream));
    uint32_t launches = 0;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    dispatch_render<false>(ctx, fp, fo, st, false, launches);
    CK(cudaGetLastError());
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    uint32_t err_word = 0;
    uint64_t hs[8] = {0};
    CK(cudaMemcpyAsync(&err_word, &st.counters[C_ERR], sizeof(err_word), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaMemcpyAsync(hs, st.stats, sizeof(hs), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    // the statistics this call measures; the counting pass and per-family profiling do not apply
    // (their fields read 0); the BVH fields describe the scene and stay
    const vgb_stats keep = ctx->stats;
    ctx->stats = vgb_stats{};
    ctx->stats.bvh_nodes = keep.bvh_nodes;
    ctx->stats.bvh_node_bytes = keep.bvh_node_bytes;
    ctx->stats.tri_record_bytes = keep.tri_record_bytes;
    ctx->stats.rays_closest = hs[2];
    ctx->stats.rays_shadow = hs[3];
    ctx->stats.hits_closest = hs[6];
    ctx->stats.kernel_launches = launches;
    ctx->stats.ms_last = ms;
    ctx->stats.device_error = err_word;
    if (err_word)
        return fail(ctx, VGB_ERR_DEVICE_LIMIT,
                    std::string("render_noalloc: device traversal limit hit:") + ((err_word & kErrStack) ? " stack" : "") +
                        ((err_word & kErrIter) ? " iterations" : ""));
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}


// Out-of-line traversal for the kernels that trace both ray kinds in one large body (k_batch,
// the adjoint replay): one copy of the loop, called for closest-hit and occlusion rays, keeps
// those kernels' instruction footprint small (instruction fetch was their leading stall; the
// batch kernel ran 12 % and the adjoint 28 % faster than with both loops inlined).
template <int L>
__device__ __noinline__ void trace_ool(const DevScene& s, WRay r, float tmax, bool any, HitOut& h, uint32_t& err) {
    Counters c{0, 0};
    if (L == 8) traverse8_rt<false>(s.nodes, s.tris, r, tmax, any, h, err, c, s.iter_cap);
    else traverse_rt<false>(reinterpret_cast<const float4*>(s.nodes), s.tris, r, tmax, any, h, err, c, s.iter_cap);
}

// ====================================================================== batched trajectory
namespace {

struct DevFrame {
    vgb_camera cam;
    vgb_light lights[VGB_MAX_LIGHTS];
    uint32_t nlights, samples, frame, tiles_x, tile_begin, pad[3];
    FilmOut film;
};

struct BatchParams {
    vgb_pt_options opt;
    uint32_t nframes, nb, total_tiles, grab, tile_stride;
    uint32_t sums;   // some frame requests a direct, indirect, albedo or normal plane
};

__device__ __forceinline__ uint32_t find_frame(const DevFrame* __restrict__ frames, uint32_t n, uint32_t t) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (frames[mid].tile_begin <= t) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Cold path of k_batch, out of line so that the sample loop's instruction footprint stays small:
// unidirectional's adaptive stopping rule after a sample (cpu_path_tracer.ipp:198-226).
struct AdaptStep { float s1, s2; bool stop; };
template <int NB>
__device__ __noinline__ AdaptStep batch_adaptive_step(const float* acc, int lane, uint32_t nb, uint32_t sample,
                                                      const vgb_pt_options& opt, float s1, float s2) {
    float sq = 0.f;
#pragma unroll
    for (int k = 0; k < NB; ++k) {
        const float pr = acc[(3 * NB + 4 + k) * 32 + lane];
        if (k < (int)nb) sq += pr * pr;
    }
    const float illum = sqrtf(sq);
    s1 = s1 + illum;
    s2 = s2 + illum * illum;
    bool stop = false;
    if (sample != 0 && sample % opt.samples_to_detect_miss == 0 && acc[(3 * NB + 3) * 32 + lane] == 0.f) {
        stop = true;
    } else if (sample != 0 && sample % opt.samples_per_batch == 0) {
        if (s1 == 0.f) {
            stop = true;
        } else {
            const float n = (float)sample + 1.f;
            const float mu = s1 / n;
            const float variance = (1.f / (n - 1.f)) * (s2 - (s1 * s1) / n);
            const float I = 1.96f * sqrtf(variance / n);
            stop = I <= opt.sampling_tolerance * mu;
        }
    }
    return AdaptStep{s1, s2, stop};
}

// Shared-memory planes per lane of k_batch: arad[NB] adir[NB] aalb[NB] anrm[3] adep (the
// pixel's sums over samples) | prad[NB] brad[NB] (the current sample).
__host__ __device__ constexpr int batch_planes(int nb, bool) { return 5 * nb + 4; }

// One persistent launch over every (frame, tile) item.  A warp owns an 8x4-pixel tile and loops
// over its samples and bounces in step: every lane traces its closest-hit ray, then the
// occlusion rays of its lights, so the lanes of a warp run the same traversal together.
// Accumulation order and random streams are those of the wavefront path (bit-identical film).
// DIRECT (no bounces) drops the continuation and its throughput.
template <int NB, int L, bool DIRECT>
__global__ void __launch_bounds__(256, DIRECT ? VGB_BATCH_DIRECT_MINB : 1) k_batch(const DevScene s, const DevFrame* __restrict__ frames, const __grid_constant__ BatchParams bp,
                        uint32_t* counter, uint32_t* errw, uint64_t* stats) {
    extern __shared__ float sm_acc[];
    constexpr int PL = 5 * NB + 4;  // arad[NB] adir[NB] aalb[NB] anrm[3] adep | prad[NB] brad[NB]
    const int lane = threadIdx.x & 31;
    float* acc = sm_acc + (size_t)(threadIdx.x >> 5) * PL * 32;
#define ACC(pl) acc[(pl) * 32 + lane]
    const uint32_t nb = bp.nb;
    const vgb_pt_options& opt = bp.opt;
    const uint32_t k0 = (uint32_t)opt.seed, k1 = (uint32_t)(opt.seed >> 32);
    const uint32_t n_items = (bp.total_tiles + bp.tile_stride - 1) / bp.tile_stride;
    uint32_t err = 0, nclosest = 0, nshadow = 0;
    while (true) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, bp.grab);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_items) break;
        const uint32_t end = min(base + bp.grab, n_items);
        for (uint32_t it = base; it < end; ++it) {
            const uint32_t t = it * bp.tile_stride;
            const DevFrame& F = frames[find_frame(frames, bp.nframes, t)];
            const uint32_t tile = t - F.tile_begin;
            const uint32_t tx = tile % F.tiles_x, ty = tile / F.tiles_x;
            const uint32_t pi = tx * 8u + (lane & 7u), pj = ty * 4u + (lane >> 3);
            const uint32_t W = F.cam.width, H = F.cam.height;
            if (pi >= W || pj >= H) continue;
            const uint32_t slot = pj * W + pi;
#pragma unroll
            for (int p = 0; p < PL; ++p) acc[p * 32 + lane] = 0.f;
            uint32_t first_tri = VGB_NO_HIT;
            uint32_t count = 0;
            float s1 = 0.f, s2 = 0.f;   // adaptive sampling: magnitude sums
            uint32_t stopped = 0;       // adaptive sampling: sample index at which the pixel stopped
            for (uint32_t sample = 0; sample < F.samples; ++sample) {
                // camera ray (camera_ray with this frame's camera and key)
                F3 ro, rd;
                pixel_ray(F.cam, pi, pj, slot, sample, F.frame, k0, k1, ro, rd);
                float thr[NB], alb[NB];
#define PRAD(k) acc[(3 * NB + 4 + (k)) * 32 + lane]
#define BRAD(k) acc[(4 * NB + 4 + (k)) * 32 + lane]
#pragma unroll
                for (int k = 0; k < NB; ++k) { thr[k] = 1.f; PRAD(k) = 0.f; BRAD(k) = 0.f; }
                uint32_t pend = 0;
                const uint32_t last_bounce = DIRECT ? 0u : opt.bounces;
                for (uint32_t bounce = 0; bounce <= last_bounce; ++bounce) {
                    if (pend) {
#pragma unroll
                        for (int k = 0; k < NB; ++k) {
                            PRAD(k) += BRAD(k);
                            if (pend == 1u && k < (int)nb) ACC(NB + k) += BRAD(k);
                        }
                        pend = 0;
                    }
                    HitOut h;
                    h.U = h.V = h.W = 0.f; h.det = 1.f;
                    const WRay wr = make_wray(ro, rd);
                    trace_ool<L>(s, wr, 0.f, false, h, err);
                    nclosest++;
                    if (h.id == VGB_NO_HIT) {
                        if (opt.simulate_lighting && opt.show_background) {
                            const float4 bw = background_weights(rd);
                            const float a = bw.x, b = bw.y, c = bw.z, e = bw.w;
#pragma unroll
                            for (int k = 0; k < NB; ++k) {
                                const float bgv = opt.background[k];
                                float bg = ((a * bgv + b * bgv) + c * bgv) + e * bgv;
                                PRAD(k) = PRAD(k) + thr[k] * (bg * 1.f);
                            }
                        }
                        break;
                    }
                    const float rcp = 1.0f / h.det;
                    const float w0 = h.V * rcp, w1 = h.W * rcp;
                    F3 Pp, N, fnrm, tg, bt, nf;
                    surface_at<NB>(s, nb, opt.smooth_shading != 0, h.id, w0, w1, Pp, N, fnrm, tg, bt, nf, alb);
                    if (bounce == 0) {
                        if (first_tri == VGB_NO_HIT) {
                            first_tri = h.id;
                            if (F.film.tsz || F.film.vel_g || F.film.vel_c)
                                first_hit_passes(s, F.cam, h.id, Pp, F.film.vel_g, F.film.vel_c, F.film.tsz,
                                                 (size_t)W * H, slot);
                        }
#pragma unroll
                        for (int k = 0; k < NB; ++k) if (k < (int)nb) ACC(2 * NB + k) += alb[k];
                        ACC(3 * NB + 0) += N.x; ACC(3 * NB + 1) += N.y; ACC(3 * NB + 2) += N.z;
                        ACC(3 * NB + 3) += h.t;
                        count += 1u;
                    }
                    if (!opt.simulate_lighting) break;
                    Pp = F3{offset1(Pp.x, fnrm.x), offset1(Pp.y, fnrm.y), offset1(Pp.z, fnrm.z)};
#pragma unroll
                    for (int k = 0; k < NB; ++k)
                        BRAD(k) = (bounce == 0 && opt.has_ambient && k < (int)nb) ? 0.f + thr[k] * (opt.ambient[k] * alb[k]) : 0.f;
                    pend = (bounce == 0) ? 1u : 2u;
                    const U4 r0 = philox(U4{slot, sample, F.frame, (bounce << 8) | kSlotMain}, k0, k1);
                    for (uint32_t l = 0; l < F.nlights; ++l) {
                        float ru1, ru2;
                        if (l == 0) { ru1 = u01(r0.x); ru2 = u01(r0.y); }
                        else {
                            U4 rl = philox(U4{slot, sample, F.frame, (bounce << 8) | (1u + l)}, k0, k1);
                            ru1 = u01(rl.x); ru2 = u01(rl.y);
                        }
                        // nee_light, with the contribution formed only once the shadow ray is clear
                        F3 Ld; float dist, lpdf = 0.f;
                        light_sample(F.lights[l], Pp, opt.deterministic_light != 0, ru1, ru2, Ld, dist, lpdf);
                        if (lpdf > 0) {
                            HitOut hs;
                            const WRay ws = make_wray(Pp, Ld);
                            trace_ool<L>(s, ws, dist, true, hs, err);
                            nshadow++;
                            if (hs.id == VGB_NO_HIT) {
                                const float nl = dot(N, Ld);
                                const float cos_t = smax(0.0f, dot(Ld, N));
                                const float mpdf = (nl <= 0.f) ? 0.f : nl * kInvPi;
                                const float wgt = power_heuristic(lpdf, mpdf);
#pragma unroll
                                for (int k = 0; k < NB; ++k) {
                                    const float bsdf = alb[k] * kInvPi * smax(nl, 0.f);
                                    const float con = (k < (int)nb) ? thr[k] * bsdf * F.lights[l].radiance[k] * cos_t * wgt / lpdf : 0.f;
                                    BRAD(k) += con;
                                }
                            }
                        }
                    }
                    if (DIRECT || bounce >= opt.bounces) break;
                    bool new_ray = false;
                    F3 nd;
                    const bool cont = continue_path<NB>(F.lights, F.nlights, opt, nb, Pp, N, tg, bt, nf, alb, thr, r0, slot,
                                                        sample, F.frame, bounce, nd, new_ray);
                    if (!cont) break;
                    if (new_ray) { ro = Pp; rd = nd; }
                }
                if (pend) {
#pragma unroll
                    for (int k = 0; k < NB; ++k) {
                        PRAD(k) += BRAD(k);
                        if (pend == 1u && k < (int)nb) ACC(NB + k) += BRAD(k);
                    }
                }
#pragma unroll
                for (int k = 0; k < NB; ++k) if (k < (int)nb) ACC(k) = ACC(k) + PRAD(k);
                if (opt.adaptive_sampling) {
                    const AdaptStep st = batch_adaptive_step<NB>(acc, lane, nb, sample, opt, s1, s2);
                    s1 = st.s1;
                    s2 = st.s2;
                    if (st.stop) { stopped = sample; break; }
                }
#undef PRAD
#undef BRAD
            }
            // RenderPasses::updateImages for this pixel
            const size_t P = (size_t)W * H;
            const float sf = stopped ? (float)stopped : (float)F.samples;  // the reference divides by the last index
            const FilmOut& f = F.film;
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                if (k < (int)nb) {
                    const float total = ACC(k) / sf;
                    const float direct = ACC(NB + k) / sf;
                    if (f.total) f.total[k * P + slot] = total;
                    if (f.direct) f.direct[k * P + slot] = direct;
                    if (f.indirect) f.indirect[k * P + slot] = total - direct;
                    if (f.albedo) f.albedo[k * P + slot] = ACC(2 * NB + k) / sf;
                    if (f.power) f.power[k * P + slot] = (F.cam.power_scale[k] * f.omega[slot]) * total;
                }
            }
            if (f.normal) {
                F3 n = normalize(F3{ACC(3 * NB + 0), ACC(3 * NB + 1), ACC(3 * NB + 2)});
                f.normal[slot] = n.x; f.normal[P + slot] = n.y; f.normal[2 * P + slot] = n.z;
            }
            if (f.depth) f.depth[slot] = (count == 0) ? __int_as_float(0x7f800000) : ACC(3 * NB + 3) / (float)count;
            if (f.alpha) f.alpha[slot] = (float)count / sf;
            if (f.tri) f.tri[slot] = first_tri;
            if (first_tri == VGB_NO_HIT) {   // never hit: the passes' initial values
                if (f.tsz) f.tsz[slot] = __int_as_float(0x7f800000);
                if (f.vel_g) { f.vel_g[slot] = 0.f; f.vel_g[P + slot] = 0.f; f.vel_g[2 * P + slot] = 0.f; }
                if (f.vel_c) { f.vel_c[slot] = 0.f; f.vel_c[P + slot] = 0.f; f.vel_c[2 * P + slot] = 0.f; }
            }
        }
    }
#undef ACC
    if (err) atomicOr(errw, err);
    warp_reduce_add(&stats[2], nclosest);
    warp_reduce_add(&stats[3], nshadow);
}

// k_batch for direct lighting without adaptive sampling, with the per-pixel sums in registers:
// with no bounce the path throughput stays 1 and a sample's path radiance is its bounce-0
// radiance (ambient + the unoccluded light contributions, or the background of a miss), so the
// shared-memory planes of k_batch reduce to per-lane sums over the samples.  SUMS keeps the
// direct, albedo and normal sums (films that request those planes or the indirect one).  The
// arithmetic and its order are k_batch's (and the wavefront's): the planes are bit-identical.
template <int NB, int L, bool SUMS>
__global__ void __launch_bounds__(256, VGB_BATCH_LEAN_MINB) k_batch_direct(const DevScene s, const DevFrame* __restrict__ frames,
                                                              const __grid_constant__ BatchParams bp, uint32_t* counter,
                                                              uint32_t* errw, uint64_t* stats) {
    // The warp's lanes stay converged through every traversal (lanes outside the frame or whose
    // ray missed carry flags), so the binary layout can trace the tile's rays as warp packets.
    constexpr bool PACKET = L == 2 && VGB_BATCH_PACKET;
    const int lane = threadIdx.x & 31;
    const uint32_t nb = bp.nb;
    const vgb_pt_options& opt = bp.opt;
    const uint32_t k0 = (uint32_t)opt.seed, k1 = (uint32_t)(opt.seed >> 32);
    const uint32_t n_items = (bp.total_tiles + bp.tile_stride - 1) / bp.tile_stride;
    const float4* nodes2 = reinterpret_cast<const float4*>(s.nodes);
    uint32_t err = 0, nclosest = 0, nshadow = 0;
    while (true) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(counter, bp.grab);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= n_items) break;
        const uint32_t end = min(base + bp.grab, n_items);
        for (uint32_t it = base; it < end; ++it) {
            const uint32_t t = it * bp.tile_stride;
            const DevFrame& F = frames[find_frame(frames, bp.nframes, t)];
            const uint32_t tile = t - F.tile_begin;
            const uint32_t tx = tile % F.tiles_x, ty = tile / F.tiles_x;
            const uint32_t pi = tx * 8u + (lane & 7u), pj = ty * 4u + (lane >> 3);
            const uint32_t W = F.cam.width, H = F.cam.height;
            const bool valid = pi < W && pj < H;
            const uint32_t slot = valid ? pj * W + pi : 0u;
            float tot[NB], dir[SUMS ? NB : 1], albs[SUMS ? NB : 1];
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                tot[k] = 0.f;
                if (SUMS) { dir[k] = 0.f; albs[k] = 0.f; }
            }
            F3 nsum{0.f, 0.f, 0.f};
            float dsum = 0.f;
            uint32_t count = 0, first_tri = VGB_NO_HIT;
            for (uint32_t sample = 0; sample < F.samples; ++sample) {
                F3 ro{0.f, 0.f, 0.f}, rd{0.f, 0.f, 1.f};
                if (valid) pixel_ray(F.cam, pi, pj, slot, sample, F.frame, k0, k1, ro, rd);
                HitOut h;
                h.U = h.V = h.W = 0.f; h.det = 1.f;
                h.id = VGB_NO_HIT;
                if (PACKET) {
                    traverse_packet<false>(nodes2, s.tris, make_wray(ro, rd), 0.f, valid, h, err, s.iter_cap);
                } else if (valid) {
                    if (VGB_BATCH_LEAN_OOL) {
                        trace_ool<L>(s, make_wray(ro, rd), 0.f, false, h, err);
                    } else {
                        Counters c{0, 0};
                        traverse_any_layout<L, false, false>(s.nodes, s.tris, make_wray(ro, rd), 0.f, h, err, c,
                                                             s.iter_cap);
                    }
                }
                if (valid) nclosest++;
                const bool hit = valid && h.id != VGB_NO_HIT;
                if (valid && !hit && opt.simulate_lighting && opt.show_background) {
                    const float4 bw = background_weights(rd);
#pragma unroll
                    for (int k = 0; k < NB; ++k) {
                        const float bgv = opt.background[k];
                        const float bg = ((bw.x * bgv + bw.y * bgv) + bw.z * bgv) + bw.w * bgv;
                        tot[k] = tot[k] + (0.f + 1.f * (bg * 1.f));
                    }
                }
                float alb[NB], br[NB];
                F3 Pp{0.f, 0.f, 0.f}, N{0.f, 0.f, 1.f};
#pragma unroll
                for (int k = 0; k < NB; ++k) { alb[k] = 0.f; br[k] = 0.f; }
                const bool lit = hit && opt.simulate_lighting;
                if (hit) {
                    const float rcp = 1.0f / h.det;
                    F3 fnrm, tg, bt, nf;
                    surface_at<NB, false>(s, nb, opt.smooth_shading != 0, h.id, h.V * rcp, h.W * rcp, Pp, N, fnrm, tg, bt,
                                          nf, alb);
                    if (first_tri == VGB_NO_HIT) {
                        first_tri = h.id;
                        if (F.film.tsz || F.film.vel_g || F.film.vel_c)
                            first_hit_passes(s, F.cam, h.id, Pp, F.film.vel_g, F.film.vel_c, F.film.tsz, (size_t)W * H, slot);
                    }
                    if (SUMS) {
#pragma unroll
                        for (int k = 0; k < NB; ++k) if (k < (int)nb) albs[k] += alb[k];
                        nsum = F3{nsum.x + N.x, nsum.y + N.y, nsum.z + N.z};
                    }
                    dsum += h.t;
                    count += 1u;
                    if (lit) {
                        Pp = F3{offset1(Pp.x, fnrm.x), offset1(Pp.y, fnrm.y), offset1(Pp.z, fnrm.z)};
#pragma unroll
                        for (int k = 0; k < NB; ++k)
                            br[k] = (opt.has_ambient && k < (int)nb) ? 0.f + 1.f * (opt.ambient[k] * alb[k]) : 0.f;
                    }
                }
                U4 r0{0, 0, 0, 0};
                if (lit) r0 = philox(U4{slot, sample, F.frame, kSlotMain}, k0, k1);
                for (uint32_t l = 0; l < F.nlights; ++l) {
                    F3 Ld{0.f, 0.f, 1.f};
                    float dist = 0.f, lpdf = 0.f;
                    if (lit) {
                        float ru1, ru2;
                        if (l == 0) { ru1 = u01(r0.x); ru2 = u01(r0.y); }
                        else {
                            const U4 rl = philox(U4{slot, sample, F.frame, 1u + l}, k0, k1);
                            ru1 = u01(rl.x); ru2 = u01(rl.y);
                        }
                        light_sample(F.lights[l], Pp, opt.deterministic_light != 0, ru1, ru2, Ld, dist, lpdf);
                    }
                    const bool shadow = lit && lpdf > 0;
                    HitOut hs;
                    hs.id = VGB_NO_HIT;
                    if (PACKET) {
                        if (__any_sync(0xffffffffu, shadow))
                            traverse_packet<true>(nodes2, s.tris, make_wray(Pp, Ld), dist, shadow, hs, err, s.iter_cap);
                    } else if (shadow) {
                        if (VGB_BATCH_LEAN_OOL) {
                            trace_ool<L>(s, make_wray(Pp, Ld), dist, true, hs, err);
                        } else {
                            Counters c{0, 0};
                            traverse_any_layout<L, true, false>(s.nodes, s.tris, make_wray(Pp, Ld), dist, hs, err, c,
                                                                s.iter_cap);
                        }
                    }
                    if (shadow) {
                        nshadow++;
                        if (hs.id == VGB_NO_HIT) {
                            const float nl = dot(N, Ld);
                            const float cos_t = smax(0.0f, dot(Ld, N));
                            const float mpdf = (nl <= 0.f) ? 0.f : nl * kInvPi;
                            const float wgt = power_heuristic(lpdf, mpdf);
#pragma unroll
                            for (int k = 0; k < NB; ++k) {
                                const float bsdf = alb[k] * kInvPi * smax(nl, 0.f);
                                br[k] += (k < (int)nb) ? 1.f * bsdf * F.lights[l].radiance[k] * cos_t * wgt / lpdf : 0.f;
                            }
                        }
                    }
                }
                if (lit) {
#pragma unroll
                    for (int k = 0; k < NB; ++k) {
                        tot[k] = tot[k] + (0.f + br[k]);
                        if (SUMS && k < (int)nb) dir[k] += br[k];
                    }
                }
            }
            if (!valid) continue;
            // RenderPasses::updateImages for this pixel
            const size_t P = (size_t)W * H;
            const float sf = (float)F.samples;
            const FilmOut& f = F.film;
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                if (k < (int)nb) {
                    const float total = tot[k] / sf;
                    const float direct = SUMS ? dir[k] / sf : 0.f;
                    if (f.total) f.total[k * P + slot] = total;
                    if (SUMS && f.direct) f.direct[k * P + slot] = direct;
                    if (SUMS && f.indirect) f.indirect[k * P + slot] = total - direct;
                    if (SUMS && f.albedo) f.albedo[k * P + slot] = albs[k] / sf;
                    if (f.power) f.power[k * P + slot] = (F.cam.power_scale[k] * f.omega[slot]) * total;
                }
            }
            if (SUMS && f.normal) {
                const F3 n = normalize(nsum);
                f.normal[slot] = n.x; f.normal[P + slot] = n.y; f.normal[2 * P + slot] = n.z;
            }
            if (f.depth) f.depth[slot] = (count == 0) ? __int_as_float(0x7f800000) : dsum / (float)count;
            if (f.alpha) f.alpha[slot] = (float)count / sf;
            if (f.tri) f.tri[slot] = first_tri;
            if (first_tri == VGB_NO_HIT) {
                if (f.tsz) f.tsz[slot] = __int_as_float(0x7f800000);
                if (f.vel_g) { f.vel_g[slot] = 0.f; f.vel_g[P + slot] = 0.f; f.vel_g[2 * P + slot] = 0.f; }
                if (f.vel_c) { f.vel_c[slot] = 0.f; f.vel_c[P + slot] = 0.f; f.vel_c[2 * P + slot] = 0.f; }
            }
        }
    }
    if (err) atomicOr(errw, err);
    warp_reduce_add(&stats[2], nclosest);
    warp_reduce_add(&stats[3], nshadow);
}

// The lean direct-lighting kernel applies when there is no bounce and no adaptive sampling; SUMS
// when a frame requests the direct, indirect, albedo or normal plane.
inline bool batch_lean(const BatchParams& bp) { return bp.opt.bounces == 0 && !bp.opt.adaptive_sampling; }

template <int NB, int L, bool SUMS>
cudaError_t launch_batch_lean(vgb_context* ctx, const DevFrame* d_frames, const BatchParams& bp, uint32_t threads,
                              uint32_t bps) {
    int maxb = 0;
#if VGB_L1_CARVEOUT >= 0
    static bool carved = false;
    if (!carved) {
        cudaFuncSetAttribute(k_batch_direct<NB, L, SUMS>, cudaFuncAttributePreferredSharedMemoryCarveout, VGB_L1_CARVEOUT);
        carved = true;
    }
#endif
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, k_batch_direct<NB, L, SUMS>, (int)threads, 0);
    const uint32_t b = std::max<uint32_t>(1, std::min<uint32_t>(bps, (uint32_t)std::max(1, maxb)));
    cudaMemsetAsync(&ctx->d_counters[C_BATCH], 0, sizeof(uint32_t), ctx->stream);
    k_batch_direct<NB, L, SUMS><<<b * ctx->num_sms, threads, 0, ctx->stream>>>(dev_scene(ctx), d_frames, bp,
                                                                              &ctx->d_counters[C_BATCH],
                                                                              &ctx->d_counters[C_ERR], ctx->d_stats);
    return cudaGetLastError();
}

template <int NB, int L, bool DIRECT>
cudaError_t launch_batch_t(vgb_context* ctx, const DevFrame* d_frames, const BatchParams& bp, uint32_t threads,
                           uint32_t bps) {
    const size_t smem = (size_t)(threads / 32) * batch_planes(NB, DIRECT) * 32 * sizeof(float);
    cudaError_t e = cudaFuncSetAttribute(k_batch<NB, L, DIRECT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int maxb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&maxb, k_batch<NB, L, DIRECT>, (int)threads, smem);
    const uint32_t b = std::max<uint32_t>(1, std::min<uint32_t>(bps, (uint32_t)std::max(1, maxb)));
    cudaMemsetAsync(&ctx->d_counters[C_BATCH], 0, sizeof(uint32_t), ctx->stream);
    k_batch<NB, L, DIRECT><<<b * ctx->num_sms, threads, smem, ctx->stream>>>(dev_scene(ctx), d_frames, bp,
                                                                             &ctx->d_counters[C_BATCH],
                                                                             &ctx->d_counters[C_ERR], ctx->d_stats);
    return cudaGetLastError();
}

template <int NB, int L>
cudaError_t launch_batch(vgb_context* ctx, const DevFrame* d_frames, const BatchParams& bp, uint32_t threads,
                         uint32_t bps) {
    if (batch_lean(bp)) {
        if (bp.sums) return launch_batch_lean<NB, L, true>(ctx, d_frames, bp, threads, bps);
        return launch_batch_lean<NB, L, false>(ctx, d_frames, bp, threads, bps);
    }
    if (bp.opt.bounces == 0) return launch_batch_t<NB, L, true>(ctx, d_frames, bp, threads, bps);
    return launch_batch_t<NB, L, false>(ctx, d_frames, bp, threads, bps);
}

cudaError_t launch_batch_any(vgb_context* ctx, const DevFrame* d_frames, const BatchParams& bp, uint32_t threads,
                             uint32_t bps) {
    if (ctx->bvh_layout == 8) {
        if (bp.nb <= 1) return launch_batch<1, 8>(ctx, d_frames, bp, threads, bps);
        if (bp.nb <= 4) return launch_batch<4, 8>(ctx, d_frames, bp, threads, bps);
        return launch_batch<8, 8>(ctx, d_frames, bp, threads, bps);
    }
    if (bp.nb <= 1) return launch_batch<1, 2>(ctx, d_frames, bp, threads, bps);
    if (bp.nb <= 4) return launch_batch<4, 2>(ctx, d_frames, bp, threads, bps);
    return launch_batch<8, 2>(ctx, d_frames, bp, threads, bps);
}

}  // namespace

extern "C" VGB_API vgb_status vgb_batch_tuning(vgb_context* ctx, uint32_t* threads, uint32_t* bps, uint32_t* grab) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (threads) *threads = ctx->tuned_threads;
    if (bps) *bps = ctx->tuned_bps;
    if (grab) *grab = ctx->tuned_grab;
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

extern "C" VGB_API vgb_status vgb_render_batch(vgb_context* ctx, const vgb_frame* frames, uint32_t nframes,
                                               const vgb_pt_options* opts, const vgb_batch_options* bo) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!frames || nframes == 0 || !opts) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_batch: no frames or options");
    if (!ctx->bvh_ready) return fail(ctx, VGB_ERR_NOT_READY, "render_batch: build the BVH first");
    if (opts->nbands != ctx->nbands) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_batch: nbands differs from the scene");
    if (opts->adaptive_sampling && (opts->samples_per_batch == 0 || opts->samples_to_detect_miss == 0))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_batch: adaptive sampling needs samples_per_batch and samples_to_detect_miss >= 1");
    // schedule: frames by decreasing samples per pixel (cost per tile), then by index
    std::vector<uint32_t> order(nframes);
    for (uint32_t f = 0; f < nframes; ++f) {
        const vgb_frame& fr = frames[f];
        if (fr.samples == 0 || !frame_fits(fr.camera.width, fr.camera.height) || fr.nlights > VGB_MAX_LIGHTS ||
            !fr.film.on_device || (fr.film.received_power && !fr.film.pixel_solid_angle))
            return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_batch: frame " + std::to_string(f) +
                                                           ": samples/resolution/lights/film invalid (film must be device memory)");
        if (opts->denoise && (!fr.film.direct_radiance || !fr.film.indirect_radiance || !fr.film.albedo ||
                              !fr.film.depth || !fr.film.normal_global))
            return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_batch: frame " + std::to_string(f) +
                                                           ": denoising needs direct, indirect, albedo, depth and normal planes");
        order[f] = f;
    }
    std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return frames[a].samples > frames[b].samples; });
    cudaSetDevice(ctx->device);
    if (nframes > ctx->cap_frames) {
        dfree(ctx->d_frames);
        if (ctx->h_frames) cudaFreeHost(ctx->h_frames);
        ctx->d_frames = nullptr; ctx->h_frames = nullptr; ctx->cap_frames = 0;
        vgb_status s = dalloc(ctx, &ctx->d_frames, sizeof(DevFrame) * nframes);
        if (s != VGB_OK) return s;
        CK(cudaMallocHost(&ctx->h_frames, sizeof(DevFrame) * nframes));
        ctx->cap_frames = nframes;
        if (ctx->graph_exec) { cudaGraphExecDestroy(ctx->graph_exec); ctx->graph_exec = nullptr; }
    }
    CK(cudaStreamSynchronize(ctx->stream));  // the pinned table may still feed a previous copy
    DevFrame* hf = static_cast<DevFrame*>(ctx->h_frames);
    uint64_t total_tiles = 0;
    for (uint32_t i = 0; i < nframes; ++i) {
        const vgb_frame& fr = frames[order[i]];
        DevFrame& d = hf[i];
        std::memset(&d, 0, sizeof(d));
        d.cam = fr.camera;
        for (uint32_t l = 0; l < fr.nlights; ++l) d.lights[l] = fr.lights[l];
        d.nlights = fr.nlights;
        d.samples = fr.samples;
        d.frame = fr.frame;
        d.tiles_x = (fr.camera.width + 7) / 8;
        d.tile_begin = (uint32_t)total_tiles;
        total_tiles += (uint64_t)d.tiles_x * ((fr.camera.height + 3) / 4);
        d.film.total = fr.film.total_radiance; d.film.direct = fr.film.direct_radiance;
        d.film.indirect = fr.film.indirect_radiance; d.film.power = fr.film.received_power;
        d.film.albedo = fr.film.albedo; d.film.normal = fr.film.normal_global; d.film.depth = fr.film.depth;
        d.film.alpha = fr.film.alpha; d.film.tri = fr.film.triangle_id; d.film.omega = fr.film.pixel_solid_angle;
        d.film.vel_g = fr.film.velocity_global; d.film.vel_c = fr.film.velocity_camera; d.film.tsz = fr.film.triangle_size;
    }
    if (total_tiles >= (1ull << 31)) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_batch: too many pixels");
    CK(cudaMemcpyAsync(ctx->d_frames, hf, sizeof(DevFrame) * nframes, cudaMemcpyHostToDevice, ctx->stream));
    BatchParams bp;
    std::memset(&bp, 0, sizeof(bp));
    bp.opt = *opts;
    bp.nframes = nframes;
    bp.nb = ctx->nbands;
    bp.total_tiles = (uint32_t)total_tiles;
    for (uint32_t f = 0; f < nframes; ++f) {
        const vgb_film& fl = frames[f].film;
        if (fl.direct_radiance || fl.indirect_radiance || fl.albedo || fl.normal_global) bp.sums = 1;
    }
    const DevFrame* dfr = static_cast<const DevFrame*>(ctx->d_frames);
    uint32_t threads = bo && bo->block_threads ? bo->block_threads : (ctx->tuned_threads ? ctx->tuned_threads : 256);
    uint32_t bps = bo && bo->blocks_per_sm ? bo->blocks_per_sm : (ctx->tuned_bps ? ctx->tuned_bps : 4);
    uint32_t grab = bo && bo->tiles_per_grab ? bo->tiles_per_grab : (ctx->tuned_grab ? ctx->tuned_grab : 1);
    if (threads != 64 && threads != 128 && threads != 256)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_batch: block_threads must be 64, 128 or 256");
    CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(uint64_t) * 8, ctx->stream));
    if (bo && bo->autotune) {
        // autotuner: time candidate launch shapes on every 16th tile, keep the fastest
        const uint32_t cand_t[] = {64, 128, 256};
        const uint32_t cand_b[] = {2, 4, 8, 16};
        const uint32_t cand_g[] = {1, 4};
        float best = INFINITY;
        BatchParams probe = bp;
        probe.tile_stride = 16;
        for (uint32_t ct : cand_t)
            for (uint32_t cb : cand_b)
                for (uint32_t cg : cand_g) {
                    probe.grab = cg;
                    CK(cudaEventRecord(ctx->ev0, ctx->stream));
                    CK(launch_batch_any(ctx, dfr, probe, ct, cb));
                    CK(cudaEventRecord(ctx->ev1, ctx->stream));
                    CK(cudaEventSynchronize(ctx->ev1));
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
                    if (ms < best) { best = ms; threads = ct; bps = cb; grab = cg; }
                }
        ctx->tuned_threads = threads; ctx->tuned_bps = bps; ctx->tuned_grab = grab;
        CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(uint64_t) * 8, ctx->stream));
        vgb_status es = check_device_error(ctx);
        if (es != VGB_OK) return es;
    }
    bp.grab = grab;
    bp.tile_stride = 1;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    if (bo && bo->use_graph) {
        const uint64_t key = ((uint64_t)nframes << 40) ^ ((uint64_t)total_tiles << 8) ^ ((uint64_t)threads << 4) ^ bps ^
                             ((uint64_t)grab << 56) ^ ((uint64_t)ctx->nbands << 60) ^ ((uint64_t)ctx->bvh_layout << 20) ^
                             ((uint64_t)opts->bounces << 24) ^ ((uint64_t)opts->samples << 28);
        static_assert(sizeof(BatchParams) < 4096, "kernel parameters");
        // the graph holds the launch with these parameters; rebuild it when they change
        if (!ctx->graph_exec || ctx->graph_key != key ||
            std::memcmp(&ctx->graph_params_probe, &bp, sizeof(bp)) != 0) {
            if (ctx->graph_exec) { cudaGraphExecDestroy(ctx->graph_exec); ctx->graph_exec = nullptr; }
            cudaGraph_t g = nullptr;
            CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
            cudaError_t le = launch_batch_any(ctx, dfr, bp, threads, bps);
            cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
            CK(le);
            CK(ce);
            cudaError_t ie = cudaGraphInstantiate(&ctx->graph_exec, g, 0);
            cudaGraphDestroy(g);
            CK(ie);
            ctx->graph_key = key;
            std::memcpy(&ctx->graph_params_probe, &bp, sizeof(bp));
        }
        CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    } else {
        CK(launch_batch_any(ctx, dfr, bp, threads, bps));
    }
    if (opts->denoise) {
        // options.denoise per frame, on the frame's own planes (checked above)
        size_t most = 0;
        for (uint32_t f = 0; f < nframes; ++f) most = std::max(most, (size_t)frames[f].camera.width * frames[f].camera.height);
        vgb_status ds = ensure_dn_scratch(ctx, dn_work_floats(ctx->nbands, most));
        if (ds != VGB_OK) return ds;
        for (uint32_t f = 0; f < nframes; ++f) {
            const vgb_frame& fr = frames[f];
            const vgb_film& fl = fr.film;
            PowerScale ps{};
            for (uint32_t k = 0; k < ctx->nbands && k < VGB_MAX_BANDS; ++k) ps.v[k] = fr.camera.power_scale[k];
            launch_denoise(ctx, fl.direct_radiance, fl.indirect_radiance, fl.albedo, fl.depth, fl.normal_global,
                           fr.camera.width, fr.camera.height, ctx->nbands, dn_opts(&opts->denoiser), ctx->d_dn,
                           fl.direct_radiance, fl.indirect_radiance, fl.total_radiance, fl.received_power,
                           fl.pixel_solid_angle, ps);
        }
        CK(cudaGetLastError());
    }
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    uint64_t hs[8];
    CK(cudaMemcpy(hs, ctx->d_stats, sizeof(hs), cudaMemcpyDeviceToHost));
    ctx->stats.rays_closest = hs[2];
    ctx->stats.rays_shadow = hs[3];
    ctx->stats.kernel_launches = 1;
    ctx->stats.ms_last = ms;
    return check_device_error(ctx);
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}


// ====================================================================== adjoint (path replay)
// Gradients of the loss L(I) with respect to the albedo texels and the vertex positions, given
// dL/dI for the total-radiance planes.  Each pixel sample's path is replayed from its random
// stream (nothing is stored between the forward render and this pass), its vertices are kept
// in local memory for the length of the path, and the gradients are scattered with atomics:
//   albedo     every contribution at or after vertex b is linear in alb_b, so
//              dI/d alb_b = (suffix radiance from b) / alb_b, then through alb = va * bilinear(tex)
//   positions  the shading normal N in every NEE term, d C / d(N.L) = C (2 / (N.L) + w'/w),
//              back through the face normal (flat shading) or through N = normalize(sum w_i n_i)
//              to the vertex normals n_i (smooth shading; k_vnormal_backward carries those to
//              the positions of each vertex's 1-ring); and the motion of the hit point on the
//              triangle for a fixed ray, d[t, b1, b2]/dp_q = w_q M^-1 (M = [d | A-B | A-C]),
//              which moves the texture coordinates, the interpolated albedo and normal.
// Excluded and stated: visibility (shadow and silhouette edges), the rotation of the sampled
// continuation direction with the normal, the motion of the shading point (light direction and
// shadow-ray origin), and Russian roulette decisions.
namespace {

constexpr int kAdjMaxVerts = 4;

template <int NB>
struct AdjVtx {
    uint32_t tri;
    float w0, w1;
    float m[3][2];        // M^-1 e_a for a = x, y, z: the barycentric components (b1, b2)
    float uvx, uvy;
    float gnx, gny, gnz;  // dL/dN at this vertex (already weighted by dL/dI)
    float alb[NB], va[NB], tex[NB], rad[NB];
};

struct AdjOut {
    float* gtex;        // [th][tw][B] or null
    float* gpos;        // [nverts][3] or null
    float* gvn;         // [nverts][3] vertex-normal gradients (smooth shading) or null
};

// Replays one pixel sample and records its path vertices; returns their number.  `g` (dL/dI
// per band, already divided by the sample count) may be null: no normal gradients are formed.
// prad receives the sample's path radiance, summed in the order of the forward renderer.
template <int NB, int L>
__device__ __forceinline__ int adj_replay(const DevScene& s, const vgb_camera& cam, const vgb_light* lights,
                                          uint32_t nlights, const vgb_pt_options& opt, uint32_t nb, uint32_t pi,
                                          uint32_t pj, uint32_t slot, uint32_t sample, uint32_t frame,
                                          const float* g, AdjVtx<NB>* vx, float* bgc, float* prad,
                                          uint32_t& err, uint32_t& nrays) {
    const uint32_t k0 = (uint32_t)opt.seed, k1 = (uint32_t)(opt.seed >> 32);
    F3 ro, rd;
    pixel_ray(cam, pi, pj, slot, sample, frame, k0, k1, ro, rd);
    float thr[NB];
#pragma unroll
    for (int k = 0; k < NB; ++k) { thr[k] = 1.f; bgc[k] = 0.f; prad[k] = 0.f; }
    int nv = 0;
    for (uint32_t bounce = 0; bounce <= opt.bounces && nv < kAdjMaxVerts; ++bounce) {
        HitOut h;
        h.U = h.V = h.W = 0.f; h.det = 1.f;
        const WRay wr = make_wray(ro, rd);
        trace_ool<L>(s, wr, 0.f, false, h, err);
        nrays++;
        if (h.id == VGB_NO_HIT) {
            if (opt.simulate_lighting && opt.show_background) {
                float x = rd.x, y = rd.y, z = rd.z;
                float u = atan2f(y, x) / (2 * kPi);
                float v = atan2f(sqrtf(x * x + y * y), z) / kPi;
                float px = fmodf(u * 1.f, 1.f), py = fmodf(v * 1.f, 1.f);
                if (px < 0) px += 1.f;
                if (py < 0) py += 1.f;
                float a = (1.f - px) * (1.f - py), b = px * (1.f - py), c = (1.f - px) * py, e = px * py;
#pragma unroll
                for (int k = 0; k < NB; ++k) {
                    const float bgv = opt.background[k];
                    bgc[k] = thr[k] * ((((a * bgv + b * bgv) + c * bgv) + e * bgv) * 1.f);
                    prad[k] = prad[k] + bgc[k];
                }
            }
            break;
        }
        AdjVtx<NB>& V = vx[nv++];
        const float rcp = 1.0f / h.det;
        V.tri = h.id;
        V.w0 = h.V * rcp;
        V.w1 = h.W * rcp;
        F3 Pp, N, fnrm, tg, bt, nf;
        float uv[2];
        surface_at<NB>(s, nb, opt.smooth_shading != 0, h.id, V.w0, V.w1, Pp, N, fnrm, tg, bt, nf, V.alb, V.va, V.tex, uv);
        V.uvx = uv[0]; V.uvy = uv[1];
        if (g) {
            // M^-1 e_a for the hit-point motion (caller order A=v0, B=v1, C=v2), by Cramer's rule:
            // b1 = det[d, e_a, c2] / det, b2 = det[d, c1, e_a] / det
            const uint32_t ia = __ldg(&s.idx[3 * h.id]), ib = __ldg(&s.idx[3 * h.id + 1]), ic = __ldg(&s.idx[3 * h.id + 2]);
            const F3 A = ld3(__ldg(&s.vpos[ia])), B = ld3(__ldg(&s.vpos[ib])), C = ld3(__ldg(&s.vpos[ic]));
            const F3 c1 = A - B, c2 = A - C;
            const float det = dot(rd, cross(c1, c2));
            const float idet = (det != 0.f) ? 1.f / det : 0.f;
            const F3 u1 = cross(c2, rd), u2 = cross(rd, c1);  // det[d, e_a, c2] = e_a . (c2 x d)
            V.m[0][0] = u1.x * idet; V.m[1][0] = u1.y * idet; V.m[2][0] = u1.z * idet;
            V.m[0][1] = u2.x * idet; V.m[1][1] = u2.y * idet; V.m[2][1] = u2.z * idet;
        }
        V.gnx = V.gny = V.gnz = 0.f;
#pragma unroll
        for (int k = 0; k < NB; ++k) V.rad[k] = 0.f;
        if (!opt.simulate_lighting) break;
        Pp = F3{offset1(Pp.x, fnrm.x), offset1(Pp.y, fnrm.y), offset1(Pp.z, fnrm.z)};
#pragma unroll
        for (int k = 0; k < NB; ++k)
            V.rad[k] = (bounce == 0 && opt.has_ambient && k < (int)nb) ? 0.f + thr[k] * (opt.ambient[k] * V.alb[k]) : 0.f;
        const U4 r0 = philox(U4{slot, sample, frame, (bounce << 8) | kSlotMain}, k0, k1);
        for (uint32_t l = 0; l < nlights; ++l) {
            float ru1, ru2;
            if (l == 0) { ru1 = u01(r0.x); ru2 = u01(r0.y); }
            else {
                U4 rl = philox(U4{slot, sample, frame, (bounce << 8) | (1u + l)}, k0, k1);
                ru1 = u01(rl.x); ru2 = u01(rl.y);
            }
            F3 Ld; float dist, lpdf = 0.f;
            light_sample(lights[l], Pp, opt.deterministic_light != 0, ru1, ru2, Ld, dist, lpdf);
            if (!(lpdf > 0)) continue;
            HitOut hs;
            const WRay ws = make_wray(Pp, Ld);
            trace_ool<L>(s, ws, dist, true, hs, err);
            nrays++;
            if (hs.id != VGB_NO_HIT) continue;
            const float nl = dot(N, Ld);
            const float cos_t = smax(0.0f, dot(Ld, N));
            const float mpdf = (nl <= 0.f) ? 0.f : nl * kInvPi;
            const float wgt = power_heuristic(lpdf, mpdf);
            float gc = 0.f;
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                const float bsdf = V.alb[k] * kInvPi * smax(nl, 0.f);
                const float con = (k < (int)nb) ? thr[k] * bsdf * lights[l].radiance[k] * cos_t * wgt / lpdf : 0.f;
                V.rad[k] += con;
                if (g) gc += g[k] * con;
            }
            if (g && nl > 0.f && wgt > 0.f) {
                // d/dc of c^2 w(c) with w = lp^2 / (lp^2 + (c/pi)^2)
                const float m = nl * kInvPi;
                const float dw_over_w = -2.f * m * kInvPi / (lpdf * lpdf + m * m);
                const float s_c = gc * (2.f / nl + dw_over_w);
                V.gnx += s_c * Ld.x; V.gny += s_c * Ld.y; V.gnz += s_c * Ld.z;
            }
        }
#pragma unroll
        for (int k = 0; k < NB; ++k) prad[k] = prad[k] + V.rad[k];
        if (bounce >= opt.bounces) break;
        bool new_ray = false;
        F3 nd;
        const bool cont = continue_path<NB>(lights, nlights, opt, nb, Pp, N, tg, bt, nf, V.alb, thr, r0, slot, sample,
                                            frame, bounce, nd, new_ray);
        if (!cont) break;
        if (new_ray) { ro = Pp; rd = nd; }
    }
    return nv;
}

// Backward over the recorded vertices of one sample: suffix radiance, then the scatter.
template <int NB>
__device__ __forceinline__ void adj_scatter(const DevScene& s, uint32_t nb, bool smooth, const AdjVtx<NB>* vx,
                                            int nv, const float* bgc, const float* g, const AdjOut& out) {
    float S[NB];
#pragma unroll
    for (int k = 0; k < NB; ++k) S[k] = bgc[k];
    for (int b = nv - 1; b >= 0; --b) {
        const AdjVtx<NB>& V = vx[b];
        float ga[NB];
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            S[k] += V.rad[k];
            ga[k] = (k < (int)nb && V.alb[k] != 0.f) ? g[k] * S[k] / V.alb[k] : 0.f;
        }
        // texel weights of sample_uvs at (uvx, uvy)
        const float rx = (float)s.tw, ry = (float)s.th;
        float px = fmodf(V.uvx * rx, rx), py = fmodf(V.uvy * ry, ry);
        if (px < 0) px += rx;
        if (py < 0) py += ry;
        int x0 = min((int)floorf(px), (int)s.tw - 1), y0 = min((int)floorf(py), (int)s.th - 1);
        int x1 = min(x0 + 1, (int)s.tw - 1), y1 = min(y0 + 1, (int)s.th - 1);
        const float dx = px - (float)x0, dy = py - (float)y0;
        const float wt[4] = {(1.f - dx) * (1.f - dy), dx * (1.f - dy), (1.f - dx) * dy, dx * dy};
        const size_t tx[4] = {(size_t)y0 * s.tw + x0, (size_t)y0 * s.tw + x1, (size_t)y1 * s.tw + x0,
                              (size_t)y1 * s.tw + x1};
        if (out.gtex) {
#pragma unroll
            for (int k = 0; k < NB; ++k) {
                if (k >= (int)nb || ga[k] == 0.f) continue;
                const float base = ga[k] * V.va[k];
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (wt[q] != 0.f) atomicAdd(&out.gtex[tx[q] * nb + k], base * wt[q]);
            }
        }
        if (!out.gpos) continue;
        const uint32_t ia = __ldg(&s.idx[3 * V.tri]), ib = __ldg(&s.idx[3 * V.tri + 1]), ic = __ldg(&s.idx[3 * V.tri + 2]);
        const F3 A = ld3(__ldg(&s.vpos[ia])), B = ld3(__ldg(&s.vpos[ib])), C = ld3(__ldg(&s.vpos[ic]));
        const F3 gN{V.gnx, V.gny, V.gnz};
        // dL/d(w0, w1) through the albedo (vertex albedo and texture coordinates)
        const float2 uvA = __ldg(&s.vuv[ia]), uvB = __ldg(&s.vuv[ib]), uvC = __ldg(&s.vuv[ic]);
        float gw0 = 0.f, gw1 = 0.f;
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            if (k >= (int)nb || ga[k] == 0.f) continue;
            float t00, t10, t01, t11;
            if (s.tex_mono) {
                t00 = __ldg(&s.tex[tx[0]]); t10 = __ldg(&s.tex[tx[1]]);
                t01 = __ldg(&s.tex[tx[2]]); t11 = __ldg(&s.tex[tx[3]]);
            } else {
                t00 = __ldg(&s.tex[tx[0] * nb + k]); t10 = __ldg(&s.tex[tx[1] * nb + k]);
                t01 = __ldg(&s.tex[tx[2] * nb + k]); t11 = __ldg(&s.tex[tx[3] * nb + k]);
            }
            const float dtdx = (1.f - dy) * (t10 - t00) + dy * (t11 - t01);
            const float dtdy = (1.f - dx) * (t01 - t00) + dx * (t11 - t10);
            // d px / d w0 = rx * (uvB - uvA).x, ... (Interaction order: w0 ~ B, w1 ~ C)
            const float dt_dw0 = dtdx * rx * (uvB.x - uvA.x) + dtdy * ry * (uvB.y - uvA.y);
            const float dt_dw1 = dtdx * rx * (uvC.x - uvA.x) + dtdy * ry * (uvC.y - uvA.y);
            float dva_dw0 = 0.f, dva_dw1 = 0.f;
            if (!s.albedo_uniform) {
                const float aA = __ldg(&s.valb[(size_t)ia * nb + k]), aB = __ldg(&s.valb[(size_t)ib * nb + k]);
                const float aC = __ldg(&s.valb[(size_t)ic * nb + k]);
                dva_dw0 = aB - aA; dva_dw1 = aC - aA;
            }
            gw0 += ga[k] * (dva_dw0 * V.tex[k] + V.va[k] * dt_dw0);
            gw1 += ga[k] * (dva_dw1 * V.tex[k] + V.va[k] * dt_dw1);
        }
        F3 gp[3] = {F3{0.f, 0.f, 0.f}, F3{0.f, 0.f, 0.f}, F3{0.f, 0.f, 0.f}};  // A, B, C
        const float wA = 1.0f - V.w0 - V.w1;
        if (!smooth) {
            // face normal N = -n/|n|, n = cross(a, bb), a = A-B, bb = C-A
            const F3 a = A - B, bb = C - A;
            const F3 n = cross(a, bb);
            const float ln = length(n);
            if (ln > 0.f) {
                const F3 nh = n * (1.f / ln);
                const F3 gn = (gN - nh * dot(nh, gN)) * (-1.f / ln);   // dL/dn
                const F3 ga_ = cross(bb, gn), gb_ = cross(gn, a);       // dL/da, dL/dbb
                gp[0] = ga_ - gb_; gp[1] = F3{0.f, 0.f, 0.f} - ga_; gp[2] = gb_;
            }
        } else {
            // N = S/|S|, S = w0 n_B + w1 n_C + wA n_A (surface_at's order)
            const F3 nA = ld3(__ldg(&s.vnrm[ia])), nB = ld3(__ldg(&s.vnrm[ib])), nC = ld3(__ldg(&s.vnrm[ic]));
            const F3 Sv = (V.w0 * nB + V.w1 * nC) + wA * nA;
            const float lS = length(Sv);
            if (lS > 0.f && out.gvn) {
                const F3 Nn = Sv * (1.f / lS);
                const F3 gS = (gN - Nn * dot(Nn, gN)) * (1.f / lS);
                gw0 += dot(gS, nB - nA);
                gw1 += dot(gS, nC - nA);
                const uint32_t vid[3] = {ia, ib, ic};
                const float wv[3] = {wA, V.w0, V.w1};
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    if (wv[q] == 0.f) continue;
                    atomicAdd(&out.gvn[3 * (size_t)vid[q] + 0], wv[q] * gS.x);
                    atomicAdd(&out.gvn[3 * (size_t)vid[q] + 1], wv[q] * gS.y);
                    atomicAdd(&out.gvn[3 * (size_t)vid[q] + 2], wv[q] * gS.z);
                }
            }
        }
        // hit-point motion: dL/dp_q,a = w_q (gw0 m_a1 + gw1 m_a2)
        const F3 gm{gw0 * V.m[0][0] + gw1 * V.m[0][1], gw0 * V.m[1][0] + gw1 * V.m[1][1],
                    gw0 * V.m[2][0] + gw1 * V.m[2][1]};
        const uint32_t vid[3] = {ia, ib, ic};
        const float wv[3] = {wA, V.w0, V.w1};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const F3 t = gp[q] + gm * wv[q];
            if (t.x != 0.f) atomicAdd(&out.gpos[3 * (size_t)vid[q] + 0], t.x);
            if (t.y != 0.f) atomicAdd(&out.gpos[3 * (size_t)vid[q] + 1], t.y);
            if (t.z != 0.f) atomicAdd(&out.gpos[3 * (size_t)vid[q] + 2], t.z);
        }
    }
}

template <int NB, int L>
__global__ void __launch_bounds__(VGB_ADJOINT_BLOCK) k_adjoint(const DevScene s, const __grid_constant__ FrameParams fp,
                                                 const float* __restrict__ dldi, const AdjOut out, uint32_t* errw,
                                                 uint64_t* stats) {
    const uint32_t nb = fp.nb;
    const vgb_pt_options& opt = fp.opt;
    const uint32_t npix = fp.cam.width * fp.cam.height;
    const uint32_t n_items = fp.tiles_x * fp.tiles_y * 32u;
    const float sf = (float)opt.samples;
    const bool smooth = opt.smooth_shading != 0;
    uint32_t err = 0, nrays = 0;
    for (uint32_t item = blockIdx.x * blockDim.x + threadIdx.x; item < n_items; item += gridDim.x * blockDim.x) {
        const uint32_t tile = item >> 5, ln = item & 31u;
        const uint32_t pi = (tile % fp.tiles_x) * 8u + (ln & 7u), pj = (tile / fp.tiles_x) * 4u + (ln >> 3);
        if (pi >= fp.cam.width || pj >= fp.cam.height) continue;
        const uint32_t slot = pj * fp.cam.width + pi;
        float g[NB];
        bool any = false;
#pragma unroll
        for (int k = 0; k < NB; ++k) {
            g[k] = (k < (int)nb) ? dldi[(size_t)k * npix + slot] / sf : 0.f;
            any |= g[k] != 0.f;
        }
        if (!any) continue;
        for (uint32_t sample = 0; sample < opt.samples; ++sample) {
            AdjVtx<NB> vx[kAdjMaxVerts];
            float bgc[NB], prad[NB];
            const int nv = adj_replay<NB, L>(s, fp.cam, fp.lights, fp.nlights, opt, nb, pi, pj, slot, sample,
                                             opt.frame, g, vx, bgc, prad, err, nrays);
            adj_scatter<NB>(s, nb, smooth, vx, nv, bgc, g, out);
        }
    }
    if (err) atomicOr(errw, err);
    warp_reduce_add(&stats[2], nrays);
}

// Sums of the unit face normals per vertex (vgb_compute_vertex_normals before its normalisation).
__global__ void k_vnormal_sums(const float4* __restrict__ vpos, const uint32_t* __restrict__ idx, uint32_t ntris,
                               float* __restrict__ sums) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntris; t += gridDim.x * blockDim.x) {
        const uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
        const F3 p0 = ld3(vpos[i0]), p1 = ld3(vpos[i1]), p2 = ld3(vpos[i2]);
        if (isinf(p0.x) || isinf(p1.x) || isinf(p2.x)) continue;
        const F3 c = cross(p1 - p0, p2 - p0);
        const float lc = length(c);
        if (!(lc > 0.f)) continue;
        const F3 u = c * (1.f / lc);
        const uint32_t v[3] = {i0, i1, i2};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            atomicAdd(&sums[3 * (size_t)v[q] + 0], u.x);
            atomicAdd(&sums[3 * (size_t)v[q] + 1], u.y);
            atomicAdd(&sums[3 * (size_t)v[q] + 2], u.z);
        }
    }
}

// Vertex-normal gradients to position gradients.  n_v = A_v/|A_v|, A_v = sum of the unit face
// normals u_f = c_f/|c_f|, c_f = cross(p1 - p0, p2 - p0) over the faces of v:
// dL/dA_v = (G_v - n_v (n_v.G_v)) / |A_v|; per face dL/du_f = sum of dL/dA_v of its vertices,
// dL/dc_f = (dL/du_f - u_f (u_f.dL/du_f)) / |c_f|, dL/de1 = e2 x dL/dc, dL/de2 = dL/dc x e1.
__global__ void k_vnormal_backward(const float4* __restrict__ vpos, const uint32_t* __restrict__ idx, uint32_t ntris,
                                   const float* __restrict__ sums, const float* __restrict__ gvn,
                                   float* __restrict__ gpos) {
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < ntris; t += gridDim.x * blockDim.x) {
        const uint32_t v[3] = {idx[3 * t], idx[3 * t + 1], idx[3 * t + 2]};
        const F3 p0 = ld3(vpos[v[0]]), p1 = ld3(vpos[v[1]]), p2 = ld3(vpos[v[2]]);
        if (isinf(p0.x) || isinf(p1.x) || isinf(p2.x)) continue;
        const F3 e1 = p1 - p0, e2 = p2 - p0;
        const F3 c = cross(e1, e2);
        const float lc = length(c);
        if (!(lc > 0.f)) continue;
        F3 gu{0.f, 0.f, 0.f};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const size_t o = 3 * (size_t)v[q];
            const F3 Av{sums[o], sums[o + 1], sums[o + 2]};
            const F3 G{gvn[o], gvn[o + 1], gvn[o + 2]};
            const float la = length(Av);
            if (!(la > 0.f)) continue;
            const F3 n = Av * (1.f / la);
            gu = gu + (G - n * dot(n, G)) * (1.f / la);
        }
        const F3 u = c * (1.f / lc);
        const F3 gc = (gu - u * dot(u, gu)) * (1.f / lc);
        const F3 g1 = cross(e2, gc), g2 = cross(gc, e1);
        const F3 g0 = F3{0.f, 0.f, 0.f} - (g1 + g2);
        const F3 gq[3] = {g0, g1, g2};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const size_t o = 3 * (size_t)v[q];
            if (gq[q].x != 0.f) atomicAdd(&gpos[o + 0], gq[q].x);
            if (gq[q].y != 0.f) atomicAdd(&gpos[o + 1], gq[q].y);
            if (gq[q].z != 0.f) atomicAdd(&gpos[o + 2], gq[q].z);
        }
    }
}

// z components of a [n][3] array added into a [n] array.
__global__ void k_add_z(const float* __restrict__ xyz, uint32_t n, float* __restrict__ z) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) z[i] += xyz[3 * (size_t)i + 2];
}

// ---------------------------------------------------------------- fused forward + adjoint
struct DevView {
    vgb_camera cam;
    vgb_light lights[VGB_MAX_LIGHTS];
    uint32_t nlights, samples, frame, tiles_x, tile_begin, pad[3];
    const float* target;
    float* radiance;
};

struct AdjBatchParams {
    vgb_pt_options opt;
    uint32_t nviews, nb, total_tiles;
};

// One persistent launch over every (view, 8x4-pixel tile) item; a lane owns a pixel: its
// samples are traced (forward radiance, in the forward renderer's order), dL/dI = 2 (I - T)
// is formed and the samples are replayed for the gradients.
template <int NB, int L>
__global__ void __launch_bounds__(128) k_adjoint_batch(const DevScene s, const DevView* __restrict__ views,
                                                       const __grid_constant__ AdjBatchParams bp, const AdjOut out,
                                                       uint32_t* counter, double* loss, uint32_t* errw,
                                                       uint64_t* stats) {
    const int lane = threadIdx.x & 31;
    const uint32_t nb = bp.nb;
    const vgb_pt_options& opt = bp.opt;
    const bool smooth = opt.smooth_shading != 0;
    uint32_t err = 0, nrays = 0;
    double lsum = 0.0;
    while (true) {
        uint32_t it = 0;
        if (lane == 0) it = atomicAdd(counter, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= bp.total_tiles) break;
        uint32_t lo = 0, hi = bp.nviews - 1;
        while (lo < hi) {
            const uint32_t mid = (lo + hi + 1) >> 1;
            if (views[mid].tile_begin <= it) lo = mid; else hi = mid - 1;
        }
        const DevView& Vw = views[lo];
        const uint32_t tile = it - Vw.tile_begin;
        const uint32_t pi = (tile % Vw.tiles_x) * 8u + (lane & 7u), pj = (tile / Vw.tiles_x) * 4u + (lane >> 3);
        const uint32_t W = Vw.cam.width, H = Vw.cam.height;
        if (pi >= W || pj >= H) continue;
        const uint32_t slot = pj * W + pi;
        const size_t P = (size_t)W * H;
        const float sf = (float)Vw.samples;
        float acc[NB], g[NB];
#pragma unroll
        for (int k = 0; k < NB; ++k) acc[k] = 0.f;
        for (uint32_t pass = 0; pass < 2; ++pass) {
            if (pass == 1) {
                // RenderPasses::updateImages, then the L2 loss and its gradient for this pixel
                bool any = false;
#pragma unroll
                for (int k = 0; k < NB; ++k) {
                    g[k] = 0.f;
                    if (k < (int)nb) {
                        const float I = acc[k] / sf;
                        if (Vw.radiance) Vw.radiance[k * P + slot] = I;
                        const float d = I - __ldg(&Vw.target[k * P + slot]);
                        lsum += (double)d * (double)d;
                        g[k] = (2.f * d) / sf;
                        any |= g[k] != 0.f;
                    }
                }
                if (!any || (!out.gtex && !out.gpos)) break;
            }
            for (uint32_t sample = 0; sample < Vw.samples; ++sample) {
                AdjVtx<NB> vx[kAdjMaxVerts];
                float bgc[NB], prad[NB];
                const int nv = adj_replay<NB, L>(s, Vw.cam, Vw.lights, Vw.nlights, opt, nb, pi, pj, slot, sample,
                                                 Vw.frame, pass ? g : nullptr, vx, bgc, prad, err, nrays);
                if (pass == 0) {
#pragma unroll
                    for (int k = 0; k < NB; ++k) if (k < (int)nb) acc[k] = acc[k] + prad[k];
                } else {
                    adj_scatter<NB>(s, nb, smooth, vx, nv, bgc, g, out);
                }
            }
        }
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_down_sync(0xffffffffu, lsum, o);
    if (lane == 0 && lsum != 0.0) atomicAdd(loss, lsum);
    if (err) atomicOr(errw, err);
    warp_reduce_add(&stats[2], nrays);
}

template <int NB, int L>
void launch_adjoint(vgb_context* ctx, const FrameParams& fp, const float* dldi, const AdjOut& out) {
    const uint32_t n = fp.tiles_x * fp.tiles_y * 32u;
    const int g = grid_for(ctx, n, VGB_ADJOINT_GRID * 128 / VGB_ADJOINT_BLOCK, VGB_ADJOINT_BLOCK_ITEMS * VGB_ADJOINT_BLOCK / 128);
    k_adjoint<NB, L><<<g, VGB_ADJOINT_BLOCK, 0, ctx->stream>>>(dev_scene(ctx), fp, dldi, out, &ctx->d_counters[C_ERR], ctx->d_stats);
}

template <int NB, int L>
void launch_adjoint_batch(vgb_context* ctx, const DevView* views, const AdjBatchParams& bp, const AdjOut& out) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_adjoint_batch<NB, L>, 128, 0);
    const uint32_t blocks = (uint32_t)std::max(1, per_sm) * (uint32_t)ctx->num_sms;
    k_adjoint_batch<NB, L><<<blocks, 128, 0, ctx->stream>>>(dev_scene(ctx), views, bp, out, &ctx->d_counters[C_BATCH],
                                                            ctx->d_loss, &ctx->d_counters[C_ERR], ctx->d_stats);
}

template <typename F>
void dispatch_nb_layout(vgb_context* ctx, F&& f) {
    const bool l8 = ctx->bvh_layout == 8;
    if (ctx->nbands <= 1) { if (l8) f(std::integral_constant<int, 1>{}, std::integral_constant<int, 8>{}); else f(std::integral_constant<int, 1>{}, std::integral_constant<int, 2>{}); }
    else if (ctx->nbands <= 4) { if (l8) f(std::integral_constant<int, 4>{}, std::integral_constant<int, 8>{}); else f(std::integral_constant<int, 4>{}, std::integral_constant<int, 2>{}); }
    else { if (l8) f(std::integral_constant<int, 8>{}, std::integral_constant<int, 8>{}); else f(std::integral_constant<int, 8>{}, std::integral_constant<int, 2>{}); }
}

// Position-gradient scratch: vertex-normal gradients, normal sums and (for z-only callers)
// full position gradients, [nverts][3] each.
vgb_status ensure_adj_scratch(vgb_context* ctx) {
    const size_t need = 9 * (size_t)ctx->nverts * sizeof(float);
    if (need <= ctx->cap_adj) return VGB_OK;
    dfree(ctx->d_adj);
    ctx->d_adj = nullptr;
    ctx->cap_adj = 0;
    vgb_status s = dalloc(ctx, &ctx->d_adj, need);
    if (s != VGB_OK) return s;
    ctx->cap_adj = need;
    return VGB_OK;
}

// Runs `body(out)` with the position outputs set up; gpos: caller's [nverts][3] or null,
// gz: caller's [nverts] (z only) or null.  Smooth shading adds the vertex-normal pass.
template <typename Body>
vgb_status run_adjoint(vgb_context* ctx, bool smooth, float* gtex, float* gpos, float* gz, Body&& body) {
    AdjOut out{gtex, nullptr, nullptr};
    const size_t n3 = 3 * (size_t)ctx->nverts;
    if (gpos || gz) {
        vgb_status s = ensure_adj_scratch(ctx);
        if (s != VGB_OK) return s;
        float* gvn = ctx->d_adj;
        float* sums = ctx->d_adj + n3;
        float* full = ctx->d_adj + 2 * n3;
        out.gpos = gpos ? gpos : full;
        if (!gpos) CK(cudaMemsetAsync(full, 0, n3 * sizeof(float), ctx->stream));
        if (smooth) {
            out.gvn = gvn;
            CK(cudaMemsetAsync(gvn, 0, 2 * n3 * sizeof(float), ctx->stream));
            k_vnormal_sums<<<grid_for(ctx, ctx->ntris), 256, 0, ctx->stream>>>(ctx->d_vpos, ctx->d_idx, ctx->ntris, sums);
        }
    }
    body(out);
    CK(cudaGetLastError());
    if (out.gvn)
        k_vnormal_backward<<<grid_for(ctx, ctx->ntris), 256, 0, ctx->stream>>>(ctx->d_vpos, ctx->d_idx, ctx->ntris,
                                                                               ctx->d_adj + n3, out.gvn, out.gpos);
    if (gz) k_add_z<<<grid_for(ctx, ctx->nverts), 256, 0, ctx->stream>>>(out.gpos, ctx->nverts, gz);
    CK(cudaGetLastError());
    return VGB_OK;
}

vgb_status adjoint_common(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights, uint32_t nlights,
                          const vgb_pt_options* opts, const float* dL_dradiance, float* d_texture, float* d_pos,
                          bool xyz, int on_device, const char* what) {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    const std::string w(what);
    if (!cam || !opts || !dL_dradiance) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, w + ": null camera/options/gradient");
    if (!ctx->bvh_ready) return fail(ctx, VGB_ERR_NOT_READY, w + ": build the BVH first");
    if (opts->samples == 0 || opts->nbands != ctx->nbands || nlights > VGB_MAX_LIGHTS || (nlights && !lights))
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, w + ": samples, nbands or lights invalid");
    if (opts->adaptive_sampling || opts->denoise)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, w + ": adaptive sampling and denoising are not differentiated");
    if (opts->bounces + 1 > (uint32_t)kAdjMaxVerts) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, w + ": at most 3 bounces");
    if (!frame_fits(cam->width, cam->height)) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, w + ": bad resolution");
    if (ctx->d_nmap) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, w + ": normal maps are not differentiated");
    cudaSetDevice(ctx->device);
    FrameParams fp;
    std::memset(&fp, 0, sizeof(fp));
    fp.cam = *cam;
    fp.opt = *opts;
    for (uint32_t l = 0; l < nlights; ++l) fp.lights[l] = lights[l];
    fp.nlights = nlights;
    fp.nb = ctx->nbands;
    fp.tiles_x = (cam->width + 7) / 8;
    fp.tiles_y = (cam->height + 3) / 4;
    const size_t npix = (size_t)cam->width * cam->height;
    const size_t ntex = (size_t)ctx->tw * ctx->th * ctx->nbands;
    const size_t npos = (xyz ? 3 : 1) * (size_t)ctx->nverts;
    const float* dl = dL_dradiance;
    float *gt = d_texture, *gp = d_pos;
    vgb_status s;
    if (!on_device) {
        const size_t need = npix * ctx->nbands + (d_texture ? ntex : 0) + (d_pos ? npos : 0);
        if ((s = ensure_staging(ctx, need * sizeof(float))) != VGB_OK) return s;
        float* cur = (float*)ctx->staging_base;
        CK(cudaMemcpyAsync(cur, dL_dradiance, npix * ctx->nbands * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        dl = cur; cur += npix * ctx->nbands;
        if (d_texture) { gt = cur; CK(cudaMemcpyAsync(gt, d_texture, ntex * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); cur += ntex; }
        if (d_pos) { gp = cur; CK(cudaMemcpyAsync(gp, d_pos, npos * sizeof(float), cudaMemcpyHostToDevice, ctx->stream)); }
    }
    CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(uint64_t) * 8, ctx->stream));
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    s = run_adjoint(ctx, opts->smooth_shading != 0, gt, xyz ? gp : nullptr, xyz ? nullptr : gp, [&](const AdjOut& out) {
        dispatch_nb_layout(ctx, [&](auto nbc, auto lc) { launch_adjoint<decltype(nbc)::value, decltype(lc)::value>(ctx, fp, dl, out); });
    });
    if (s != VGB_OK) return s;
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    if (!on_device) {
        if (d_texture) CK(cudaMemcpyAsync(d_texture, gt, ntex * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        if (d_pos) CK(cudaMemcpyAsync(d_pos, gp, npos * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
    }
    CK(cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    uint64_t hs[8];
    CK(cudaMemcpy(hs, ctx->d_stats, sizeof(hs), cudaMemcpyDeviceToHost));
    ctx->stats.rays_closest = hs[2];
    ctx->stats.rays_shadow = 0;
    ctx->stats.kernel_launches = 1;
    ctx->stats.ms_last = ms;
    return check_device_error(ctx);
}

}  // namespace

extern "C" VGB_API vgb_status vgb_adjoint(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights,
                                          uint32_t nlights, const vgb_pt_options* opts, const float* dL_dradiance,
                                          float* d_texture, float* d_height, int on_device) try {
    return adjoint_common(ctx, cam, lights, nlights, opts, dL_dradiance, d_texture, d_height, false, on_device, "adjoint");
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

extern "C" VGB_API vgb_status vgb_adjoint_positions(vgb_context* ctx, const vgb_camera* cam, const vgb_light* lights,
                                                    uint32_t nlights, const vgb_pt_options* opts,
                                                    const float* dL_dradiance, float* d_texture, float* d_position,
                                                    int on_device) try {
    return adjoint_common(ctx, cam, lights, nlights, opts, dL_dradiance, d_texture, d_position, true, on_device,
                          "adjoint_positions");
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

extern "C" VGB_API vgb_status vgb_render_adjoint_batch(vgb_context* ctx, const vgb_view* views, uint32_t nviews,
                                                       const vgb_pt_options* opts, float* d_texture, float* d_position,
                                                       double* loss) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!views || nviews == 0 || !opts) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_adjoint_batch: no views or options");
    if (!ctx->bvh_ready) return fail(ctx, VGB_ERR_NOT_READY, "render_adjoint_batch: build the BVH first");
    if (opts->nbands != ctx->nbands) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_adjoint_batch: nbands differs from the scene");
    if (opts->bounces + 1 > (uint32_t)kAdjMaxVerts)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_adjoint_batch: at most 3 bounces");
    if (opts->adaptive_sampling || opts->denoise)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_adjoint_batch: adaptive sampling and denoising are not differentiated");
    if (ctx->d_nmap) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_adjoint_batch: normal maps are not differentiated");
    cudaSetDevice(ctx->device);
    std::vector<DevView> hv(nviews);
    uint32_t tiles = 0;
    for (uint32_t i = 0; i < nviews; ++i) {
        const vgb_view& v = views[i];
        if (v.samples == 0 || v.nlights > VGB_MAX_LIGHTS || !v.target || !frame_fits(v.camera.width, v.camera.height))
            return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_adjoint_batch: view " + std::to_string(i) + " invalid");
        DevView& d = hv[i];
        std::memset(&d, 0, sizeof(d));
        d.cam = v.camera;
        for (uint32_t l = 0; l < v.nlights; ++l) d.lights[l] = v.lights[l];
        d.nlights = v.nlights;
        d.samples = v.samples;
        d.frame = v.frame;
        d.tiles_x = (v.camera.width + 7) / 8;
        d.tile_begin = tiles;
        d.target = v.target;
        d.radiance = v.radiance;
        const uint64_t t = (uint64_t)tiles + (uint64_t)d.tiles_x * ((v.camera.height + 3) / 4);
        if (t > 0xFFFFFFFFull) return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "render_adjoint_batch: too many tiles");
        tiles = (uint32_t)t;
    }
    vgb_status s;
    if (nviews * sizeof(DevView) > ctx->cap_views) {
        dfree(ctx->d_views);
        ctx->d_views = nullptr;
        ctx->cap_views = 0;
        if ((s = dalloc(ctx, &ctx->d_views, nviews * sizeof(DevView))) != VGB_OK) return s;
        ctx->cap_views = nviews * sizeof(DevView);
    }
    if (!ctx->d_loss && (s = dalloc(ctx, &ctx->d_loss, sizeof(double))) != VGB_OK) return s;
    CK(cudaMemcpyAsync(ctx->d_views, hv.data(), nviews * sizeof(DevView), cudaMemcpyHostToDevice, ctx->stream));
    CK(cudaMemsetAsync(ctx->d_loss, 0, sizeof(double), ctx->stream));
    CK(cudaMemsetAsync(&ctx->d_counters[C_BATCH], 0, sizeof(uint32_t), ctx->stream));
    CK(cudaMemsetAsync(ctx->d_stats, 0, sizeof(uint64_t) * 8, ctx->stream));
    AdjBatchParams bp;
    std::memset(&bp, 0, sizeof(bp));
    bp.opt = *opts;
    bp.nviews = nviews;
    bp.nb = ctx->nbands;
    bp.total_tiles = tiles;
    CK(cudaEventRecord(ctx->ev0, ctx->stream));
    s = run_adjoint(ctx, opts->smooth_shading != 0, d_texture, d_position, nullptr, [&](const AdjOut& out) {
        dispatch_nb_layout(ctx, [&](auto nbc, auto lc) {
            launch_adjoint_batch<decltype(nbc)::value, decltype(lc)::value>(ctx, (const DevView*)ctx->d_views, bp, out);
        });
    });
    if (s != VGB_OK) return s;
    CK(cudaEventRecord(ctx->ev1, ctx->stream));
    double hl = 0.0;
    CK(cudaMemcpyAsync(&hl, ctx->d_loss, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    CK(cudaStreamSynchronize(ctx->stream));
    if (loss) *loss = hl;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
    uint64_t hs[8];
    CK(cudaMemcpy(hs, ctx->d_stats, sizeof(hs), cudaMemcpyDeviceToHost));
    ctx->stats.rays_closest = hs[2];
    ctx->stats.rays_shadow = 0;
    ctx->stats.kernel_launches = 1;
    ctx->stats.ms_last = ms;
    return check_device_error(ctx);
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}

// Albedo texture update without re-uploading the mesh or rebuilding the BVH.
extern "C" VGB_API vgb_status vgb_texture_update(vgb_context* ctx, const float* texture, uint32_t tex_w, uint32_t tex_h) try {
    if (!ctx) return VGB_ERR_INVALID_ARGUMENT;
    if (!texture || tex_w != ctx->tw || tex_h != ctx->th)
        return fail(ctx, VGB_ERR_INVALID_ARGUMENT, "texture_update: size differs from the uploaded texture");
    if (ctx->nverts == 0) return fail(ctx, VGB_ERR_NOT_READY, "texture_update: no scene uploaded");
    cudaSetDevice(ctx->device);
    const size_t ntex = (size_t)tex_w * tex_h;
    const uint32_t B = ctx->nbands;
    bool mono = true;
    for (size_t t = 0; t < ntex && mono; ++t)
        for (uint32_t k = 1; k < B; ++k)
            if (std::memcmp(&texture[t * B + k], &texture[t * B], 4) != 0) { mono = false; break; }
    CK(cudaStreamSynchronize(ctx->stream));
    if (mono != (ctx->tex_mono != 0)) {
        dfree(ctx->d_tex);
        ctx->d_tex = nullptr;
        vgb_status s = dalloc(ctx, &ctx->d_tex, sizeof(float) * (mono ? ntex : ntex * B));
        if (s != VGB_OK) return s;
        ctx->tex_mono = mono ? 1u : 0u;
    }
    if (mono) {
        std::vector<float> m(ntex);
        for (size_t t = 0; t < ntex; ++t) m[t] = texture[t * B];
        CK(cudaMemcpy(ctx->d_tex, m.data(), ntex * sizeof(float), cudaMemcpyHostToDevice));
    } else {
        CK(cudaMemcpy(ctx->d_tex, texture, ntex * B * sizeof(float), cudaMemcpyHostToDevice));
    }
    return VGB_OK;
} catch (...) {
    return vgb::status_of_exception(ctx ? &ctx->err : nullptr);
}
