// vgb_mesh.cu -- DEM triangulation and vertex normals on the GPU, bit-identical to the host
// restatements in vgb_host.cpp.
//
// Triangulation: DEM::makeVertexBuffer (dem.ipp:165-211, non-OGR mapping of
// dem_projection.ipp:131-141) per post in FP64 as the host does, and imageToIndexBuffer
// (image_utils.ipp:364-409): quad (i, j), i outer, j inner, gives {(i,j+1),(i+1,j),(i,j)} and
// {(i+1,j),(i,j+1),(i+1,j+1)} unless a corner height is infinite; each quad's output position is
// an exclusive scan of the per-quad triangle counts, so the index buffer equals the host's.
// Normals: Mesh::calculateNormals (mesh.ipp:199-233): unit face normals summed per vertex and
// normalised.  The host adds a face's normal to its three corners in face order; here each
// vertex gathers its (face, corner) entries sorted ascending, so every sum is formed in the
// same order and rounds identically.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <vector>

#include "vgb_device.cuh"
#include "vgb_internal.h"

using namespace vgbd;
using vgb::DemPose;
using vgb::QuipuDecode;
using vgb::quipu_dequantize;

namespace {

// The grid's x per column and y per row (FP64, then FP32): a vertex's position is
// (xs[i], ys[j], h) -- each coordinate of DEMProjection::transformToWorld depends on one index.
__global__ void k_dem_axes(uint32_t W, uint32_t H, DemPose pose, float* __restrict__ xs, float* __restrict__ ys) {
    for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < (size_t)W + H; k += (size_t)gridDim.x * blockDim.x) {
        if (k < W) {
            const double s = ((double)k + pose.xo) * pose.scale_x;
            xs[k] = (float)(pose.ax * (-pose.half_x + 2. * s));
        } else {
            const double s = -((double)(k - W) + pose.yo) * pose.scale_y;
            ys[k - W] = (float)(pose.ay * (pose.half_y + 2. * s));
        }
    }
}

__device__ __forceinline__ F3 dem_point(const float* __restrict__ h, const float* __restrict__ xs,
                                        const float* __restrict__ ys, uint32_t W, uint32_t i, uint32_t j) {
    const float z = h[(size_t)j * W + i];
    if (isinf(z) || isnan(z)) {
        const float inf = __int_as_float(0x7f800000);
        return F3{inf, inf, inf};
    }
    return F3{xs[i], ys[j], z};
}

// Positions, and with NORMALS the vertex normals Mesh::calculateNormals gives on this grid's
// index buffer: the faces around vertex (i, j) in index-buffer order are
//   quad (i-1, j-1) t1, quad (i-1, j) t0 and t1, quad (i, j-1) t0 and t1, quad (i, j) t0
// (quads ordered i outer, j inner; t0 = {a, b, c}, t1 = {b, a, d}); a face exists when none of
// its heights is infinite, contributes when no corner's x is infinite and its normal is not
// NaN, and the contributions are summed in that order -- the general path's sum, bit for bit.
template <bool NORMALS>
__global__ void k_dem_vertices(const float* __restrict__ h, uint32_t W, uint32_t H, const float* __restrict__ xs,
                               const float* __restrict__ ys, float* __restrict__ pos, float* __restrict__ nrm) {
    const size_t n = (size_t)W * H;
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(v % W), j = (uint32_t)(v / W);
        const F3 p = dem_point(h, xs, ys, W, i, j);
        pos[3 * v] = p.x; pos[3 * v + 1] = p.y; pos[3 * v + 2] = p.z;
        if constexpr (NORMALS) {
            F3 acc{0.f, 0.f, 0.f};
            auto face = [&](uint32_t i0, uint32_t j0, uint32_t i1, uint32_t j1, uint32_t i2, uint32_t j2) {
                if (isinf(h[(size_t)j0 * W + i0]) || isinf(h[(size_t)j1 * W + i1]) || isinf(h[(size_t)j2 * W + i2]))
                    return;  // not in the index buffer
                const F3 p0 = dem_point(h, xs, ys, W, i0, j0), p1 = dem_point(h, xs, ys, W, i1, j1),
                         p2 = dem_point(h, xs, ys, W, i2, j2);
                if (isinf(p0.x) || isinf(p1.x) || isinf(p2.x)) return;
                const F3 f = normalize(cross(p1 - p0, p2 - p0));
                if (isnan(f.x) || isnan(f.y) || isnan(f.z)) return;
                acc = acc + f;
            };
            if (i >= 1 && j >= 1) face(i, j - 1, i - 1, j, i, j);                       // quad (i-1, j-1) t1
            if (i >= 1 && j + 1 < H) {
                face(i - 1, j + 1, i, j, i - 1, j);                                     // quad (i-1, j) t0
                face(i, j, i - 1, j + 1, i, j + 1);                                     //               t1
            }
            if (i + 1 < W && j >= 1) {
                face(i, j, i + 1, j - 1, i, j - 1);                                     // quad (i, j-1) t0
                face(i + 1, j - 1, i, j, i + 1, j);                                     //               t1
            }
            if (i + 1 < W && j + 1 < H) face(i, j + 1, i + 1, j, i, j);                 // quad (i, j) t0
            if (sqrtf(dot(acc, acc)) != 0.f) acc = normalize(acc);
            nrm[3 * v] = acc.x; nrm[3 * v + 1] = acc.y; nrm[3 * v + 2] = acc.z;
        }
    }
}

// Quipu LoD decode: heights from their stored codes (fixedToFloat, or FP32 as stored) and the
// per-vertex albedo DEM::makeVertexBuffer assigns (dem.ipp:191-200; Vertex's default 1 where
// the height is not finite), with readBuffers' grey-plane profile (dem_quipu.ipp:184-194).
template <typename T>
__global__ void k_quipu_decode(QuipuDecode d, const T* __restrict__ codes, const uint8_t* __restrict__ planes,
                               float* __restrict__ h, float* __restrict__ alb, bool vec4) {
    const size_t n = (size_t)d.W * d.H;
    const float m = sizeof(T) == 1 ? 255.f : 65535.f;
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
        float z;
        if constexpr (sizeof(T) == 4) z = codes[v];
        else z = quipu_dequantize((uint32_t)codes[v], m, d.hmin, d.hmax);
        h[v] = z;
        if (!alb) continue;
        const bool valid = !(isinf(z) || isnan(z));
        float av[VGB_MAX_BANDS];
        if (!valid || d.albedo_type == 0 || d.albedo_type == VGB_QUIPU_NO_ALBEDO) {
#pragma unroll
            for (uint32_t b = 0; b < VGB_MAX_BANDS; ++b) av[b] = valid ? d.constant[b] : 1.f;
        } else if (d.albedo_type == 1) {
            const float g = quipu_dequantize(planes[v], 255.f, d.pmin[0], d.pmax[0]);
#pragma unroll
            for (uint32_t b = 0; b < VGB_MAX_BANDS; ++b) av[b] = d.profile[b] * g;
        } else {
#pragma unroll
            for (uint32_t b = 0; b < VGB_MAX_BANDS; ++b)
                av[b] = b < d.nbands ? quipu_dequantize(planes[b * n + v], 255.f, d.pmin[b], d.pmax[b]) : 0.f;
        }
        // 16-byte stores when the rows allow them (4 or 8 bands on an aligned array)
        float* a = alb + v * d.nbands;
        if (vec4 && d.nbands == 8) {
            reinterpret_cast<float4*>(a)[0] = make_float4(av[0], av[1], av[2], av[3]);
            reinterpret_cast<float4*>(a)[1] = make_float4(av[4], av[5], av[6], av[7]);
        } else if (vec4 && d.nbands == 4) {
            reinterpret_cast<float4*>(a)[0] = make_float4(av[0], av[1], av[2], av[3]);
        } else {
#pragma unroll
            for (uint32_t b = 0; b < VGB_MAX_BANDS; ++b)
                if (b < d.nbands) a[b] = av[b];
        }
    }
}

// quad q = i * (H - 1) + j (the host's loop order)
__device__ __forceinline__ void quad_corners(uint32_t q, uint32_t W, uint32_t H, uint32_t& a, uint32_t& b, uint32_t& c,
                                             uint32_t& d) {
    const uint32_t i = q / (H - 1), j = q % (H - 1);
    a = i + (j + 1) * W; b = i + 1 + j * W; c = i + j * W; d = i + 1 + (j + 1) * W;
}

__global__ void k_dem_quad_counts(const float* __restrict__ h, uint32_t W, uint32_t H, uint32_t* __restrict__ cnt) {
    const size_t nq = (size_t)(W - 1) * (H - 1);
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (size_t)gridDim.x * blockDim.x) {
        uint32_t a, b, c, d;
        quad_corners((uint32_t)q, W, H, a, b, c, d);
        const bool t0 = !isinf(h[a]) && !isinf(h[b]) && !isinf(h[c]);
        const bool t1 = !isinf(h[b]) && !isinf(h[a]) && !isinf(h[d]);
        cnt[q] = (t0 ? 1u : 0u) + (t1 ? 1u : 0u);
    }
}

// One block per chunk of 256 quads: the chunk's faces are one contiguous run of the index buffer
// (the scan's offsets), so they are assembled in shared memory and written out coalesced.
__global__ void __launch_bounds__(256) k_dem_faces(const float* __restrict__ h, uint32_t W, uint32_t H,
                                                   const uint32_t* __restrict__ off, uint32_t* __restrict__ idx) {
    __shared__ uint32_t stage[256 * 6];
    const size_t nq = (size_t)(W - 1) * (H - 1);
    for (size_t q0 = (size_t)blockIdx.x * 256; q0 < nq; q0 += (size_t)gridDim.x * 256) {
        const size_t q = q0 + threadIdx.x;
        const uint32_t base = off[q0];
        const uint32_t total = off[min(q0 + 256, nq)] - base;
        if (q < nq) {
            uint32_t a, b, c, d;
            quad_corners((uint32_t)q, W, H, a, b, c, d);
            uint32_t k = 3 * (off[q] - base);
            if (!isinf(h[a]) && !isinf(h[b]) && !isinf(h[c])) { stage[k++] = a; stage[k++] = b; stage[k++] = c; }
            if (!isinf(h[b]) && !isinf(h[a]) && !isinf(h[d])) { stage[k++] = b; stage[k++] = a; stage[k++] = d; }
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < 3 * total; i += 256) idx[3 * (size_t)base + i] = stage[i];
        __syncthreads();
    }
}

// Exclusive scan of 32-bit counts, 1024 per block; block totals to `sums`.
__global__ void k_scan_block(const uint32_t* __restrict__ in, uint32_t* __restrict__ out, size_t n,
                             uint32_t* __restrict__ sums) {
    __shared__ uint32_t warp_tot[32];
    const size_t i = (size_t)blockIdx.x * 1024 + threadIdx.x;
    const uint32_t v = i < n ? in[i] : 0u;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        uint32_t t = warp_tot[lane];
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;  // inclusive totals of warps
    }
    __syncthreads();
    const uint32_t base = w ? warp_tot[w - 1] : 0u;
    if (i < n) out[i] = base + x - v;
    if (threadIdx.x == 1023 && sums) sums[blockIdx.x] = base + x;
}

__global__ void k_scan_add(uint32_t* __restrict__ out, size_t n, const uint32_t* __restrict__ add) {
    const size_t i = (size_t)blockIdx.x * 1024 + threadIdx.x;
    if (i < n && blockIdx.x > 0) out[i] += add[blockIdx.x];
}

// Exclusive scan of n counts into out; tmp holds the per-level block sums (see scan_temp_words).
void scan(cudaStream_t s, const uint32_t* in, uint32_t* out, size_t n, uint32_t* tmp) {
    const size_t blocks = (n + 1023) / 1024;
    if (blocks <= 1) {
        k_scan_block<<<1, 1024, 0, s>>>(in, out, n, nullptr);
        return;
    }
    uint32_t* sums = tmp;
    uint32_t* sums_scanned = tmp + blocks;
    k_scan_block<<<(unsigned)blocks, 1024, 0, s>>>(in, out, n, sums);
    scan(s, sums, sums_scanned, blocks, tmp + 2 * blocks);
    k_scan_add<<<(unsigned)blocks, 1024, 0, s>>>(out, n, sums_scanned);
}

__global__ void k_face_normals(const float* __restrict__ pos, const uint32_t* __restrict__ idx, uint32_t nt,
                               float* __restrict__ fn) {
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < nt; t += (size_t)gridDim.x * blockDim.x) {
        const uint32_t i0 = idx[3 * t], i1 = idx[3 * t + 1], i2 = idx[3 * t + 2];
        const F3 p0{pos[3 * (size_t)i0], pos[3 * (size_t)i0 + 1], pos[3 * (size_t)i0 + 2]};
        const F3 p1{pos[3 * (size_t)i1], pos[3 * (size_t)i1 + 1], pos[3 * (size_t)i1 + 2]};
        const F3 p2{pos[3 * (size_t)i2], pos[3 * (size_t)i2 + 1], pos[3 * (size_t)i2 + 2]};
        F3 n{__int_as_float(0x7fc00000), 0.f, 0.f};  // NaN marks a face the sums skip
        if (!isinf(p0.x) && !isinf(p1.x) && !isinf(p2.x)) n = normalize(cross(p1 - p0, p2 - p0));
        fn[3 * t] = n.x; fn[3 * t + 1] = n.y; fn[3 * t + 2] = n.z;
    }
}

__global__ void k_check_indices(const uint32_t* __restrict__ idx, size_t ncorner, uint32_t nv, uint32_t* bad) {
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncorner; c += (size_t)gridDim.x * blockDim.x)
        if (idx[c] >= nv) { atomicOr(bad, 1u); return; }
}

__global__ void k_corner_counts(const uint32_t* __restrict__ idx, size_t ncorner, uint32_t* __restrict__ cnt) {
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncorner; c += (size_t)gridDim.x * blockDim.x)
        atomicAdd(&cnt[idx[c]], 1u);
}

__global__ void k_corner_fill(const uint32_t* __restrict__ idx, size_t ncorner, const uint32_t* __restrict__ off,
                              uint32_t* __restrict__ cursor, uint32_t* __restrict__ list) {
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < ncorner; c += (size_t)gridDim.x * blockDim.x) {
        const uint32_t v = idx[c];
        list[off[v] + atomicAdd(&cursor[v], 1u)] = (uint32_t)c;  // corner c = 3 t + k
    }
}

__global__ void k_vertex_normals(const float* __restrict__ fn, const uint32_t* __restrict__ off,
                                 const uint32_t* __restrict__ cnt, uint32_t* __restrict__ list, uint32_t nv,
                                 float* __restrict__ out) {
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += (size_t)gridDim.x * blockDim.x) {
        uint32_t* e = list + off[v];
        const uint32_t m = cnt[v];
        // insertion sort of this vertex's corners (their face order is the host's sum order)
        for (uint32_t a = 1; a < m; ++a) {
            const uint32_t key = e[a];
            uint32_t b = a;
            while (b > 0 && e[b - 1] > key) { e[b] = e[b - 1]; --b; }
            e[b] = key;
        }
        F3 n{0.f, 0.f, 0.f};
        for (uint32_t a = 0; a < m; ++a) {
            const size_t t = e[a] / 3;
            const F3 f{fn[3 * t], fn[3 * t + 1], fn[3 * t + 2]};
            if (isnan(f.x) || isnan(f.y) || isnan(f.z)) continue;
            n = n + f;
        }
        if (sqrtf(dot(n, n)) != 0.f) n = normalize(n);
        out[3 * v] = n.x; out[3 * v + 1] = n.y; out[3 * v + 2] = n.z;
    }
}

int grid(size_t n, int sms) { return (int)std::max<size_t>(1, std::min<size_t>((n + 255) / 256, (size_t)sms * 8)); }

}  // namespace

namespace vgb {

size_t scan_temp_words(size_t n) {
    size_t words = 0;
    for (size_t b = (n + 1023) / 1024; b > 1; b = (b + 1023) / 1024) words += 2 * b;
    return words + 64;
}

int launch_quipu_decode(void* stream, int sms, const QuipuDecode& d, const void* codes, const uint8_t* planes,
                        float* heights, float* alb) {
    cudaStream_t s = (cudaStream_t)stream;
    const int g = grid((size_t)d.W * d.H, sms);
    const bool vec4 = ((uintptr_t)alb & 15u) == 0 && (d.nbands == 4 || d.nbands == 8);
    if (d.precision == 3) k_quipu_decode<uint8_t><<<g, 256, 0, s>>>(d, (const uint8_t*)codes, planes, heights, alb, vec4);
    else if (d.precision == 4) k_quipu_decode<uint16_t><<<g, 256, 0, s>>>(d, (const uint16_t*)codes, planes, heights, alb, vec4);
    else k_quipu_decode<float><<<g, 256, 0, s>>>(d, (const float*)codes, planes, heights, alb, vec4);
    return (int)cudaGetLastError();
}

int launch_dem_triangulate(void* stream, int sms, const float* h, uint32_t W, uint32_t H, const DemPose& pose,
                           float* pos, uint32_t* idx, uint32_t* work, uint32_t* nt_out, float* nrm) {
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nq = (size_t)(W - 1) * (H - 1);
    uint32_t* cnt = work;
    uint32_t* off = work + nq + 1;
    float* xs = reinterpret_cast<float*>(off + nq + 1);
    float* ys = xs + W;
    uint32_t* tmp = reinterpret_cast<uint32_t*>(ys + H);
    k_dem_axes<<<grid((size_t)W + H, sms), 256, 0, s>>>(W, H, pose, xs, ys);
    if (nrm) k_dem_vertices<true><<<grid((size_t)W * H, sms), 256, 0, s>>>(h, W, H, xs, ys, pos, nrm);
    else k_dem_vertices<false><<<grid((size_t)W * H, sms), 256, 0, s>>>(h, W, H, xs, ys, pos, nullptr);
    k_dem_quad_counts<<<grid(nq, sms), 256, 0, s>>>(h, W, H, cnt);
    cudaMemsetAsync(cnt + nq, 0, sizeof(uint32_t), s);
    scan(s, cnt, off, nq + 1, tmp);  // off[nq] = total triangles
    k_dem_faces<<<grid(nq, sms), 256, 0, s>>>(h, W, H, off, idx);
    cudaMemcpyAsync(nt_out, off + nq, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    return e != cudaSuccess ? (int)e : (int)cudaGetLastError();
}

size_t dem_work_words(uint32_t W, uint32_t H) {
    const size_t nq = (size_t)(W - 1) * (H - 1);
    return 2 * (nq + 1) + (size_t)W + H + scan_temp_words(nq + 1);
}

size_t normals_work_words(uint32_t nv, uint32_t nt) {
    return 3 * (size_t)nt /* face normals */ + 3 * (size_t)nv + 2 /* counts, offsets, cursors */ +
           3 * (size_t)nt /* corner lists */ + scan_temp_words((size_t)nv + 1);
}

int launch_vertex_normals(void* stream, int sms, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt,
                          float* out, uint32_t* work) {
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nc = 3 * (size_t)nt;
    float* fn = reinterpret_cast<float*>(work);
    uint32_t* cnt = work + nc;
    uint32_t* off = cnt + nv + 1;
    uint32_t* cur = off + nv + 1;
    uint32_t* list = cur + nv;
    uint32_t* tmp = list + nc;
    // every index must name a vertex: the gathers below index per-vertex arrays with them
    cudaMemsetAsync(cnt, 0, sizeof(uint32_t), s);
    k_check_indices<<<grid(nc, sms), 256, 0, s>>>(idx, nc, nv, cnt);
    uint32_t bad = 0;
    cudaMemcpyAsync(&bad, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e0 = cudaStreamSynchronize(s);
    if (e0 != cudaSuccess) return (int)e0;
    if (bad) return -1;
    cudaMemsetAsync(cnt, 0, ((size_t)nv + 1) * sizeof(uint32_t), s);
    cudaMemsetAsync(cur, 0, (size_t)nv * sizeof(uint32_t), s);
    k_face_normals<<<grid(nt, sms), 256, 0, s>>>(pos, idx, nt, fn);
    k_corner_counts<<<grid(nc, sms), 256, 0, s>>>(idx, nc, cnt);
    scan(s, cnt, off, (size_t)nv + 1, tmp);
    k_corner_fill<<<grid(nc, sms), 256, 0, s>>>(idx, nc, off, cur, list);
    k_vertex_normals<<<grid(nv, sms), 256, 0, s>>>(fn, off, cnt, list, nv, out);
    cudaError_t e = cudaStreamSynchronize(s);
    return e != cudaSuccess ? (int)e : (int)cudaGetLastError();
}

size_t vertex_normal_list_words(uint32_t nv, uint32_t nt) { return 2 * ((size_t)nv + 1) + 3 * (size_t)nt; }

int launch_vertex_normal_lists(void* stream, int sms, const uint32_t* idx, uint32_t nv, uint32_t nt, uint32_t* lists,
                               uint32_t* work) {
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nc = 3 * (size_t)nt;
    uint32_t* cnt = lists;
    uint32_t* off = cnt + nv + 1;
    uint32_t* list = off + nv + 1;
    uint32_t* cur = work;
    uint32_t* tmp = work + nv;
    cudaMemsetAsync(cnt, 0, sizeof(uint32_t), s);
    k_check_indices<<<grid(nc, sms), 256, 0, s>>>(idx, nc, nv, cnt);
    uint32_t bad = 0;
    cudaMemcpyAsync(&bad, cnt, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e0 = cudaStreamSynchronize(s);
    if (e0 != cudaSuccess) return (int)e0;
    if (bad) return -1;
    cudaMemsetAsync(cnt, 0, ((size_t)nv + 1) * sizeof(uint32_t), s);
    cudaMemsetAsync(cur, 0, (size_t)nv * sizeof(uint32_t), s);
    k_corner_counts<<<grid(nc, sms), 256, 0, s>>>(idx, nc, cnt);
    scan(s, cnt, off, (size_t)nv + 1, tmp);
    k_corner_fill<<<grid(nc, sms), 256, 0, s>>>(idx, nc, off, cur, list);
    cudaError_t e = cudaStreamSynchronize(s);
    return e != cudaSuccess ? (int)e : (int)cudaGetLastError();
}

int launch_vertex_normals_listed(void* stream, int sms, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt,
                                 uint32_t* lists, float* fn, float* out) {
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t* cnt = lists;
    uint32_t* off = cnt + nv + 1;
    uint32_t* list = off + nv + 1;
    k_face_normals<<<grid(nt, sms), 256, 0, s>>>(pos, idx, nt, fn);
    // the first call sorts each vertex's corners into face order in place; later calls find
    // them sorted (one comparison per corner)
    k_vertex_normals<<<grid(nv, sms), 256, 0, s>>>(fn, off, cnt, list, nv, out);
    return (int)cudaGetLastError();
}

}  // namespace vgb

// ---------------------------------------------------------------- BVH refit
namespace {

__global__ void k_refit_tris(const float4* __restrict__ vpos, const uint32_t* __restrict__ idx, uint32_t ntris,
                             float4* __restrict__ tris) {
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < ntris; r += (size_t)gridDim.x * blockDim.x) {
        const float idbits = tris[3 * r].w;
        const uint32_t t = __float_as_uint(idbits);
        const float4 a = vpos[idx[3 * (size_t)t]], b = vpos[idx[3 * (size_t)t + 1]], c = vpos[idx[3 * (size_t)t + 2]];
        tris[3 * r] = make_float4(a.x, a.y, a.z, idbits);
        tris[3 * r + 1] = make_float4(b.x, b.y, b.z, 0.f);
        tris[3 * r + 2] = make_float4(c.x, c.y, c.z, 0.f);
    }
}

struct RBox { float lx, hx, ly, hy, lz, hz; };

__device__ __forceinline__ uint32_t atomic_add_acq_rel(uint32_t* p, uint32_t v) {
    uint32_t old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ void put_box(uint32_t* nodes, uint32_t node, int side, const RBox& b) {
    uint32_t* n = nodes + 16 * (size_t)node;
    const int o = side ? 4 : 0;
    n[o + 0] = __float_as_uint(b.lx); n[o + 1] = __float_as_uint(b.hx);
    n[o + 2] = __float_as_uint(b.ly); n[o + 3] = __float_as_uint(b.hy);
    n[8 + 2 * side] = __float_as_uint(b.lz); n[9 + 2 * side] = __float_as_uint(b.hz);
}

__device__ __forceinline__ RBox get_box(const uint32_t* nodes, uint32_t node, int side) {
    const uint32_t* n = nodes + 16 * (size_t)node;
    const int o = side ? 4 : 0;
    // the other side was written by another thread: read through L2
    return RBox{__uint_as_float(__ldcg(n + o)), __uint_as_float(__ldcg(n + o + 1)), __uint_as_float(__ldcg(n + o + 2)),
                __uint_as_float(__ldcg(n + o + 3)), __uint_as_float(__ldcg(n + 8 + 2 * side)),
                __uint_as_float(__ldcg(n + 9 + 2 * side))};
}

// One thread per (node, side) whose child is a leaf: the leaf's box from its triangle records,
// then up the tree: the second of a node's two sides to finish writes that node's box into its
// parent.  Walks are bounded by `cap` steps (the tree depth); a walk that would exceed it flags.
__global__ void k_refit_nodes(const float4* __restrict__ tris, uint32_t* nodes, uint32_t nnodes,
                              const uint32_t* __restrict__ parent, uint32_t* counts, uint32_t cap, uint32_t* flag) {
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < 2 * (size_t)nnodes;
         q += (size_t)gridDim.x * blockDim.x) {
        uint32_t node = (uint32_t)(q >> 1);
        const int side = (int)(q & 1);
        const int32_t link = (int32_t)nodes[16 * (size_t)node + 12 + side];
        if (link >= 0) continue;
        const uint32_t x = ~(uint32_t)link;
        const uint32_t start = x >> 3, cnt = (x & 7u) + 1u;
        RBox b{INFINITY, -INFINITY, INFINITY, -INFINITY, INFINITY, -INFINITY};
        for (uint32_t k = 0; k < cnt; ++k)
            for (int v = 0; v < 3; ++v) {
                const float4 p = tris[3 * (size_t)(start + k) + v];
                b.lx = fminf(b.lx, p.x); b.hx = fmaxf(b.hx, p.x);
                b.ly = fminf(b.ly, p.y); b.hy = fmaxf(b.hy, p.y);
                b.lz = fminf(b.lz, p.z); b.hz = fmaxf(b.hz, p.z);
            }
        put_box(nodes, node, side, b);
        for (uint32_t step = 0;; ++step) {
            // release: this side's box is visible before the count; acquire: the other side's is
            // visible to the second arrival
            if (atomic_add_acq_rel(&counts[node], 1u) == 0u) break;  // the other side is not done yet
            if (step >= cap) { atomicOr(flag, 1u); break; }
            const RBox a = get_box(nodes, node, 0), c = get_box(nodes, node, 1);
            const RBox u{fminf(a.lx, c.lx), fmaxf(a.hx, c.hx), fminf(a.ly, c.ly),
                         fmaxf(a.hy, c.hy), fminf(a.lz, c.lz), fmaxf(a.hz, c.hz)};
            const uint32_t pr = parent[node];
            if (pr == vgb::kNoParent) break;
            node = pr >> 1;
            put_box(nodes, node, (int)(pr & 1u), u);
        }
    }
}

}  // namespace

namespace vgb {

int launch_refit(void* stream, int sms, const void* vpos, const uint32_t* idx, uint32_t ntris, void* tris,
                 uint32_t* nodes, uint32_t nnodes, const uint32_t* parent, uint32_t* counts) {
    cudaStream_t s = (cudaStream_t)stream;
    uint32_t* flag = counts + nnodes;
    cudaMemsetAsync(counts, 0, ((size_t)nnodes + 1) * sizeof(uint32_t), s);
    k_refit_tris<<<grid(ntris, sms), 256, 0, s>>>((const float4*)vpos, idx, ntris, (float4*)tris);
    k_refit_nodes<<<grid(2 * (size_t)nnodes, sms), 256, 0, s>>>((const float4*)tris, nodes, nnodes, parent, counts,
                                                                 4096u, flag);
    uint32_t bad = 0;
    cudaMemcpyAsync(&bad, flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return (int)e;
    return bad ? -2 : (int)cudaGetLastError();
}

}  // namespace vgb

// ---------------------------------------------------------------- GPU BVH build (binary layout)
// Linear BVH after Karras (HPG 2012): triangles sorted by the 63-bit Morton code of their
// centroid in the scene's bounding cube (ties by triangle index), internal nodes from the longest common prefixes of
// neighbouring keys, every node a contiguous range of the sorted triangles.  Nodes whose range
// holds at most `max_leaf` triangles become leaves of that range; the kept nodes are compacted
// in Karras order (the root stays node 0), the triangle records are written in sorted order, and
// the boxes come from the bottom-up refit.
namespace {

constexpr int kSortThreads = 256, kSortItems = 8, kSortTile = kSortThreads * kSortItems;

__device__ __forceinline__ uint32_t ordered(float f) {   // float -> uint32 preserving order
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unordered(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

__device__ __forceinline__ F3 centroid_of(const float4* __restrict__ vpos, const uint32_t* __restrict__ idx, size_t t) {
    const F3 a = ld3(vpos[idx[3 * t]]), b = ld3(vpos[idx[3 * t + 1]]), c = ld3(vpos[idx[3 * t + 2]]);
    return F3{(a.x + b.x + c.x) * (1.f / 3.f), (a.y + b.y + c.y) * (1.f / 3.f), (a.z + b.z + c.z) * (1.f / 3.f)};
}

// bounds of the finite centroids: lo[3], hi[3] as ordered uint32 (lo initialised to ~0, hi to 0)
__global__ void k_centroid_bounds(const float4* __restrict__ vpos, const uint32_t* __restrict__ idx, uint32_t n,
                                  uint32_t* __restrict__ bounds) {
    uint32_t lo[3] = {~0u, ~0u, ~0u}, hi[3] = {0u, 0u, 0u};
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const F3 c = centroid_of(vpos, idx, t);
        const float v[3] = {c.x, c.y, c.z};
        if (!(isfinite(v[0]) && isfinite(v[1]) && isfinite(v[2]))) continue;
#pragma unroll
        for (int k = 0; k < 3; ++k) { lo[k] = min(lo[k], ordered(v[k])); hi[k] = max(hi[k], ordered(v[k])); }
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            lo[k] = min(lo[k], __shfl_xor_sync(0xffffffffu, lo[k], o));
            hi[k] = max(hi[k], __shfl_xor_sync(0xffffffffu, hi[k], o));
        }
    }
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k) { atomicMin(&bounds[k], lo[k]); atomicMax(&bounds[3 + k], hi[k]); }
    }
}

using MKey = unsigned long long;

__device__ __forceinline__ MKey spread21(uint32_t v) {   // 21 bits -> every third bit of 63
    MKey x = v & 0x1FFFFFull;
    x = (x | (x << 32)) & 0x1F00000000FFFFull;
    x = (x | (x << 16)) & 0x1F0000FF0000FFull;
    x = (x | (x << 8)) & 0x100F00F00F00F00Full;
    x = (x | (x << 4)) & 0x10C30C30C30C30C3ull;
    x = (x | (x << 2)) & 0x1249249249249249ull;
    return x;
}

__global__ void k_morton(const float4* __restrict__ vpos, const uint32_t* __restrict__ idx, uint32_t n,
                         const uint32_t* __restrict__ bounds, MKey* __restrict__ keys, uint32_t* __restrict__ vals) {
    // one scale for all three axes (the largest extent): a flat terrain's heights then take few
    // of the code's bits instead of a third of them, so the splits stay mostly horizontal
    float lo[3], ext[3], emax = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        lo[k] = bounds[k] == ~0u ? 0.f : unordered(bounds[k]);
        const float h = bounds[k] == ~0u ? 0.f : unordered(bounds[3 + k]);
        emax = fmaxf(emax, h - lo[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; ++k) ext[k] = emax;
    for (size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (size_t)gridDim.x * blockDim.x) {
        const F3 c = centroid_of(vpos, idx, t);
        const float v[3] = {c.x, c.y, c.z};
        uint32_t q[3];
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            const float u = ext[k] > 0.f ? (v[k] - lo[k]) / ext[k] : 0.f;
            const float sc = u * 2097152.f;
            q[k] = (sc >= 2097151.f) ? 2097151u : (sc > 0.f ? (uint32_t)sc : 0u);   // NaN -> 0
        }
        keys[t] = (spread21(q[0]) << 2) | (spread21(q[1]) << 1) | spread21(q[2]);
        vals[t] = (uint32_t)t;
    }
}

// LSD radix sort, 8-bit digits: per-tile digit counts (digit-major over tiles) ...
__global__ void k_sort_hist(const MKey* __restrict__ keys, uint32_t n, int shift, uint32_t ntiles,
                            uint32_t* __restrict__ counts) {
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const size_t base = (size_t)blockIdx.x * kSortTile;
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const size_t i = base + (size_t)j * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[(keys[i] >> shift) & 0xFFu], 1u);
    }
    __syncthreads();
    counts[(size_t)threadIdx.x * ntiles + blockIdx.x] = h[threadIdx.x];
}

// ... then a stable scatter: within a tile each warp owns 256 consecutive keys (8 rounds of 32),
// ranks come from __match_any_sync and per-warp running digit counts, warps are ordered by an
// exclusive prefix over the warps, tiles by the scanned counts.
__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(const MKey* __restrict__ keys,
                                                               const uint32_t* __restrict__ vals, uint32_t n, int shift,
                                                               uint32_t ntiles, const uint32_t* __restrict__ offsets,
                                                               MKey* __restrict__ okeys, uint32_t* __restrict__ ovals) {
    __shared__ uint32_t wcnt[kSortThreads / 32][256];
    __shared__ uint32_t toff[256];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = lane; d < 256; d += 32) wcnt[w][d] = 0;
    toff[threadIdx.x] = offsets[(size_t)threadIdx.x * ntiles + blockIdx.x];
    __syncwarp();
    const size_t base = (size_t)blockIdx.x * kSortTile + (size_t)w * 32 * kSortItems;
    const uint32_t lt = (1u << lane) - 1u;
    MKey k[kSortItems];
    uint32_t v[kSortItems], rank[kSortItems];
    int dg[kSortItems];
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        const size_t i = base + (size_t)j * 32 + lane;
        const bool ok = i < n;
        k[j] = ok ? keys[i] : 0ull;
        v[j] = ok ? vals[i] : 0u;
        dg[j] = ok ? (int)((k[j] >> shift) & 0xFFu) : 256 + lane;   // invalid lanes match only themselves
        const uint32_t m = __match_any_sync(0xffffffffu, dg[j]);
        const uint32_t lower = __popc(m & lt);
        uint32_t b = 0;
        if (ok) b = wcnt[w][dg[j]];
        __syncwarp();
        if (ok && lower == 0) wcnt[w][dg[j]] = b + (uint32_t)__popc(m);
        __syncwarp();
        rank[j] = b + lower;
    }
    __syncthreads();
    {   // exclusive prefix over the warps, per digit
        uint32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < kSortThreads / 32; ++ww) {
            const uint32_t c = wcnt[ww][threadIdx.x];
            wcnt[ww][threadIdx.x] = run;
            run += c;
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < kSortItems; ++j) {
        if (dg[j] >= 256) continue;
        const uint32_t pos = toff[dg[j]] + wcnt[w][dg[j]] + rank[j];
        okeys[pos] = k[j];
        ovals[pos] = v[j];
    }
}

__device__ __forceinline__ int lcp(const MKey* __restrict__ keys, uint32_t n, int64_t i, int64_t j) {
    if (j < 0 || j >= (int64_t)n) return -1;
    const MKey a = keys[i], b = keys[j];
    if (a != b) return __clzll((long long)(a ^ b));
    return 64 + __clz((uint32_t)i ^ (uint32_t)j);
}

// Karras internal node i: its range [first, last] and split g (left child covers [first, g]).
__global__ void k_karras(const MKey* __restrict__ keys, uint32_t n, uint32_t* __restrict__ first,
                         uint32_t* __restrict__ last, uint32_t* __restrict__ split) {
    for (size_t ii = (size_t)blockIdx.x * blockDim.x + threadIdx.x; ii + 1 < n; ii += (size_t)gridDim.x * blockDim.x) {
        const int64_t i = (int64_t)ii;
        const int d = (lcp(keys, n, i, i + 1) - lcp(keys, n, i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = lcp(keys, n, i, i - d);
        int64_t lmax = 2;
        while (lcp(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
        int64_t l = 0;
        for (int64_t t = lmax / 2; t >= 1; t /= 2)
            if (lcp(keys, n, i, i + (l + t) * d) > dmin) l += t;
        const int64_t j = i + l * d;
        const int dnode = lcp(keys, n, i, j);
        int64_t s = 0;
        for (int64_t div = 2;; div *= 2) {
            const int64_t t = (l + div - 1) / div;
            if (lcp(keys, n, i, i + (s + t) * d) > dnode) s += t;
            if (t == 1) break;
        }
        const int64_t g = i + s * d + (d < 0 ? -1 : 0);
        first[i] = (uint32_t)(i < j ? i : j);
        last[i] = (uint32_t)(i < j ? j : i);
        split[i] = (uint32_t)g;
    }
}

__global__ void k_lbvh_keep(const uint32_t* __restrict__ first, const uint32_t* __restrict__ last, uint32_t n,
                            uint32_t max_leaf, uint32_t* __restrict__ kept) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i + 1 < n; i += (size_t)gridDim.x * blockDim.x)
        kept[i] = (last[i] - first[i] + 1u > max_leaf) ? 1u : 0u;
}

__global__ void k_lbvh_emit(const uint32_t* __restrict__ first, const uint32_t* __restrict__ last,
                            const uint32_t* __restrict__ split, const uint32_t* __restrict__ kept,
                            const uint32_t* __restrict__ newidx, uint32_t n, uint32_t max_leaf,
                            uint32_t* __restrict__ nodes, uint32_t* __restrict__ parent) {
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i + 1 < n; i += (size_t)gridDim.x * blockDim.x) {
        if (!kept[i]) continue;
        const uint32_t me = newidx[i], g = split[i];
        const uint32_t cf[2] = {first[i], g + 1u}, cl[2] = {g, last[i]};
        uint32_t* nd = nodes + 16 * (size_t)me;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            const uint32_t cnt = cl[s] - cf[s] + 1u;
            int32_t link;
            if (cnt <= max_leaf) {
                link = ~(int32_t)((cf[s] << vgb::kLeafShift) | (cnt - 1u));
            } else {
                const uint32_t c = newidx[g + (uint32_t)s];   // the child is internal node g (left) or g + 1 (right)
                link = (int32_t)c;
                parent[c] = (me << 1) | (uint32_t)s;
            }
            nd[12 + s] = (uint32_t)link;
        }
        nd[14] = nd[15] = 0u;
        if (i == 0) parent[me] = vgb::kNoParent;
    }
}

__global__ void k_lbvh_tris(const float4* __restrict__ vpos, const uint32_t* __restrict__ idx,
                            const uint32_t* __restrict__ order, uint32_t n, float4* __restrict__ tris) {
    for (size_t r = (size_t)blockIdx.x * blockDim.x + threadIdx.x; r < n; r += (size_t)gridDim.x * blockDim.x) {
        const uint32_t t = order[r];
        const float4 a = vpos[idx[3 * (size_t)t]], b = vpos[idx[3 * (size_t)t + 1]], c = vpos[idx[3 * (size_t)t + 2]];
        tris[3 * r] = make_float4(a.x, a.y, a.z, __uint_as_float(t));
        tris[3 * r + 1] = make_float4(b.x, b.y, b.z, 0.f);
        tris[3 * r + 2] = make_float4(c.x, c.y, c.z, 0.f);
    }
}

}  // namespace

namespace vgb {

// work: keys (64-bit) x2, triangle order x2, tile digit counts and their scan, Karras ranges and
// splits, kept flags and their scan, centroid bounds
struct LbvhWork {
    MKey *keys, *keys2;
    uint32_t *vals, *vals2, *counts, *offs, *stmp, *first, *last, *split, *kept, *newidx, *ktmp, *bounds;
    size_t words;
};

LbvhWork lbvh_layout(uint32_t* w, uint32_t n) {
    const size_t tiles = ((size_t)n + kSortTile - 1) / kSortTile;
    LbvhWork L;
    size_t o = 0;
    auto take = [&](size_t words) { uint32_t* p = w ? w + o : nullptr; o += (words + 1) & ~(size_t)1; return p; };
    L.keys = reinterpret_cast<MKey*>(take(2 * (size_t)n));
    L.keys2 = reinterpret_cast<MKey*>(take(2 * (size_t)n));
    L.vals = take(n); L.vals2 = take(n);
    L.counts = take(256 * tiles); L.offs = take(256 * tiles); L.stmp = take(scan_temp_words(256 * tiles));
    L.first = take(n); L.last = take(n); L.split = take(n);
    L.kept = take((size_t)n + 1); L.newidx = take((size_t)n + 1); L.ktmp = take(scan_temp_words((size_t)n + 1));
    L.bounds = take(8);
    L.words = o;
    return L;
}

size_t lbvh_work_words(uint32_t n) { return lbvh_layout(nullptr, n).words; }

int launch_lbvh_sort_and_link(void* stream, int sms, const void* vpos_, const uint32_t* idx, uint32_t n,
                              uint32_t max_leaf, uint32_t* work, uint32_t* nkept_out) {
    cudaStream_t s = (cudaStream_t)stream;
    const float4* vpos = (const float4*)vpos_;
    const size_t tiles = ((size_t)n + kSortTile - 1) / kSortTile;
    LbvhWork L = lbvh_layout(work, n);
    const uint32_t init[6] = {~0u, ~0u, ~0u, 0u, 0u, 0u};
    cudaMemcpyAsync(L.bounds, init, sizeof(init), cudaMemcpyHostToDevice, s);
    k_centroid_bounds<<<grid(n, sms), 256, 0, s>>>(vpos, idx, n, L.bounds);
    k_morton<<<grid(n, sms), 256, 0, s>>>(vpos, idx, n, L.bounds, L.keys, L.vals);
    MKey *keys = L.keys, *keys2 = L.keys2;
    uint32_t *vals = L.vals, *vals2 = L.vals2;
    for (int pass = 0; pass < 8; ++pass) {
        const int shift = 8 * pass;
        k_sort_hist<<<(unsigned)tiles, kSortThreads, 0, s>>>(keys, n, shift, (uint32_t)tiles, L.counts);
        scan(s, L.counts, L.offs, 256 * tiles, L.stmp);
        k_sort_scatter<<<(unsigned)tiles, kSortThreads, 0, s>>>(keys, vals, n, shift, (uint32_t)tiles, L.offs, keys2, vals2);
        std::swap(keys, keys2);
        std::swap(vals, vals2);
    }
    // after eight passes the sorted keys and order are back in the first arrays
    k_karras<<<grid(n, sms), 256, 0, s>>>(L.keys, n, L.first, L.last, L.split);
    k_lbvh_keep<<<grid(n, sms), 256, 0, s>>>(L.first, L.last, n, max_leaf, L.kept);
    cudaMemsetAsync(L.kept + (n - 1), 0, 2 * sizeof(uint32_t), s);
    scan(s, L.kept, L.newidx, (size_t)n, L.ktmp);   // newidx[n - 1] = number kept
    cudaMemcpyAsync(nkept_out, L.newidx + (n - 1), sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    return e != cudaSuccess ? (int)e : (int)cudaGetLastError();
}

int launch_lbvh_emit(void* stream, int sms, const void* vpos, const uint32_t* idx, uint32_t n, uint32_t max_leaf,
                     const uint32_t* work, uint32_t* nodes, uint32_t nnodes, void* tris, uint32_t* parent,
                     uint32_t* counts) {
    cudaStream_t s = (cudaStream_t)stream;
    const LbvhWork L = lbvh_layout(const_cast<uint32_t*>(work), n);
    const uint32_t *vals = L.vals, *first = L.first, *last = L.last, *split = L.split, *kept = L.kept,
                   *newidx = L.newidx;
    k_lbvh_tris<<<grid(n, sms), 256, 0, s>>>((const float4*)vpos, idx, vals, n, (float4*)tris);
    k_lbvh_emit<<<grid(n, sms), 256, 0, s>>>(first, last, split, kept, newidx, n, max_leaf, nodes, parent);
    // boxes: the refit over the new topology (triangle records are already in place)
    uint32_t* flag = counts + nnodes;
    cudaMemsetAsync(counts, 0, ((size_t)nnodes + 1) * sizeof(uint32_t), s);
    k_refit_nodes<<<grid(2 * (size_t)nnodes, sms), 256, 0, s>>>((const float4*)tris, nodes, nnodes, parent, counts,
                                                                 4096u, flag);
    uint32_t bad = 0;
    cudaMemcpyAsync(&bad, flag, sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return (int)e;
    return bad ? -2 : (int)cudaGetLastError();
}

}  // namespace vgb
