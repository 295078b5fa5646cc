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

namespace {

__global__ void k_dem_vertices(const float* __restrict__ h, uint32_t W, uint32_t H, double sx, double sy,
                               float* __restrict__ pos) {
    const double half_x = ((double)W - 1.) / 2., half_y = ((double)H - 1.) / 2.;
    const double scale_x = (half_x + 0.5) / (double)W, scale_y = (half_y + 0.5) / (double)H;
    const size_t n = (size_t)W * H;
    for (size_t v = (size_t)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (size_t)gridDim.x * blockDim.x) {
        const uint32_t i = (uint32_t)(v % W), j = (uint32_t)(v / W);
        const float z = h[v];
        if (isinf(z) || isnan(z)) {
            pos[3 * v] = pos[3 * v + 1] = pos[3 * v + 2] = __int_as_float(0x7f800000);
            continue;
        }
        const double xs = (double)i * scale_x, ys = -(double)j * scale_y;
        pos[3 * v] = (float)((1.0 * sx) * (-half_x + 2. * xs));
        pos[3 * v + 1] = (float)((1.0 * sy) * (half_y + 2. * ys));
        pos[3 * v + 2] = z;
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

__global__ void k_dem_faces(const float* __restrict__ h, uint32_t W, uint32_t H, const uint32_t* __restrict__ off,
                            uint32_t* __restrict__ idx) {
    const size_t nq = (size_t)(W - 1) * (H - 1);
    for (size_t q = (size_t)blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += (size_t)gridDim.x * blockDim.x) {
        uint32_t a, b, c, d;
        quad_corners((uint32_t)q, W, H, a, b, c, d);
        size_t k = 3 * (size_t)off[q];
        if (!isinf(h[a]) && !isinf(h[b]) && !isinf(h[c])) { idx[k++] = a; idx[k++] = b; idx[k++] = c; }
        if (!isinf(h[b]) && !isinf(h[a]) && !isinf(h[d])) { idx[k++] = b; idx[k++] = a; idx[k++] = d; }
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

int launch_dem_triangulate(void* stream, int sms, const float* h, uint32_t W, uint32_t H, double sx, double sy,
                           float* pos, uint32_t* idx, uint32_t* work, uint32_t* nt_out) {
    cudaStream_t s = (cudaStream_t)stream;
    const size_t nq = (size_t)(W - 1) * (H - 1);
    uint32_t* cnt = work;
    uint32_t* off = work + nq + 1;
    uint32_t* tmp = off + nq + 1;
    k_dem_vertices<<<grid((size_t)W * H, sms), 256, 0, s>>>(h, W, H, sx, sy, pos);
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
    return 2 * (nq + 1) + scan_temp_words(nq + 1);
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

}  // namespace vgb
