// vgb_internal.h -- layouts shared by the host builder and the CUDA kernels.
//
// Device BVH (binary, "two boxes per node"): one node is four 16-byte words.
//   w0 = (c0.lo.x, c0.hi.x, c0.lo.y, c0.hi.y)
//   w1 = (c1.lo.x, c1.hi.x, c1.lo.y, c1.hi.y)
//   w2 = (c0.lo.z, c0.hi.z, c1.lo.z, c1.hi.z)
//   w3 = (child0, child1, 0, 0) as int32: >= 0 inner node index, < 0 leaf ~(first << 3 | count-1)
// A leaf holds 1..8 consecutive triangle records.  The root is node 0; a scene whose root
// is a leaf gets one inner node whose two children are that leaf.
//
// Device BVH (compressed 8-wide): one node is five 16-byte words, see vgb_host.cpp.
//
// Triangle record (watertight test input), three 16-byte words in leaf order:
//   (v0.x, v0.y, v0.z, id as bits), (v1.xyz, 0), (v2.xyz, 0)
// id is the triangle's index in the caller's index buffer.
#pragma once
#include <cstdint>
#include <exception>
#include <limits>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "../../include/vgb.h"

#if defined(__CUDACC__)
#define VGB_HD __host__ __device__
#else
#define VGB_HD
#endif

namespace vgb {

// Entry points return statuses and let no exception cross the C boundary: each exported
// function's body is a function-try-block whose handler calls this inside the catch, for the
// status of the exception in flight (VGB_ERR_OUT_OF_MEMORY for a failed host allocation) and
// its message in *err (when err is not null).
inline vgb_status status_of_exception(std::string* err) noexcept {
    vgb_status s = VGB_ERR_INTERNAL;
    const char* msg = "unknown exception";
    try {
        throw;
    } catch (const std::bad_alloc&) {
        s = VGB_ERR_OUT_OF_MEMORY;
        msg = "host allocation failed";
    } catch (const std::exception& e) {
        msg = e.what();
    } catch (...) {
    }
    if (err) {
        try {
            *err = msg;
        } catch (...) {
        }
    }
    return s;
}

// Runs body(k) for k = 0..n-1, each on its own thread (k = 0 on the calling thread).  A thread
// that cannot start leaves its k to the calling thread; an exception thrown by any body is
// rethrown here after every thread has joined, so none escapes a thread and no thread is left
// running when the caller unwinds.
template <class F>
void parallel_for_each(uint32_t n, F&& body) {
    if (n == 0) return;
    std::vector<std::exception_ptr> errs(n);
    auto run = [&](uint32_t k) noexcept {
        try {
            body(k);
        } catch (...) {
            errs[k] = std::current_exception();
        }
    };
    std::vector<std::thread> th;
    th.reserve(n);
    uint32_t handed = 1;
    try {
        for (; handed < n; ++handed) th.emplace_back(run, handed);
    } catch (...) {
    }
    for (uint32_t k = handed; k < n; ++k) run(k);
    run(0);
    for (std::thread& t : th) t.join();
    for (const std::exception_ptr& e : errs)
        if (e) std::rethrow_exception(e);
}

constexpr int kLeafShift = 3;
constexpr uint32_t kMaxLeaf = 8;
constexpr uint32_t kMaxLeaf8 = 3;   // triangles per leaf child of an 8-wide node

struct BvhHost {
    uint32_t layout = 2;           // 2: binary (16 words per node), 8: compressed 8-wide (20 words)
    std::vector<uint32_t> nodes;
    std::vector<float> tris;       // 12 floats per triangle record
    uint32_t num_nodes = 0;
    uint32_t max_depth = 0;
    float root_lo[3] = {0, 0, 0}, root_hi[3] = {0, 0, 0};
    // binary layout: per node (parent << 1 | side), kNoParent for the root (bottom-up refits)
    std::vector<uint32_t> parent;
};
constexpr uint32_t kNoParent = 0xFFFFFFFFu;

// Binned-SAH build over the triangles of (positions, indices), emitted in the binary layout or
// collapsed into the compressed 8-wide layout.  Deterministic for a given input, leaf size and
// layout, whatever the thread count.
bool build_bvh(const float* positions, uint32_t nverts, const uint32_t* indices, uint32_t ntris,
               uint32_t max_leaf, uint32_t threads, uint32_t layout, BvhHost& out, const char** err);

// L2 read-bandwidth probe (vgb_probe.cu): `passes` streaming reads (ld.global.cg) of `bytes` of
// device memory at `buf` (16-byte aligned, a multiple of 16 bytes); sink: one device word.
int launch_l2_read(void* stream, const void* buf, size_t bytes, uint32_t passes, uint32_t* sink, int num_sms);

// Sensor chain and PSF kernels (vgb_sensor.cu); the C ABI in vgb_cuda.cu validates and stages
// the planes and calls these on the context's stream.  All pointers are device memory.
struct SensorParams {
    float exposure_time, photon_energy[8], quantum_efficiency[8], gain, max_adu;
    uint32_t photon_noise, noise_model;
    float dark_current, readout_mean, readout_std, hscale, vscale;
    uint32_t hperiod, vperiod, frame;
    uint64_t seed;
    const float* mosaic;
};
int launch_sensor(void* stream, const float* power, uint32_t width, uint32_t height, uint32_t nbands,
                  const SensorParams& sp, float* image, int num_sms);
// The RGB sensor (vgb_sensor_simulate_rgb): the conversion constants of vgb_rgb_conversion.
struct RgbParams {
    float band_min[8], band_max[8], rgb_min[3], rgb_max[3], rgb_bw[3], rgb_pe[3], rgb_qe[3];
};
int launch_sensor_rgb(void* stream, const float* power, uint32_t width, uint32_t height, uint32_t nbands,
                      const SensorParams& sp, const RgbParams& rp, float* image_rgb, int num_sms);
// out = correlation of in ([B][H][W]) with kernel ([B][kh][kw], zero padding); out != in.
int launch_psf(void* stream, const float* in, float* out, uint32_t width, uint32_t height, uint32_t nbands,
               const float* kernel, uint32_t kw, uint32_t kh);

// DEM triangulation and vertex normals (vgb_mesh.cu), equal to the host functions; all pointers
// device memory; `work` is scratch of dem_work_words / normals_work_words 32-bit words.
size_t dem_work_words(uint32_t W, uint32_t H);
size_t normals_work_words(uint32_t nv, uint32_t nt);
// DEMProjection's non-OGR mapping (dem_projection.ipp:66-71, 131-141) as FP64 constants:
//   x = ax * (-half_x + 2 * ((i + xo) * scale_x)),  y = ay * (half_y + 2 * (-(j + yo) * scale_y))
// with ax = dx * pixelScale[0], xo = xoff / dx, half_x = (Wp - 1) / 2, scale_x = (half_x + 0.5) / Wp
// for the projection's resolution Wp (and the same in y).
struct DemPose {
    double ax, ay, xo, yo, half_x, half_y, scale_x, scale_y;
};
inline DemPose dem_pose_of(double ax, double ay, double xo, double yo, uint32_t pw, uint32_t ph) {
    DemPose p;
    p.ax = ax; p.ay = ay; p.xo = xo; p.yo = yo;
    p.half_x = ((double)pw - 1.) / 2.;
    p.half_y = ((double)ph - 1.) / 2.;
    p.scale_x = (p.half_x + 0.5) / (double)pw;
    p.scale_y = (p.half_y + 0.5) / (double)ph;
    return p;
}
inline DemPose dem_pose(const vgb_quipu_projection& pr) {
    return dem_pose_of(pr.dx * pr.pixel_scale[0], pr.dy * pr.pixel_scale[1], pr.xoff / pr.dx, pr.yoff / pr.dy,
                       pr.width, pr.height);
}
// DEM::makeVertexBuffer positions and imageToIndexBuffer faces on the host (vgb_host.cpp).
void dem_vertices_host(const float* h, uint32_t W, uint32_t H, const DemPose& pose, float* pos);
void dem_faces_host(const float* h, uint32_t W, uint32_t H, uint32_t* idx, uint32_t* nt_out);
// nrm (optional): vertex normals of the grid's mesh, equal to launch_vertex_normals on its arrays.
int launch_dem_triangulate(void* stream, int sms, const float* h, uint32_t W, uint32_t H, const DemPose& pose,
                           float* pos, uint32_t* idx, uint32_t* work, uint32_t* nt_out, float* nrm = nullptr);
int launch_vertex_normals(void* stream, int sms, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt,
                          float* out, uint32_t* work);
// Vertex normals of a mesh whose topology stays while its vertices move: the per-vertex corner
// lists (counts, offsets, corners: vertex_normal_list_words) are built once, `work` holding
// nv + scan_temp_words(nv + 1) words; each evaluation then forms the face normals (fn: 3 nt
// floats) and the ordered sums -- the same normals as launch_vertex_normals.
size_t scan_temp_words(size_t n);   // scratch of the device exclusive scan of n words
size_t vertex_normal_list_words(uint32_t nv, uint32_t nt);
int launch_vertex_normal_lists(void* stream, int sms, const uint32_t* idx, uint32_t nv, uint32_t nt, uint32_t* lists,
                               uint32_t* work);
int launch_vertex_normals_listed(void* stream, int sms, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt,
                                 uint32_t* lists, float* fn, float* out);
// GPU build of the binary BVH (linear BVH, Morton order): sort and link into `work`
// (lbvh_work_words), returning the number of nodes kept; then emit nodes, triangle records and
// parents into arrays of that size and compute the boxes.  counts: nnodes + 1 words of scratch.
size_t lbvh_work_words(uint32_t ntris);
int launch_lbvh_sort_and_link(void* stream, int sms, const void* vpos, const uint32_t* idx, uint32_t ntris,
                              uint32_t max_leaf, uint32_t* work, uint32_t* nkept_out);
int launch_lbvh_emit(void* stream, int sms, const void* vpos, const uint32_t* idx, uint32_t ntris, uint32_t max_leaf,
                     const uint32_t* work, uint32_t* nodes, uint32_t nnodes, void* tris, uint32_t* parent,
                     uint32_t* counts);
// Refit of the binary BVH after the vertices moved (same triangles): triangle records rewritten
// from vpos, then every child box recomputed bottom up.  counts: nnodes words of scratch.
// Returns nonzero on a CUDA error, -2 when an upward walk exceeded its bound.
int launch_refit(void* stream, int sms, const void* vpos /* float4 */, const uint32_t* idx, uint32_t ntris,
                 void* tris /* float4 */, uint32_t* nodes, uint32_t nnodes, const uint32_t* parent, uint32_t* counts);


// ---- DEM Quipu (vgb_quipu.cpp host side, vgb_mesh.cu device decode)
// fixedToFloat (image_utils.ipp:509-527): code 0 is +inf, else (max - min) * (code / (m - 1)) + min
VGB_HD inline float quipu_dequantize(uint32_t code, float m, float mn, float mx) {
    if (code == 0) {
#if defined(__CUDA_ARCH__)
        return __int_as_float(0x7f800000);
#else
        return std::numeric_limits<float>::infinity();
#endif
    }
    const float f = (float)code / (m - 1.f);
    return ((mx - mn) * f) + mn;
}
struct ImageRefView {          // an image's pixels in the file
    uint64_t pos, stored, raw_bytes;
    uint32_t w, h, elem;
    bool compressed;
};
struct QuipuPlane { float mn, mx; ImageRefView img; };
struct QuipuPayload {
    std::string path;
    ImageRefView heights;
    uint32_t precision;        // 3 uint8, 4 uint16, 1 float
    float hmin, hmax;
    uint32_t albedo_type;      // 0 constant, 1 grey, 2 per band, VGB_QUIPU_NO_ALBEDO
    uint64_t constant_pos;
    std::vector<QuipuPlane> planes;
    vgb_quipu_projection proj;
};
vgb_status quipu_lod_payload(const vgb_quipu_dem* q, uint32_t lod, QuipuPayload* out);
// Row-major pixels of an image (LZ4-decoded, or transposed from the stored column order).
vgb_status quipu_read_pixels(const std::string& path, const ImageRefView& v, void* out);
vgb_status quipu_read_constant(const std::string& path, uint64_t pos, uint32_t nbands, float* out);
void quipu_set_error(const std::string& m);
// Device decode of one LoD: float heights [H][W] from the stored codes, and per-vertex albedo
// [H*W][nbands] (alb may be null).  planes: the uint8 albedo planes, one after the other.
struct QuipuDecode {
    uint32_t W, H, precision, albedo_type, nplanes, nbands;
    float hmin, hmax;
    float pmin[VGB_MAX_BANDS], pmax[VGB_MAX_BANDS];   // per-plane fixed-point range
    float constant[VGB_MAX_BANDS];                     // constant / default albedo
    float profile[VGB_MAX_BANDS];                      // grey-plane profile
};
int launch_quipu_decode(void* stream, int sms, const QuipuDecode& d, const void* codes, const uint8_t* planes,
                        float* heights, float* alb);

}  // namespace vgb
