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
#include <vector>

namespace vgb {

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
};

// Binned-SAH build over the triangles of (positions, indices), emitted in the binary layout or
// collapsed into the compressed 8-wide layout.  Deterministic for a given input, leaf size and
// layout, whatever the thread count.
bool build_bvh(const float* positions, uint32_t nverts, const uint32_t* indices, uint32_t ntris,
               uint32_t max_leaf, uint32_t threads, uint32_t layout, BvhHost& out, const char** err);

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
// out = correlation of in ([B][H][W]) with kernel ([B][kh][kw], zero padding); out != in.
int launch_psf(void* stream, const float* in, float* out, uint32_t width, uint32_t height, uint32_t nbands,
               const float* kernel, uint32_t kw, uint32_t kh);

// DEM triangulation and vertex normals (vgb_mesh.cu), equal to the host functions; all pointers
// device memory; `work` is scratch of dem_work_words / normals_work_words 32-bit words.
size_t dem_work_words(uint32_t W, uint32_t H);
size_t normals_work_words(uint32_t nv, uint32_t nt);
int launch_dem_triangulate(void* stream, int sms, const float* h, uint32_t W, uint32_t H, double sx, double sy,
                           float* pos, uint32_t* idx, uint32_t* work, uint32_t* nt_out);
int launch_vertex_normals(void* stream, int sms, const float* pos, uint32_t nv, const uint32_t* idx, uint32_t nt,
                          float* out, uint32_t* work);

}  // namespace vgb
