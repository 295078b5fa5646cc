// vgb.hpp -- C++ host API over the C ABI of vgb.h, shaped like Vira's scene / camera / path tracer.
//
// Vira's renderer object is CPUPathTracer with public `options`, `renderPasses` and
// render(Camera&, Scene&) (include/vira/rendering/cpu_path_tracer.hpp:46-58); Scene owns it as
// `pathtracer` and calls it from pathtraceRender (include/implementation/scene.ipp:840-845).
// vgb::GpuPathTracer keeps those names.  Poses, the sun position and the scene origin are FP64;
// everything is rebased into the local scene frame in FP64 before the FP32 cast.  Errors from
// the C ABI become vgb::Error (a std::runtime_error), as the reference reports errors.
#pragma once

#include <array>
#include <cmath>
#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <vector>

#include "vgb.h"

namespace vgb {

struct Error : std::runtime_error {
    vgb_status status;
    Error(vgb_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(vgb_status s, const vgb_context* ctx, const char* what) {
    if (s != VGB_OK) throw Error(s, std::string(what) + ": " + (ctx ? vgb_last_error(ctx) : "error"));
}

using Vec3 = std::array<double, 3>;
using Mat3 = std::array<double, 9>;  // column-major

inline Vec3 sub(const Vec3& a, const Vec3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
inline Vec3 cross(const Vec3& a, const Vec3& b) {
    return {a[1] * b[2] - b[1] * a[2], a[2] * b[0] - b[2] * a[0], a[0] * b[1] - b[0] * a[1]};
}
inline double dot(const Vec3& a, const Vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline Vec3 normalized(const Vec3& a) {
    const double s = 1.0 / std::sqrt(dot(a, a));
    return {a[0] * s, a[1] * s, a[2] * s};
}

// Band edges in metres, FP32 as SpectralData stores them (spectral_data.ipp:65-132).
struct SpectralBands {
    std::vector<float> lo, hi;
    static SpectralBands bounds(const std::vector<std::array<float, 2>>& nm) {
        SpectralBands b;
        for (auto& p : nm) {
            b.lo.push_back(std::fmin(p[0], p[1]) * 1e-9f);
            b.hi.push_back(std::fmax(p[0], p[1]) * 1e-9f);
        }
        return b;
    }
    static SpectralBands uniform(int n, float lo_nm, float hi_nm) {
        SpectralBands b;
        const float step = (hi_nm - lo_nm) / (float)n;
        for (int i = 0; i < n; ++i) {
            const float a = lo_nm + (float)i * step, c = lo_nm + (float)(i + 1) * step;
            b.lo.push_back(std::fmin(a, c) * 1e-9f);
            b.hi.push_back(std::fmax(a, c) * 1e-9f);
        }
        return b;
    }
    uint32_t size() const { return (uint32_t)lo.size(); }
    // TSpectral::photonEnergies: h c / centre wavelength in FP32 (spectral_data.ipp:125-128)
    std::vector<float> photonEnergies() const {
        std::vector<float> e;
        for (uint32_t i = 0; i < size(); ++i) e.push_back((6.62607015e-34f * 299792458.f) / ((lo[i] + hi[i]) / 2.f));
        return e;
    }
};

// PhotositeConfig (photosites/photosite.hpp:19-45); an empty quantum_efficiency means defaultQE.
struct PhotositeConfig {
    uint32_t bit_depth = 8;
    float gain = 0.333333f;
    float linear_scale_factor = 1.f;
    std::vector<float> quantum_efficiency;
    float maxADU() const { return linear_scale_factor * (std::pow(2.f, (float)bit_depth) - 1.f); }
};

// NoiseModelConfig (noise_models/noise_model.hpp:16-25)
struct NoiseModelConfig {
    float dark_current = 0, readout_noise_mean = 0, readout_noise_std = 0;
    float horizontal_scale = 0, vertical_scale = 0;
    uint32_t horizontal_pattern_period = 0, vertical_pattern_period = 0;
};

// blackBodyRadiance (spectral_data.ipp:613-629): trapezoid of Planck's law in FP64 per band.
inline std::vector<float> blackBodyRadiance(const SpectralBands& bands, double T, uint32_t steps = 1000) {
    const double c = 299792458.0, h = 6.62607015e-34, kB = 1.380649e-23;
    std::vector<float> out;
    for (uint32_t i = 0; i < bands.size(); ++i) {
        const double mn = bands.lo[i], mx = bands.hi[i], step = (mx - mn) / (double)(steps - 1);
        double area = 0, prev_l = mn, prev_r = 0;
        for (uint32_t k = 0; k < steps; ++k) {
            const double l = mn + (double)k * step;
            const double r = 2 * h * c * c / std::pow(l, 5.) * 1. / (std::exp(h * c / (l * kB * T)) - 1.);
            if (k) area += (l - prev_l) * (prev_r + r) / 2.;
            prev_l = l; prev_r = r;
        }
        out.push_back((float)area);
    }
    return out;
}

// Camera (camera.hpp:220-235 defaults), FP64 pose.
class Camera {
public:
    float focal_length = 0.05f, f_stop = 2.8f, aperture_diameter = 0.05f / 2.8f;
    uint32_t width = 1920, height = 1080;
    float sensor_x = 0.036f, sensor_y = 0.02025f;
    bool square_pixel = true, blender_frame = false;
    Vec3 position{0, 0, 0};
    Mat3 rotation{1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::vector<float> optical_efficiency{1.f};
    // the sensor chain after the film (Camera members, camera.hpp:215-268)
    float exposure_time = 0.01f;
    PhotositeConfig photosite;
    bool has_noise_model = false;
    NoiseModelConfig noise_model;
    bool simulate_photon_noise = false;
    uint64_t sensor_seed = 0;
    // lens distortion (Camera::set*DistortionCoefficients) and depth of field
    vgb_distortion_model distortion = VGB_DISTORTION_NONE;
    float distortion_coeffs[12] = {0};
    bool interpolate_distortion_directions = true;
    bool depth_of_field = false;
    float focus_distance = INFINITY;
    // the camera's own motion (global frame) for the velocity passes
    Vec3 velocity{0, 0, 0}, angular_rate{0, 0, 0};

    void setBrownDistortionCoefficients(float k1, float k2, float k3, float p1, float p2) {
        setDistortion(VGB_DISTORTION_BROWN, {k1, k2, k3, p1, p2});
    }
    void setOpenCVDistortionCoefficients(float k1, float k2, float k3, float k4, float k5, float k6, float p1, float p2,
                                         float s1, float s2, float s3, float s4) {
        setDistortion(VGB_DISTORTION_OPENCV, {k1, k2, k3, k4, k5, k6, p1, p2, s1, s2, s3, s4});
    }
    void setOwenDistortionCoefficients(float e1, float e2, float e3, float e4, float e5, float e6) {
        setDistortion(VGB_DISTORTION_OWEN, {e1, e2, e3, e4, e5, e6});
    }
    void enableDistortionInterpolation(bool on) { interpolate_distortion_directions = on; }
    void enableDepthOfField(bool on) { depth_of_field = on; }
    void setFocusDistance(double d) {
        if (std::isnan(d)) throw Error(VGB_ERR_INVALID_ARGUMENT, "Focus Distance must not be NaN");
        focus_distance = (float)d;
    }

    void setFocalLength(double f) { focal_length = (float)f; f_stop = (float)f / aperture_diameter; }
    void setFStop(double f) { f_stop = (float)f; aperture_diameter = focal_length / f_stop; }
    void setSensorSize(double x) {
        sensor_x = (float)x;
        sensor_y = (float)((double)height * (x / (double)width));
        square_pixel = true;
    }
    void setSensorSize(double x, double y) { sensor_x = (float)x; sensor_y = (float)y; square_pixel = false; }
    void setResolution(uint32_t x, uint32_t y) {
        width = x; height = y;
        if (square_pixel) setSensorSize(sensor_x);
    }
    void setFieldOfView(double deg) { setFocalLength(sensor_x / 2.0 / std::tan(deg * (M_PI / 180.0) / 2.0)); }
    void setLocalPosition(double x, double y, double z) { position = {x, y, z}; }
    void lookAt(const Vec3& target, Vec3 up = {0, 0, 1}) { lookInDirection(sub(target, position), up); }
    // Camera::lookInDirection (camera.ipp:1455-1500), FP64
    void lookInDirection(Vec3 d, Vec3 up = {0, 0, 1}) {
        up = normalized(up);
        d = normalized(d);
        if (std::fabs(dot(d, up)) > 0.999) {
            const Vec3 cand[3] = {{0, 1, 0}, {0, 0, 1}, {1, 0, 0}};
            for (auto& c : cand)
                if (std::fabs(dot(d, c)) < 0.999) { up = c; break; }
        }
        Vec3 y = blender_frame ? up : Vec3{-up[0], -up[1], -up[2]};
        Vec3 z = blender_frame ? Vec3{-d[0], -d[1], -d[2]} : d;
        Vec3 x = normalized(cross(y, z));
        y = normalized(cross(z, x));
        z = normalized(z);
        rotation = {x[0], x[1], x[2], y[0], y[1], y[2], z[0], z[1], z[2]};
    }
    vgb_camera toC(const Vec3& origin, uint32_t nbands) const {
        vgb_camera c{};
        c.width = width; c.height = height;
        for (int k = 0; k < 3; ++k) c.origin[k] = (float)(position[k] - origin[k]);
        for (int k = 0; k < 9; ++k) c.rotation[k] = (float)rotation[k];
        c.z_dir = blender_frame ? -1.f : 1.f;
        check(vgb_camera_intrinsics(focal_length, sensor_x, sensor_y, width, height, INFINITY, INFINITY, 0.f, 0.f,
                                    c.z_dir, c.kinv), nullptr, "camera_intrinsics");
        const float d = focal_length / f_stop, r = d / 2.f, area = 3.14159265358979323846f * r * r;
        for (uint32_t k = 0; k < nbands; ++k)
            c.power_scale[k] = optical_efficiency[optical_efficiency.size() == 1 ? 0 : k] * area;
        c.distortion = (uint32_t)distortion;
        for (int k = 0; k < 12; ++k) c.distortion_coeffs[k] = distortion_coeffs[k];
        c.interpolate_directions = interpolate_distortion_directions ? 1u : 0u;
        c.depth_of_field = depth_of_field ? 1u : 0u;
        c.aperture_radius = d / 2.f;
        c.focal_length = focal_length;
        c.focus_distance = focus_distance;
        c.sensor_size[0] = sensor_x;
        c.sensor_size[1] = sensor_y;
        for (int r = 0; r < 3; ++r) {
            c.velocity[r] = (float)velocity[r];
            c.angular_rate[r] = (float)angular_rate[r];
            // rotation * origin in FP64 (the velocity passes evaluate the camera's point velocity
            // at rotation * p_global, as the reference does)
            c.rot_origin[r] = (float)(rotation[r] * origin[0] + rotation[3 + r] * origin[1] + rotation[6 + r] * origin[2]);
        }
        return c;
    }

private:
    void setDistortion(vgb_distortion_model m, std::initializer_list<float> k) {
        distortion = m;
        int i = 0;
        for (float v : k) distortion_coeffs[i++] = v;
        for (; i < 12; ++i) distortion_coeffs[i] = 0.f;
    }
};

struct SphereLight {
    std::vector<float> radiance;
    float radius = 696000000.f;
    Vec3 position{0, 0, 0};
};

struct Mesh {
    std::vector<float> positions;   // 3 per vertex, mesh frame
    std::vector<uint32_t> indices;  // 3 per triangle
    std::vector<float> albedo;      // B per vertex (empty: 1)
    std::vector<float> uv;          // 2 per vertex (empty: 0)
    std::vector<float> albedo_map;  // [h][w][B] (empty: 1x1 of 1.0)
    uint32_t map_w = 0, map_h = 0;
    bool smooth_shading = false;

    // DEM::makeMesh with the non-OGR projection (dem.ipp:138-211)
    static Mesh fromDEM(const std::vector<float>& heights, uint32_t w, uint32_t h, double posting, float albedo,
                        uint32_t nbands) {
        Mesh m;
        m.positions.resize(3 * (size_t)w * h);
        m.indices.resize(6 * (size_t)(w - 1) * (h - 1));
        uint32_t nt = 0;
        check(vgb_dem_triangulate(heights.data(), w, h, posting, posting, m.positions.data(), m.indices.data(), &nt),
              nullptr, "dem_triangulate");
        m.indices.resize(3 * (size_t)nt);
        m.albedo.assign((size_t)w * h * nbands, albedo);
        return m;
    }
};

struct CPUPathTracerOptions {  // cpu_path_tracer.hpp:30-43, plus the RNG key and two additions
    size_t samples = 1;
    size_t bounces = 0;
    bool show_background = false;
    uint64_t seed = 0;
    uint32_t frame = 0;
    bool deterministic_light = false;
    uint32_t rr_depth = 0;
    bool denoise = false;                  // EATWT with the reference's default options
    bool adaptive_sampling = false;
    size_t samples_per_batch = 30;
    float sampling_tolerance = 0.05f;
    size_t samples_to_detect_miss = 30;
};

struct RenderPasses {  // passes.hpp:51-95, planar [B][H][W]
    bool simulate_lighting = false;
    bool save_velocity = false, save_triangle_size = false;
    uint32_t width = 0, height = 0, bands = 0;
    std::vector<float> total_radiance, direct_radiance, indirect_radiance, received_power, albedo, normal_global,
        depth, alpha;
    std::vector<uint32_t> triangle_id;
    // first-hit passes (passes.hpp:79-85): [3][H][W] velocities, [H][W] triangle size in pixels
    std::vector<float> velocity_global, velocity_camera, triangle_size;
};

class Scene;

class GpuPathTracer {
public:
    CPUPathTracerOptions options;
    RenderPasses renderPasses;
    void render(Camera& camera, Scene& scene);
};

class Scene {
public:
    explicit Scene(SpectralBands b, int device = 0) : bands(std::move(b)) {
        check(vgb_context_create(&ctx_, device), nullptr, "context_create");
        background.assign(bands.size(), 0.f);
    }
    ~Scene() { if (ctx_) vgb_context_destroy(ctx_); }
    Scene(const Scene&) = delete;
    Scene& operator=(const Scene&) = delete;

    SpectralBands bands;
    Vec3 origin{0, 0, 0};
    std::vector<Mesh> meshes;
    std::vector<SphereLight> lights;
    std::vector<float> ambient, background;
    GpuPathTracer pathtracer;

    size_t addMesh(Mesh m) { meshes.push_back(std::move(m)); dirty_ = true; return meshes.size() - 1; }
    size_t newSun(double temperature = 5800.0) {  // Group::newSun (scene/group.ipp:585-591)
        SphereLight s;
        s.radiance = blackBodyRadiance(bands, temperature, 1000);
        lights.push_back(s);
        return lights.size() - 1;
    }
    void setSunDirection(size_t id, double az_deg, double el_deg, double distance = 149597870700.0) {
        const double az = az_deg * (M_PI / 180.0), el = el_deg * (M_PI / 180.0);
        lights[id].position = {origin[0] + distance * std::cos(el) * std::cos(az),
                               origin[1] + distance * std::cos(el) * std::sin(az), origin[2] + distance * std::sin(el)};
    }
    void markDirty() { dirty_ = true; }

    // Scene::buildTLAS (scene.ipp:712-812): the first mesh is uploaded in the scene frame.
    void buildTLAS() {
        if (!dirty_) return;
        if (meshes.empty()) throw Error(VGB_ERR_INVALID_ARGUMENT, "buildTLAS: no mesh");
        const Mesh& m = meshes[0];
        const uint32_t nv = (uint32_t)(m.positions.size() / 3), nt = (uint32_t)(m.indices.size() / 3);
        std::vector<float> p(m.positions.size());
        for (size_t v = 0; v < nv; ++v)
            for (int k = 0; k < 3; ++k) p[3 * v + k] = (float)((double)m.positions[3 * v + k] - origin[k]);
        check(vgb_scene_upload(ctx_, p.data(), nv, m.indices.data(), nt, bands.size(),
                               m.albedo.empty() ? nullptr : m.albedo.data(), nullptr,
                               m.uv.empty() ? nullptr : m.uv.data(), m.albedo_map.empty() ? nullptr : m.albedo_map.data(),
                               m.map_w, m.map_h), ctx_, "scene_upload");
        vgb_bvh_options o{0, 0, 0, 0};
        check(vgb_bvh_build(ctx_, &o), ctx_, "bvh_build");
        dirty_ = false;
    }

    std::vector<vgb_light> cLights() const {
        std::vector<vgb_light> out;
        for (auto& L : lights) {
            vgb_light l{};
            for (int k = 0; k < 3; ++k) l.position[k] = (float)(L.position[k] - origin[k]);
            l.radius = L.radius;
            for (uint32_t b = 0; b < bands.size(); ++b) l.radiance[b] = L.radiance[b];
            out.push_back(l);
        }
        return out;
    }

    // Scene::pathtraceRender (scene.ipp:840-845): renders, then Camera::simulateSensor on the
    // received power; returns the [H][W] image in 0..1.
    const std::vector<float>& pathtraceRender(Camera& camera) {
        pathtracer.render(camera, *this);
        const std::vector<float>& power = pathtracer.renderPasses.received_power;
        const uint32_t B = bands.size();
        vgb_sensor s{};
        s.exposure_time = camera.exposure_time;
        const std::vector<float> e = bands.photonEnergies();
        float total_energy = 0;  // PhotositeConfig::defaultQE (photosite.ipp:64-79)
        for (uint32_t k = 0; k < B; ++k) total_energy += e[k] / (float)B;
        for (uint32_t k = 0; k < B; ++k) {
            s.photon_energy[k] = e[k];
            s.quantum_efficiency[k] = camera.photosite.quantum_efficiency.empty()
                                          ? 0.5f * e[k] / total_energy
                                          : camera.photosite.quantum_efficiency[k];
        }
        s.gain = camera.photosite.gain;
        s.max_adu = camera.photosite.maxADU();
        s.simulate_photon_noise = camera.simulate_photon_noise;
        if (camera.has_noise_model) {
            const NoiseModelConfig& n = camera.noise_model;
            s.noise_model = 1;
            s.dark_current = n.dark_current; s.readout_noise_mean = n.readout_noise_mean;
            s.readout_noise_std = n.readout_noise_std; s.horizontal_scale = n.horizontal_scale;
            s.vertical_scale = n.vertical_scale; s.horizontal_pattern_period = n.horizontal_pattern_period;
            s.vertical_pattern_period = n.vertical_pattern_period;
        }
        s.seed = camera.sensor_seed;
        s.frame = pathtracer.options.frame;
        sensor_image_.resize((size_t)camera.width * camera.height);
        check(vgb_sensor_simulate(ctx_, power.data(), camera.width, camera.height, B, &s, sensor_image_.data(), 0),
              ctx_, "sensor_simulate");
        return sensor_image_;
    }

    vgb_context* context() { return ctx_; }

private:
    vgb_context* ctx_ = nullptr;
    std::vector<float> sensor_image_;
    bool dirty_ = true;
};

inline void GpuPathTracer::render(Camera& camera, Scene& scene) {
    scene.buildTLAS();
    vgb_context* ctx = scene.context();
    const uint32_t B = scene.bands.size(), W = camera.width, H = camera.height;
    const size_t P = (size_t)W * H;
    vgb_camera cam = camera.toC(scene.origin, B);
    std::vector<vgb_light> lights = scene.cLights();
    vgb_pt_options o{};
    o.samples = (uint32_t)options.samples;
    o.bounces = (uint32_t)options.bounces;
    o.show_background = options.show_background;
    o.simulate_lighting = renderPasses.simulate_lighting;
    o.smooth_shading = scene.meshes.empty() ? 0 : scene.meshes[0].smooth_shading;
    o.deterministic_light = options.deterministic_light;
    o.rr_depth = options.rr_depth;
    o.seed = options.seed;
    o.frame = options.frame;
    o.nbands = B;
    o.adaptive_sampling = options.adaptive_sampling;
    o.samples_per_batch = (uint32_t)options.samples_per_batch;
    o.sampling_tolerance = options.sampling_tolerance;
    o.samples_to_detect_miss = (uint32_t)options.samples_to_detect_miss;
    o.denoise = options.denoise;
    if (!scene.ambient.empty()) {
        o.has_ambient = 1;
        for (uint32_t b = 0; b < B; ++b) o.ambient[b] = scene.ambient[b];
    }
    for (uint32_t b = 0; b < B; ++b) o.background[b] = scene.background[b];
    RenderPasses& rp = renderPasses;
    rp.width = W; rp.height = H; rp.bands = B;
    std::vector<float> omega(P);
    check(vgb_pixel_solid_angle(ctx, &cam, omega.data(), 0), ctx, "pixel_solid_angle");
    rp.depth.assign(P, 0.f); rp.alpha.assign(P, 0.f); rp.albedo.assign(B * P, 0.f); rp.normal_global.assign(3 * P, 0.f);
    rp.triangle_id.assign(P, VGB_NO_HIT);
    vgb_film f{};
    f.depth = rp.depth.data(); f.alpha = rp.alpha.data(); f.albedo = rp.albedo.data();
    f.normal_global = rp.normal_global.data(); f.triangle_id = rp.triangle_id.data();
    if (rp.save_velocity) {
        rp.velocity_global.assign(3 * P, 0.f); rp.velocity_camera.assign(3 * P, 0.f);
        f.velocity_global = rp.velocity_global.data(); f.velocity_camera = rp.velocity_camera.data();
    } else {
        rp.velocity_global.clear(); rp.velocity_camera.clear();
    }
    if (rp.save_triangle_size) {
        rp.triangle_size.assign(P, INFINITY);
        f.triangle_size = rp.triangle_size.data();
    } else {
        rp.triangle_size.clear();
    }
    if (rp.simulate_lighting) {
        rp.total_radiance.assign(B * P, 0.f); rp.direct_radiance.assign(B * P, 0.f);
        rp.indirect_radiance.assign(B * P, 0.f); rp.received_power.assign(B * P, 0.f);
        f.total_radiance = rp.total_radiance.data(); f.direct_radiance = rp.direct_radiance.data();
        f.indirect_radiance = rp.indirect_radiance.data(); f.received_power = rp.received_power.data();
        f.pixel_solid_angle = omega.data();
    }
    f.on_device = 0;
    check(vgb_render(ctx, &cam, lights.data(), (uint32_t)lights.size(), &o, &f), ctx, "render");
}

}  // namespace vgb
