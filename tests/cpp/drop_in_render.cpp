// Renders the plain direct-lighting terrain scene through the C++ host API (include/vgb.hpp), the
// way a Vira program drives CPUPathTracer: scene.pathtracer.options / renderPasses, then render.
// Usage: drop_in_render heights.bin posts resolution out.bin
// heights.bin: posts*posts float32, row-major; out.bin: total radiance [4][R][R], triangle ids,
// then the first-hit passes velocity_camera [3][R][R] and triangle_size [R][R] (camera moving at
// (30, -4, 2) m/s, turning at (0, 0.01, 0) rad/s).
#include <cmath>
#include <cstdio>
#include <fstream>
#include <vector>

#include "vgb.hpp"

int main(int argc, char** argv) {
    if (argc != 5) { std::fprintf(stderr, "usage: %s heights.bin posts resolution out.bin\n", argv[0]); return 2; }
    const uint32_t posts = (uint32_t)std::atoi(argv[2]), res = (uint32_t)std::atoi(argv[3]);
    std::vector<float> h((size_t)posts * posts);
    std::ifstream in(argv[1], std::ios::binary);
    in.read(reinterpret_cast<char*>(h.data()), (std::streamsize)(h.size() * sizeof(float)));
    if (!in) { std::fprintf(stderr, "cannot read heights\n"); return 2; }
    try {
        vgb::Scene scene(vgb::SpectralBands::bounds({{400, 500}, {500, 600}, {600, 700}, {800, 900}}));
        scene.addMesh(vgb::Mesh::fromDEM(h, posts, posts, 5120.0 / (posts - 1), 0.12f, 4));
        size_t sun = scene.newSun(5778.0);
        scene.setSunDirection(sun, 0.0, 30.0);
        vgb::Camera cam;
        cam.setResolution(res, res);
        cam.setSensorSize(36.0 / 1000.0);
        cam.setFieldOfView(30.0);
        cam.setLocalPosition(0.0, 0.0, 5000.0);
        const double a = 20.0 * (M_PI / 180.0);
        cam.lookInDirection({std::sin(a), 0.0, -std::cos(a)});
        scene.pathtracer.options.samples = 1;
        scene.pathtracer.options.bounces = 0;
        scene.pathtracer.options.deterministic_light = true;
        scene.pathtracer.options.seed = 1;
        scene.pathtracer.renderPasses.simulate_lighting = true;
        scene.pathtracer.renderPasses.save_velocity = true;
        scene.pathtracer.renderPasses.save_triangle_size = true;
        cam.velocity = {30.0, -4.0, 2.0};
        cam.angular_rate = {0.0, 0.01, 0.0};
        scene.pathtracer.render(cam, scene);
        const auto& rp = scene.pathtracer.renderPasses;
        std::ofstream out(argv[4], std::ios::binary);
        out.write(reinterpret_cast<const char*>(rp.total_radiance.data()), (std::streamsize)(rp.total_radiance.size() * 4));
        out.write(reinterpret_cast<const char*>(rp.triangle_id.data()), (std::streamsize)(rp.triangle_id.size() * 4));
        out.write(reinterpret_cast<const char*>(rp.velocity_camera.data()), (std::streamsize)(rp.velocity_camera.size() * 4));
        out.write(reinterpret_cast<const char*>(rp.triangle_size.data()), (std::streamsize)(rp.triangle_size.size() * 4));
        std::printf("rendered %ux%u, %zu triangles\n", res, res, scene.meshes[0].indices.size() / 3);
    } catch (const vgb::Error& e) {
        std::fprintf(stderr, "vgb error %d: %s\n", (int)e.status, e.what());
        return 1;
    }
    return 0;
}
