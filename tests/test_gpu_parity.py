"""GPU parity of the hot path against the oracle, through the C ABI (libvgb.so).

Bars (from the path's specification):
  * primary-ray triangle ids bit-exact (the edge-grazing count against the reference's own
    non-watertight triangle test is reported, not asserted to be zero);
  * hit distances within 1e-5 relative;
  * deterministic direct-illumination images within 1e-4 relative per pixel per band;
  * path-traced images within 3 sigma of the Monte Carlo standard error.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import gpu_render_host, oracle_render, primary_rays, rel_err, same_bits
from vira_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _trace_gpu(scene, o, d, any_hit=False, tmax=None):
    return scene.intersect(o, d, any_hit=any_hit, tmax=tmax)


@pytest.fixture(scope="module", params=[8, 2], ids=["bvh8", "bvh2"])
def direct_scene(gpu, request):
    scene, cam_id = workloads.plain_direct(posts=257, resolution=256)
    scene.bvh_options.layout = request.param
    scene.build_tlas()
    yield scene, cam_id
    scene.close()


def test_primary_rays_bit_exact(direct_scene):
    from oracle import oracle

    scene, cam_id = direct_scene
    cam = scene[cam_id].to_c(scene.origin, scene.bands.size)
    o, d = primary_rays(cam)
    tri_g, t_g, w_g = _trace_gpu(scene, o, d)
    osc = oracle.OracleScene.from_flat(scene.flat, scene.bands.size)
    tri_o, t_o, w_o = osc.trace(o, d)
    tri_r, t_r, _ = osc.trace(o, d, mode=1)
    osc.close()
    hit = tri_o != capi.NO_HIT
    assert hit.mean() > 0.5
    assert np.array_equal(tri_g, tri_o)
    assert float(rel_err(t_g[hit], t_o[hit]).max()) <= 1e-5
    assert same_bits(t_g, t_o)
    assert same_bits(w_g, w_o)
    # Edge-grazing rays: where the reference's own (non-watertight) triangle test disagrees.
    # Each one must be a crack (the reference test misses between two triangles that the
    # watertight test closes) or a tie across an edge the two triangles share, at the same t.
    bad = np.nonzero(tri_r != tri_o)[0]
    idx = scene.flat["indices"]
    for b in bad:
        if tri_r[b] == capi.NO_HIT:
            continue
        assert tri_o[b] != capi.NO_HIT
        assert len(set(idx[tri_o[b]]) & set(idx[tri_r[b]])) >= 2, "disagreement away from a shared edge"
        assert abs(float(t_r[b]) - float(t_o[b])) <= 1e-5 * float(t_o[b])
    print(f"edge-grazing rays (watertight vs reference triangle test): {len(bad)} of {hit.size}")
    assert len(bad) <= hit.size // 100


def test_shadow_rays_any_hit(direct_scene):
    from oracle import oracle

    scene, cam_id = direct_scene
    rng = np.random.default_rng(5)
    n = 20000
    o = np.stack([rng.uniform(-2500, 2500, n), rng.uniform(-2500, 2500, n), rng.uniform(-150, 250, n)], 1).astype(np.float32)
    d = rng.standard_normal((n, 3)).astype(np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    tmax = rng.uniform(1, 3000, n).astype(np.float32)
    tri_g, _, _ = _trace_gpu(scene, o, d, any_hit=True, tmax=tmax)
    osc = oracle.OracleScene.from_flat(scene.flat, scene.bands.size)
    tri_o, _, _ = osc.trace(o, d, any_hit=True, tmax=tmax)
    tri_c, t_c, _ = osc.trace(o, d)
    osc.close()
    occl_g = tri_g != capi.NO_HIT
    occl_o = tri_o != capi.NO_HIT
    assert np.array_equal(occl_g, occl_o)
    # occlusion agrees with closest hit t <= tmax
    assert np.array_equal(occl_o, (tri_c != capi.NO_HIT) & (t_c <= tmax))
    assert 0.05 < occl_o.mean() < 0.95


def test_direct_image_parity(direct_scene):
    scene, cam_id = direct_scene
    g = gpu_render_host(scene, cam_id)
    import torch

    omega = scene.pixel_solid_angle(scene[cam_id], scene[cam_id].to_c(scene.origin, 4)).cpu().numpy()
    o, counts = oracle_render(scene, cam_id, omega=omega)
    assert np.array_equal(g["triangle_id"], o["triangle_id"])
    for k in ("total_radiance", "direct_radiance", "indirect_radiance", "albedo", "depth", "alpha",
              "normal_global", "received_power"):
        e = rel_err(g[k], o[k])
        assert float(e.max()) <= 1e-4, (k, float(e.max()))
    st = scene.pathtracer.last_stats
    assert st.rays_closest == counts[0] and st.rays_shadow == counts[1]
    exact = np.mean(g["total_radiance"].view(np.uint32) == o["total_radiance"].view(np.uint32))
    print(f"bit-identical radiance values: {exact:.6f}")
    assert np.nanmean(g["total_radiance"]) > 0


def test_pixel_solid_angle(direct_scene):
    from oracle import oracle

    scene, cam_id = direct_scene
    cam = scene[cam_id].to_c(scene.origin, 4)
    g = scene.pixel_solid_angle(scene[cam_id], cam).cpu().numpy()
    o = oracle.pixel_solid_angle(cam)
    assert float(rel_err(g, o).max()) <= 1e-6
    fov = 2 * np.arctan(cam.kinv[0] * cam.width / 2)
    assert abs(g.sum() - 4 * np.arcsin(np.sin(fov / 2) ** 2)) < 1e-3


def test_host_film_equals_device_film(direct_scene):
    scene, cam_id = direct_scene
    g = gpu_render_host(scene, cam_id)
    lib = capi.load()
    ctx = scene.context()
    cam = scene[cam_id].to_c(scene.origin, 4)
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    W, H, B = cam.width, cam.height, 4
    tot = np.empty((B, H, W), np.float32)
    tri = np.empty((H, W), np.uint32)
    f = capi.Film()
    f.total_radiance = tot.ctypes.data
    f.triangle_id = tri.ctypes.data
    f.on_device = 0
    capi.check(lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)), ctx)
    assert same_bits(tot, g["total_radiance"])
    assert np.array_equal(tri, g["triangle_id"])


def test_lights_ambient_background_smooth(gpu):
    scene, cam_id = workloads.plain_direct(posts=129, resolution=160)
    # a second, dimmer sun from another direction, ambient light and a background
    s2 = scene.new_sphere_light(np.float32(1.0e6), 6.96e8)
    scene.set_sun_direction(s2, azimuth_deg=120.0, elevation_deg=50.0)
    scene.set_ambient([0.01, 0.02, 0.03, 0.04])
    scene.set_background_emission([0.5, 0.25, 0.125, 0.0625])
    scene.pathtracer.options.show_background = True
    scene.meshes[0].set_smooth_shading(True)
    g = gpu_render_host(scene, cam_id)
    o, _ = oracle_render(scene, cam_id)
    assert np.array_equal(g["triangle_id"], o["triangle_id"])
    hit = o["triangle_id"] != capi.NO_HIT
    e = rel_err(g["total_radiance"], o["total_radiance"])
    assert float(e[:, hit].max()) <= 1e-4
    # background uses atan2: allow a few ulp
    assert float(e[:, ~hit].max()) <= 1e-5
    scene.close()


def _noise_sigma(a, b):
    return np.sqrt(np.maximum(np.var(a - b, axis=(1, 2)) / 2.0, 1e-30))


def test_path_traced_statistical(gpu):
    kw = dict(posts=129, tex=128, resolution=96, spp=8, bounces=3, rr_depth=2)
    scene, cam_id = workloads.path_traced(seed=7, **kw)
    g7 = gpu_render_host(scene, cam_id)
    o7, counts = oracle_render(scene, cam_id)
    scene.pathtracer.options.seed = 8
    g8 = gpu_render_host(scene, cam_id)
    scene.close()
    assert np.array_equal(g7["triangle_id"], o7["triangle_id"])
    a, b, c = g7["total_radiance"], o7["total_radiance"], g8["total_radiance"]
    sig = _noise_sigma(a, c)                       # per-pixel noise from two seeds
    n = a.shape[1] * a.shape[2]
    # image means agree within 3 sigma of the mean's standard error
    dm = np.abs(a.mean(axis=(1, 2)) - b.mean(axis=(1, 2)))
    assert np.all(dm <= 3 * sig * np.sqrt(2.0 / n) + 1e-6), (dm, sig)
    # same seed: the streams are shared, so almost every pixel agrees to 1e-4
    close = rel_err(a, b) <= 1e-4
    assert close.mean() >= 0.98, close.mean()
    # per-pixel z scores of the same-seed difference stay inside 3 sigma almost everywhere
    z = np.abs(a - b) / sig[:, None, None]
    assert (z > 3).mean() <= 0.01
    assert g7["indirect_radiance"].mean() > 0


def test_render_errors(gpu):
    from vira_gb300 import Scene, FOUR_BAND

    lib = capi.load()
    scene, cam_id = workloads.plain_direct(posts=33, resolution=16)
    ctx = scene.context()
    cam = scene[cam_id].to_c(scene.origin, 4)
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    f = capi.Film()
    f.on_device = 0
    assert lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)) == 4  # no BVH yet
    scene.build_tlas()
    opts.samples = 0
    assert lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)) == 1
    opts.samples = 1
    opts.nbands = 3
    assert lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)) == 1
    assert b"nbands" in lib.vgb_last_error(ctx)
    opts.nbands = 4
    assert lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)) == 0
    scene.close()


def test_small_frame_after_large_frame(gpu):
    """Scratch keeps the largest frame's size; film planes must still use each frame's own size."""
    import torch

    scene, cam_id = workloads.plain_direct(posts=65, resolution=96)
    big = gpu_render_host(scene, cam_id)
    scene[cam_id].set_resolution(40, 40)
    small = gpu_render_host(scene, cam_id)
    scene.close()
    fresh_scene, fresh_id = workloads.plain_direct(posts=65, resolution=96)
    fresh_scene[fresh_id].set_resolution(40, 40)
    fresh = gpu_render_host(fresh_scene, fresh_id)
    fresh_scene.close()
    for k in fresh:
        assert same_bits(small[k], fresh[k]) if k != "triangle_id" else np.array_equal(small[k], fresh[k])
    assert big["total_radiance"].shape[1] == 96


def test_plane_subsets_equal_full_film(gpu):
    """The per-pixel sums a film does not request are skipped; requested planes must not change.
    Path-traced frame with bounces, background and ambient (every fold of the path radiance)."""
    scene, cam_id = workloads.path_traced(posts=65, tex=64, resolution=40, spp=3, bounces=2, rr_depth=1, seed=3)
    scene.set_ambient(0.02)
    scene.set_background_emission(0.3)
    scene.pathtracer.options.show_background = True
    full = gpu_render_host(scene, cam_id)
    lib = capi.load()
    ctx = scene.context()
    cam = scene[cam_id].to_c(scene.origin, 8)
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    W, H, B = cam.width, cam.height, 8
    shapes = {"total_radiance": (B, H, W), "direct_radiance": (B, H, W), "indirect_radiance": (B, H, W),
              "albedo": (B, H, W), "normal_global": (3, H, W), "depth": (H, W), "alpha": (H, W)}
    subsets = [("total_radiance",), ("direct_radiance",), ("indirect_radiance", "alpha"), ("albedo", "depth"),
               ("normal_global", "triangle_id")]
    for sub in subsets:
        f = capi.Film()
        out = {}
        for k in sub:
            out[k] = np.empty((H, W), np.uint32) if k == "triangle_id" else np.empty(shapes[k], np.float32)
            setattr(f, k, out[k].ctypes.data)
        f.on_device = 0
        capi.check(lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)), ctx)
        for k, v in out.items():
            if k == "triangle_id":
                assert np.array_equal(v, full[k]), sub
            else:
                assert same_bits(v, full[k]), (sub, k)
    scene.close()


def test_adaptive_sampling_matches_oracle(gpu):
    """Adaptive sampling with deterministic light sampling: every stopping decision depends on
    float sums that the kernels and the oracle form identically, so the planes are bit-exact,
    including the reference's division by the index of the last sample and the early stop of
    pixels that see only sky."""
    scene, cam_id = workloads.plain_direct(posts=129, resolution=48)
    cam = scene[cam_id]
    cam.look_in_direction((0.454, 0.0, -0.891))  # part of the view is sky
    opt = scene.pathtracer.options
    opt.samples = 40
    opt.adaptive_sampling = True
    opt.samples_per_batch = 8
    opt.samples_to_detect_miss = 5
    opt.sampling_tolerance = 0.03
    g = gpu_render_host(scene, cam_id)
    o, _ = oracle_render(scene, cam_id)
    for k in ("total_radiance", "direct_radiance", "albedo", "depth", "alpha"):
        assert same_bits(g[k], o[k]), k
    assert np.array_equal(g["triangle_id"], o["triangle_id"])
    alpha = g["alpha"]
    assert (alpha == 0).any(), "no sky pixel"
    assert (alpha > 1.0).any(), "no pixel stopped early (alpha = hits / last index exceeds 1)"
    scene.close()


@pytest.mark.parametrize("budget,refill", [(16, 8), (1, 1), (4, 32)])
def test_persistent_traversal_equals_grid_stride(gpu, budget, refill):
    """The persistent closest-hit and occlusion kernels (warps hand queue rays to free lanes,
    rays advance a bounded number of node visits between hand-outs) give every plane bit for bit
    as the one-thread-per-ray kernels, whatever the budget and refill threshold; the counting
    pass sees the same node and triangle visits."""
    scene, cam_id = workloads.path_traced(posts=129, tex=64, resolution=72, spp=3, bounces=3, rr_depth=2, seed=4)
    s2 = scene.new_sphere_light(np.float32(4.0e5), 6.96e8)
    scene.set_sun_direction(s2, azimuth_deg=210.0, elevation_deg=25.0)
    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    out = {}
    for mode in ("grid", "persistent"):
        if mode == "grid":
            capi.check(lib.vgb_set_wavefront_tuning(ctx, 0, 0, 0), ctx)
        else:
            capi.check(lib.vgb_set_wavefront_tuning(ctx, 1, budget, refill), ctx)
        lib.vgb_set_count_pass(ctx, 1)
        out[mode] = gpu_render_host(scene, cam_id)
        lib.vgb_set_count_pass(ctx, 0)
        st = scene.pathtracer.last_stats
        out[mode]["_counts"] = (st.rays_closest, st.rays_shadow, st.nodes_visited, st.tris_tested, st.nodes_closest)
    capi.check(lib.vgb_set_wavefront_tuning(ctx, 0, 0, 0), ctx)
    a, b = out["grid"], out["persistent"]
    assert a["_counts"] == b["_counts"]
    for k in a:
        if k == "_counts":
            continue
        assert np.array_equal(a[k], b[k]) if k == "triangle_id" else same_bits(a[k], b[k]), k
    assert a["indirect_radiance"].mean() > 0
    scene.close()
