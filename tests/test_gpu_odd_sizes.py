"""Frames whose sizes are not whole 8x4-pixel tiles.

The wavefront kernels number the camera rays of bounce 0 by 8x4-pixel warp tiles, so a frame of
W x H pixels launches ceil(W/8) * ceil(H/4) * 32 items, more than W * H when either side is not
a multiple of the tile.  These tests render such frames (100x50, 1001x37, 37x1001) through
every entry point that runs those kernels and check them against the oracle, which walks the
true W x H pixels as the reference does (cpu_path_tracer.ipp:65-89):

  * vgb_render: triangle ids bit-exact, every plane within 1e-4 relative (direct lighting,
    deterministic light sampling);
  * vgb_render_noalloc: bit-identical to vgb_render, direct and path-traced;
  * vgb_render_batch: frames of those sizes bit-identical to per-frame vgb_render, and a
    three-frame batch against the oracle directly.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import gpu_render_host, oracle_render, rel_err, same_bits
from vira_gb300 import capi, workloads
from vira_gb300.scene import BatchFrame, Camera

pytestmark = pytest.mark.gpu

SIZES = [(100, 50), (1001, 37), (37, 1001)]
IDS = [f"{w}x{h}" for w, h in SIZES]
PLANES = ("total_radiance", "direct_radiance", "indirect_radiance", "received_power", "albedo", "normal_global",
          "depth", "alpha")


@pytest.fixture(scope="module")
def direct(gpu):
    scene, cam_id = workloads.plain_direct(posts=129, resolution=64)
    scene.build_tlas()
    yield scene, cam_id
    scene.close()


@pytest.mark.parametrize("size", SIZES, ids=IDS)
def test_render_matches_oracle(direct, size):
    scene, cam_id = direct
    cam = scene[cam_id]
    cam.set_resolution(*size)
    g = gpu_render_host(scene, cam_id)
    omega = scene.pixel_solid_angle(cam, cam.to_c(scene.origin, scene.bands.size)).cpu().numpy()
    o, counts = oracle_render(scene, cam_id, omega=omega)
    W, H = size
    assert g["total_radiance"].shape == (4, H, W)
    assert np.array_equal(g["triangle_id"], o["triangle_id"])
    for k in PLANES:
        assert float(rel_err(g[k], o[k]).max()) <= 1e-4, k
    st = scene.pathtracer.last_stats
    assert st.rays_closest == counts[0] == W * H
    assert st.rays_shadow == counts[1]
    assert (g["triangle_id"] != capi.NO_HIT).mean() > 0.05


def _device_film(torch, B, H, W, dev, omega):
    planes = {}
    for name in PLANES + ("triangle_id",):
        if name in ("depth", "alpha"):
            shape, dt = (H, W), torch.float32
        elif name == "triangle_id":
            shape, dt = (H, W), torch.int32
        elif name == "normal_global":
            shape, dt = (3, H, W), torch.float32
        else:
            shape, dt = (B, H, W), torch.float32
        planes[name] = torch.full(shape, -7, dtype=dt, device=dev)
    f = capi.Film()
    for name, t in planes.items():
        setattr(f, name, t.data_ptr())
    f.pixel_solid_angle = omega.data_ptr()
    f.on_device = 1
    return planes, f


def _render_both(scene, cam_id):
    """vgb_render and vgb_render_noalloc of the same frame into device films."""
    import torch

    lib = capi.load()
    ctx = scene.context()
    camera = scene[cam_id]
    cam = camera.to_c(scene.origin, scene.bands.size)
    lights, nl = scene.c_lights()
    omega = scene.pixel_solid_angle(camera, cam)
    opts = scene.pathtracer.c_options(scene)
    B, H, W = scene.bands.size, cam.height, cam.width
    ref, f1 = _device_film(torch, B, H, W, omega.device, omega)
    out, f2 = _device_film(torch, B, H, W, omega.device, omega)
    capi.check(lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f1)), ctx, "render")
    capi.check(lib.vgb_render_noalloc(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f2)), ctx,
               "render_noalloc")
    torch.cuda.synchronize()
    return {k: v.cpu().numpy() for k, v in ref.items()}, {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("size", SIZES, ids=IDS)
def test_noalloc_bit_identical_direct(direct, size):
    scene, cam_id = direct
    scene[cam_id].set_resolution(*size)
    ref, out = _render_both(scene, cam_id)
    for k in ref:
        assert same_bits(out[k], ref[k]), k


def test_noalloc_bit_identical_path_traced(gpu):
    """Bounces, Russian roulette, two lights, ambient and background at 100x50 (8 bands)."""
    scene, cam_id = workloads.path_traced(posts=65, tex=64, resolution=64, spp=3, bounces=2, rr_depth=1, seed=5)
    s2 = scene.new_sphere_light(np.float32(5.0e5), 6.96e8)
    scene.set_sun_direction(s2, azimuth_deg=200.0, elevation_deg=40.0)
    scene.set_ambient(0.02)
    scene.set_background_emission(0.3)
    scene.pathtracer.options.show_background = True
    scene.build_tlas()
    scene[cam_id].set_resolution(100, 50)
    ref, out = _render_both(scene, cam_id)
    for k in ref:
        assert same_bits(out[k], ref[k]), k
    assert ref["indirect_radiance"].mean() > 0
    scene.close()


def _per_frame(scene, frames, planes):
    import torch

    out = []
    pt = scene.pathtracer
    saved = [L.position.copy() for L in scene.lights]
    for fr in frames:
        for k, L in enumerate(scene.lights):
            L.position = np.asarray(fr.light_positions[k], np.float64)
        pt.options.samples = fr.samples
        pt.options.frame = fr.frame
        rp = pt.render(fr.camera, scene)
        torch.cuda.synchronize()
        out.append({k: getattr(rp, k).cpu().numpy() for k in planes})
    for k, L in enumerate(scene.lights):
        L.position = saved[k]
    return out


def _odd_frames(frames):
    """The trajectory's first frames re-sized to the odd sizes."""
    out = []
    for fr, (w, h) in zip(frames, SIZES):
        cam = Camera()
        cam.set_resolution(w, h)
        cam.set_sensor_size(36.0 / 1000.0)
        cam.set_field_of_view(30.0)
        cam.set_local_position(fr.camera.position)
        cam.rotation = fr.camera.rotation.copy()
        out.append(BatchFrame(camera=cam, samples=fr.samples, frame=fr.frame, light_positions=fr.light_positions))
    return out


@pytest.mark.parametrize("bounces", [0, 2], ids=["direct", "path"])
def test_batch_odd_sizes_equal_per_frame(gpu, bounces):
    import torch

    scene, frames = workloads.trajectory(nframes=3, posts=129, resolutions=(64,), spps=(1, 3), seed=9,
                                         alt_top=6000.0, alt_bottom=2000.0)
    scene.pathtracer.options.bounces = bounces
    scene.pathtracer.options.rr_depth = 1 if bounces else 0
    frames = _odd_frames(frames)
    planes = ("total_radiance", "received_power", "triangle_id", "depth")
    batch = scene.render_batch(frames, autotune=False, use_graph=False, planes=planes)
    torch.cuda.synchronize()
    ref = _per_frame(scene, frames, planes)
    for i, (b, r) in enumerate(zip(batch, ref)):
        for k in planes:
            bb = b[k].cpu().numpy()
            assert bb.shape == r[k].shape, (i, k)
            assert np.array_equal(bb.view(np.uint32), r[k].view(np.uint32)), (i, k)
    scene.close()


def test_batch_matches_oracle(gpu):
    """Three frames of uneven size in one persistent launch against the oracle frame by frame
    (deterministic light sampling, one sample per pixel at the pixel corner)."""
    import torch
    from oracle import oracle

    scene, frames = workloads.trajectory(nframes=3, posts=129, resolutions=(64,), spps=(1,), seed=9,
                                         alt_top=6000.0, alt_bottom=2000.0)
    scene.pathtracer.options.deterministic_light = True
    frames = _odd_frames(frames)
    planes = ("total_radiance", "received_power", "triangle_id", "depth")
    batch = scene.render_batch(frames, autotune=False, use_graph=False, planes=planes)
    torch.cuda.synchronize()
    if scene.flat is None:
        scene.flatten()
    osc = oracle.OracleScene.from_flat(scene.flat, scene.bands.size)
    saved = [L.position.copy() for L in scene.lights]
    try:
        for fr, b in zip(frames, batch):
            for k, L in enumerate(scene.lights):
                L.position = np.asarray(fr.light_positions[k], np.float64)
            cam = fr.camera.to_c(scene.origin, scene.bands.size)
            omega = scene.pixel_solid_angle(fr.camera, cam).cpu().numpy()
            lights, nl = scene.c_lights()
            opts = scene.pathtracer.c_options(scene)
            opts.samples = fr.samples
            opts.frame = fr.frame
            o, _ = osc.render(cam, lights, nl, opts, omega=omega)
            assert np.array_equal(b["triangle_id"].cpu().numpy().view(np.uint32), o["triangle_id"])
            for k in ("total_radiance", "received_power", "depth"):
                assert float(rel_err(b[k].cpu().numpy(), o[k]).max()) <= 1e-4, k
    finally:
        for k, L in enumerate(scene.lights):
            L.position = saved[k]
        osc.close()
    scene.close()
