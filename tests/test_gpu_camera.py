"""Lens distortion and depth of field on the GPU against the oracle (row a5: Camera::pixelToRay
with its distortion models and aperture sampling, camera.ipp:1105-1163, 1738-1771).

  * distortion (Brown, OpenCV, Owen), with and without the interpolated direction table: the
    rays are +, *, /, sqrt only, so direct-lighting renders with deterministic light sampling are
    bit-identical to the oracle, also at several jittered samples; the FP64 pixel solid angle
    (undistorted corners) within 1e-6; the rasterizer's projection (distort) bit-identical;
  * depth of field: samples >= 1 go through a point of the aperture (cosf/sinf, which CUDA and
    glibc may round differently by an ulp), so same-seed renders agree to 1e-4 on almost every
    pixel and their means within 3 sigma; sample 0 stays the pinhole ray;
  * batch and adjoint with a distorted, defocused camera equal per-frame renders and the
    oracle's FP64 gradient.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import gpu_render_host, oracle_render, rel_err, same_bits, same_bits_or_nan
from vira_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

MODELS = {
    "brown": lambda c: c.set_brown_distortion_coefficients(k1=-0.12, k2=0.03, k3=-0.004, p1=2e-3, p2=-1e-3),
    "opencv": lambda c: c.set_opencv_distortion_coefficients(k1=-0.1, k2=0.02, k4=0.01, k5=-0.002, p1=1e-3,
                                                             p2=-2e-3, s1=1e-3, s3=-1e-3),
    "owen": lambda c: c.set_owen_distortion_coefficients(e1=1e-3, e2=-0.08, e3=2e-3, e4=0.01, e5=1e-3, e6=-1e-3),
}
PLANES = ("total_radiance", "direct_radiance", "albedo", "depth", "alpha", "normal_global", "received_power")


@pytest.fixture(scope="module")
def direct(gpu):
    scene, cam_id = workloads.plain_direct(posts=129, resolution=72)
    scene.build_tlas()
    yield scene, cam_id
    scene.close()


@pytest.mark.parametrize("interp", [True, False], ids=["table", "direct"])
@pytest.mark.parametrize("model", sorted(MODELS))
def test_distorted_render_bit_exact(direct, model, interp):
    from oracle import oracle

    scene, cam_id = direct
    cam = scene[cam_id]
    cam.set_resolution(75, 61)
    MODELS[model](cam)
    cam.enable_distortion_interpolation(interp)
    opt = scene.pathtracer.options
    opt.samples = 3
    try:
        c = cam.to_c(scene.origin, 4)
        omega_g = scene.pixel_solid_angle(cam, c).cpu().numpy()
        omega_o = oracle.pixel_solid_angle(c)
        assert float(rel_err(omega_g, omega_o).max()) <= 1e-6
        g = gpu_render_host(scene, cam_id)
        o, _ = oracle_render(scene, cam_id, omega=omega_g)
        assert np.array_equal(g["triangle_id"], o["triangle_id"])
        for k in PLANES:
            assert same_bits_or_nan(g[k], o[k]), k
        assert (g["triangle_id"] != capi.NO_HIT).mean() > 0.5
    finally:
        cam.clear_distortion()
        opt.samples = 1


def test_distortion_moves_the_image(direct):
    scene, cam_id = direct
    cam = scene[cam_id]
    cam.set_resolution(64, 64)
    plain = gpu_render_host(scene, cam_id)
    MODELS["brown"](cam)
    try:
        bent = gpu_render_host(scene, cam_id)
    finally:
        cam.clear_distortion()
    # the centre pixel keeps its ray, the corners move
    assert plain["triangle_id"][32, 32] == bent["triangle_id"][32, 32]
    assert (plain["triangle_id"] != bent["triangle_id"]).mean() > 0.1


def test_depth_of_field_matches_oracle(direct):
    scene, cam_id = direct
    cam = scene[cam_id]
    cam.set_resolution(64, 48)
    cam.enable_depth_of_field(True)
    cam.set_f_stop(0.05)                 # a wide aperture, so the blur spans pixels
    cam.set_focus_distance(5200.0)
    opt = scene.pathtracer.options
    opt.samples = 16
    try:
        g = gpu_render_host(scene, cam_id)
        o, _ = oracle_render(scene, cam_id)
        opt.seed = 99
        g2 = gpu_render_host(scene, cam_id)
    finally:
        cam.enable_depth_of_field(False)
        cam.set_f_stop(2.8)
        opt.samples = 1
        opt.seed = 1
    a, b, c = g["total_radiance"], o["total_radiance"], g2["total_radiance"]
    close = rel_err(a, b) <= 1e-4
    assert close.mean() >= 0.98, close.mean()
    sig = np.sqrt(np.maximum(np.var(a - c, axis=(1, 2)) / 2.0, 1e-30))
    n = a.shape[1] * a.shape[2]
    assert np.all(np.abs(a.mean(axis=(1, 2)) - b.mean(axis=(1, 2))) <= 3 * sig * np.sqrt(2.0 / n) + 1e-6)
    assert not np.array_equal(a, c)   # the aperture samples do move the rays


def test_depth_of_field_sample_zero_is_the_pinhole_ray(direct):
    scene, cam_id = direct
    cam = scene[cam_id]
    cam.set_resolution(40, 40)
    base = gpu_render_host(scene, cam_id)
    cam.enable_depth_of_field(True)
    cam.set_f_stop(0.05)
    cam.set_focus_distance(4000.0)
    try:
        dof = gpu_render_host(scene, cam_id)
    finally:
        cam.enable_depth_of_field(False)
        cam.set_f_stop(2.8)
    for k in ("total_radiance", "depth"):
        assert same_bits(dof[k], base[k]), k


@pytest.mark.parametrize("model", sorted(MODELS))
def test_rasterizer_projection_with_distortion(gpu, model):
    """Camera::projectCameraPoint distorts before K: every raster pass bit-identical to the
    oracle's sequential rasterizer, and the distortion does change the coverage."""
    from test_gpu_raster import _compare, _dem_scene

    s, cid = _dem_scene(res=80)
    plain = s.rasterizer.render(s[cid], s).depth.cpu().numpy()
    MODELS[model](s[cid])
    covered, _ = _compare(s, cid, model)
    assert covered > 0.5
    bent = s.rasterizer.render(s[cid], s).depth.cpu().numpy()
    assert not np.array_equal(np.isfinite(plain), np.isfinite(bent)) or not np.array_equal(plain, bent)
    s.close()


def test_batch_with_distortion_and_depth_of_field_equals_per_frame(gpu):
    import torch

    from vira_gb300.scene import BatchFrame, Camera

    scene, frames = workloads.trajectory(nframes=3, posts=129, resolutions=(40, 56), spps=(3, 5), seed=5,
                                         alt_top=5000.0, alt_bottom=2500.0)
    out = []
    for i, fr in enumerate(frames):
        cam = fr.camera
        list(MODELS.values())[i](cam)
        if i != 1:
            cam.enable_depth_of_field(True)
            cam.set_f_stop(0.1)
            cam.set_focus_distance(3000.0)
        out.append(fr)
    planes = ("total_radiance", "triangle_id", "depth")
    batch = scene.render_batch(out, autotune=False, use_graph=False, planes=planes)
    torch.cuda.synchronize()
    pt = scene.pathtracer
    for fr, b in zip(out, batch):
        for k, L in enumerate(scene.lights):
            L.position = np.asarray(fr.light_positions[k], np.float64)
        pt.options.samples = fr.samples
        pt.options.frame = fr.frame
        rp = pt.render(fr.camera, scene)
        torch.cuda.synchronize()
        for k in planes:
            assert np.array_equal(b[k].cpu().numpy().view(np.uint32), getattr(rp, k).cpu().numpy().view(np.uint32)), k
    scene.close()


def test_adjoint_with_distorted_defocused_camera_matches_oracle(gpu):
    from oracle import oracle

    scene, views = workloads.inversion(posts=65, tex=32, resolution=24, nviews=1, spp=3, bounces=1)
    scene.build_tlas()
    v = views[0]
    MODELS["owen"](v.camera)
    v.camera.enable_depth_of_field(True)
    v.camera.set_f_stop(0.2)
    v.camera.set_focus_distance(2000.0)
    cam = v.camera.to_c(scene.origin, scene.bands.size)
    from vira_gb300.autograd import _lights_for

    lights = _lights_for(scene, v)
    opts = scene.pathtracer.c_options(scene)
    opts.frame = v.frame
    dl = np.random.default_rng(1).standard_normal((scene.bands.size, 24, 24)).astype(np.float32)
    gt = np.zeros(scene.meshes[0].albedo_map.shape, np.float32)
    gp = np.zeros((scene.meshes[0].positions.shape[0], 3), np.float32)
    lib = capi.load()
    ctx = scene.context()
    capi.check(lib.vgb_adjoint_positions(ctx, C.byref(cam), lights, 1, C.byref(opts), capi.ptr(dl), capi.ptr(gt),
                                         capi.ptr(gp), 0), ctx, "adjoint_positions")
    osc = oracle.OracleScene.from_flat(scene.flat, scene.bands.size)
    ot, op = osc.adjoint_positions(cam, lights, 1, opts, dl, tex_shape=gt.shape, nverts=gp.shape[0])
    osc.close()
    scene.close()
    for a, b in ((gt, ot), (gp, op)):
        rel = float(np.linalg.norm(a.astype(np.float64) - b) / max(np.linalg.norm(b), 1e-30))
        assert rel <= 1e-3, rel
