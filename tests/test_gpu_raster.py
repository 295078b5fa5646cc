"""The GPU rasterizer (vgb_rasterize, Scene.rasterizer) against the oracle's literal restatement of
CPURasterizer::render: every pass bit-identical -- depth, alpha, albedo, normal, triangle id,
radiance and received power -- on a textured crater DEM (flat and smooth shading), an icosphere
seen from outside (back faces behind front faces), a close-up whose triangles cover thousands of
pixels each (the one-block-per-triangle path), a Blender-frame camera, duplicated coplanar
instances (ties go to the earlier triangle; ids restart per instance) and triangles reaching
behind and right up to the camera plane.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle
from vira_gb300 import FOUR_BAND, Mesh, Scene, capi, synthetic

pytestmark = pytest.mark.gpu


def _dem_scene(posts=129, tex=64, smooth=False, cam_pos=(150.0, -300.0, 900.0), target=(0.0, 0.0, 0.0), res=96,
               blender=False):
    h = synthetic.fbm_heights(posts, 0.8, seed=3, lo=-60.0, hi=60.0)
    h = synthetic.add_crater_field(h, 1000.0 / (posts - 1), seed=4, dmin=40, dmax=300)
    s = Scene(FOUR_BAND)
    m = Mesh.from_dem(h, 1000.0 / (posts - 1), albedo=np.array([0.1, 0.12, 0.14, 0.2], np.float32), nbands=4)
    m.uv = synthetic.grid_uvs(posts, posts, posts - 1)
    alb = synthetic.lognormal_albedo(tex, 0.12, 0.3, seed=5)
    m.albedo_map = np.ascontiguousarray(np.repeat(alb[:, :, None], 4, axis=2))
    m.set_smooth_shading(smooth)
    s.add_mesh(m)
    s.new_instance(("mesh", 0))
    sun = s.new_sun(5778.0)
    s.set_sun_direction(sun, 40.0, 25.0)
    cid = s.new_camera()
    c = s[cid]
    if blender:
        c.enable_blender_frame()
    c.set_resolution(res, res)
    c.set_sensor_size(0.036)
    c.set_field_of_view(40.0)
    c.set_local_position(*cam_pos)
    c.look_at(target)
    s.rasterizer.render_passes.simulate_lighting = True
    return s, cid


def _compare(s, cid, what=""):
    import torch

    rp = s.rasterizer.render(s[cid], s)
    torch.cuda.synchronize()
    B = s.bands.size
    cam = s[cid].to_c(s.origin, B)
    lights, nl = s.c_lights()
    omega = s.pixel_solid_angle(s[cid], cam).cpu().numpy()
    osc = oracle.OracleScene.from_flat(s.flat, B)
    ref = osc.rasterize(cam, s[cid].intrinsic_matrix(), lights, nl, True, s.smooth_shading(), omega)
    osc.close()
    counts = [n for (_, _, n) in s.flat["tri_offsets"]]
    tid_ref = ref["triangle_id"].astype(np.int64)
    if len(counts) > 1:   # ids restart per instance
        starts = np.cumsum([0] + counts[:-1])
        hit = tid_ref != 0xFFFFFFFF
        k = np.searchsorted(starts, tid_ref[hit] - 1, side="right") - 1
        tid_ref[hit] = tid_ref[hit] - starts[k]
    got = {k: getattr(rp, k).cpu().numpy() for k in ("depth", "alpha", "albedo", "normal_global", "total_radiance",
                                                   "received_power")}
    for k, v in got.items():
        assert np.array_equal(v, ref[k], equal_nan=True), f"{what}: {k} differs at {np.sum(v != ref[k])} values"
    tid = rp.triangle_id.cpu().numpy().astype(np.int64)
    tid_ref = np.where(tid_ref == 0xFFFFFFFF, -1, tid_ref)
    assert np.array_equal(tid, tid_ref), f"{what}: triangle ids differ"
    assert np.all(rp.direct_radiance.cpu().numpy() == 0) and np.all(rp.indirect_radiance.cpu().numpy() == 0)
    covered = np.isfinite(ref["depth"])
    assert np.all(np.isinf(got["alpha"][covered])) and np.all(got["alpha"][~covered] == 0)
    return covered.mean(), s.rasterizer.last_stats


@pytest.mark.parametrize("smooth", [False, True])
def test_dem_matches_the_oracle(gpu, smooth):
    s, cid = _dem_scene(smooth=smooth)
    cov, _ = _compare(s, cid, f"dem smooth={smooth}")
    assert cov > 0.5
    s.close()


def test_close_up_large_triangles(gpu):
    s, cid = _dem_scene(posts=9, tex=8, cam_pos=(30.0, -40.0, 180.0), target=(10.0, 0.0, 0.0), res=128)
    cov, _ = _compare(s, cid, "close-up")
    assert cov > 0.9
    s.close()


def test_blender_frame_camera(gpu):
    s, cid = _dem_scene(blender=True)
    cov, _ = _compare(s, cid, "blender")
    assert cov > 0.5
    s.close()


def test_icosphere_from_outside(gpu):
    dirs, faces = synthetic.icosphere(4)
    pos = (dirs * 250.0).astype(np.float32)
    s = Scene(FOUR_BAND)
    m = Mesh(positions=pos, indices=faces, albedo=np.full((pos.shape[0], 4), 0.3, np.float32))
    m.set_smooth_shading(True)
    s.add_mesh(m)
    s.new_instance(("mesh", 0))
    sun = s.new_sun(5778.0)
    s.set_sun_direction(sun, 10.0, 30.0)
    cid = s.new_camera()
    c = s[cid]
    c.set_resolution(80, 64)
    c.set_sensor_size(0.036)
    c.set_field_of_view(30.0)
    c.set_local_position(900.0, 300.0, 200.0)
    c.look_at((0.0, 0.0, 0.0))
    s.rasterizer.render_passes.simulate_lighting = True
    cov, _ = _compare(s, cid, "icosphere")
    assert 0.1 < cov < 0.9
    s.close()


def test_coplanar_instances_and_near_plane(gpu):
    """Two instances of one mesh at the same place: every pixel's winner is the first instance's
    triangle (equal distances), and ids restart at 1 for the second.  A second camera sits inside
    the DEM's relief, so triangles cross its image plane or project to huge coordinates."""
    s, cid = _dem_scene(posts=33, tex=16)
    s.new_instance(("mesh", 0))
    cov, _ = _compare(s, cid, "coplanar instances")
    assert cov > 0.5
    c2 = s.new_camera()
    cam = s[c2]
    cam.set_resolution(64, 64)
    cam.set_sensor_size(0.036)
    cam.set_field_of_view(90.0)
    cam.set_local_position(0.0, 0.0, float(s.meshes[0].positions[:, 2].max()) - 5.0)
    cam.look_in_direction((1.0, 0.2, -0.05))
    _compare(s, c2, "inside the relief")
    s.close()


def test_rasterize_render_returns_the_sensor_image(gpu):
    s, cid = _dem_scene(res=64)
    img = s.rasterize_render(cid)
    assert tuple(img.shape) == (64, 64)
    assert float(img.max()) > 0
    s.close()


def test_rasterize_rejects_bad_arguments(gpu):
    s, cid = _dem_scene(res=32)
    s.rasterizer.render(s[cid], s)
    lib = capi.load()
    ctx = s.context()
    cam = s[cid].to_c(s.origin, 4)
    o = capi.RasterOptions()
    o.nbands = 3
    f = capi.Film()
    import ctypes as C

    assert lib.vgb_rasterize(ctx, C.byref(cam), None, 0, C.byref(o), C.byref(f)) != 0
    assert b"nbands" in lib.vgb_last_error(ctx)
    s.close()



def test_id_passes_and_camera_normals(gpu):
    """Two instances side by side: instance_id / mesh_id / material_id of the first hit, triangle
    ids local to each instance (from 0 for the path tracer, from 1 for the rasterizer), and the
    rasterizer's normal in the camera frame (the inverse camera rotation times the normal)."""
    import torch

    s, cid = _dem_scene(posts=33, tex=16, cam_pos=(500.0, -900.0, 1400.0), target=(500.0, 0.0, 0.0))
    inst = s.new_instance(("mesh", 0))
    s[inst].position = np.array([1000.0, 0.0, 0.0])
    s.pathtracer.render_passes.simulate_lighting = True
    s.pathtracer.options.samples = 1
    nt = s.meshes[0].indices.shape[0]
    for renderer, first in ((s.pathtracer, 0), (s.rasterizer, 1)):
        rp = renderer.render(s[cid], s)
        torch.cuda.synchronize()
        tid = rp.triangle_id.cpu().numpy()
        iid = rp.instance_id.cpu().numpy()
        hit = tid != -1
        assert set(np.unique(iid[hit])) == {0, 1}                     # both instances seen
        assert np.all(iid[~hit] == -1) and np.all(rp.mesh_id.cpu().numpy()[hit] == 0)
        assert np.all(rp.material_id.cpu().numpy()[hit] == 0)
        assert tid[hit].min() >= first and tid[hit].max() < nt + first
        n = rp.normal_global.cpu().numpy()
        nc = rp.normal_camera.cpu().numpy()
        if renderer is s.rasterizer:
            R = s[cid].rotation.astype(np.float32)
            want = np.stack([(n[0] * R[0, r] + n[1] * R[1, r]) + n[2] * R[2, r] for r in range(3)])
            assert np.array_equal(nc, want)
        else:
            assert np.all(nc == 0)
    s.close()


def test_host_film_and_no_lighting(gpu):
    """vgb_rasterize with host planes (staged on the device and copied back) equals the device
    planes; without simulate_lighting the geometry passes are unchanged."""
    import ctypes as C

    import torch

    s, cid = _dem_scene(res=48)
    rp = s.rasterizer.render(s[cid], s)
    torch.cuda.synchronize()
    B = s.bands.size
    cam = s[cid].to_c(s.origin, B)
    lights, nl = s.c_lights()
    o = capi.RasterOptions()
    o.intrinsic[:] = [float(x) for x in s[cid].intrinsic_matrix()]
    o.simulate_lighting = 1
    o.nbands = B
    H = W = 48
    host = {"depth": np.empty((H, W), np.float32), "alpha": np.empty((H, W), np.float32),
            "albedo": np.empty((B, H, W), np.float32), "normal_global": np.empty((3, H, W), np.float32),
            "triangle_id": np.empty((H, W), np.uint32), "total_radiance": np.empty((B, H, W), np.float32),
            "received_power": np.empty((B, H, W), np.float32)}
    omega = s.pixel_solid_angle(s[cid], cam).cpu().numpy().copy()
    f = capi.Film()
    for k, a in host.items():
        setattr(f, k, a.ctypes.data)
    f.pixel_solid_angle = omega.ctypes.data
    f.on_device = 0
    lib = capi.load()
    ctx = s.context()
    capi.check(lib.vgb_rasterize(ctx, C.byref(cam), lights, nl, C.byref(o), C.byref(f)), ctx, "rasterize")
    for k in ("depth", "alpha", "albedo", "normal_global", "total_radiance", "received_power"):
        assert np.array_equal(host[k], getattr(rp, k).cpu().numpy(), equal_nan=True), k
    tid = host["triangle_id"].astype(np.int64)
    tid[tid == 0xFFFFFFFF] = -1
    assert np.array_equal(tid, rp.triangle_id.cpu().numpy().astype(np.int64))
    s.rasterizer.render_passes.simulate_lighting = False
    rq = s.rasterizer.render(s[cid], s)
    torch.cuda.synchronize()
    assert rq.total_radiance is None and rq.received_power is None
    assert np.array_equal(rq.depth.cpu().numpy(), host["depth"], equal_nan=True)
    assert np.array_equal(rq.albedo.cpu().numpy(), host["albedo"])
    s.close()


def test_render_total_power_reuses_the_render(gpu):
    s, cid = _dem_scene(res=32)
    s.pathtracer.render_passes.simulate_lighting = True
    s.pathtracer.options.samples = 2
    p1 = s.render_total_power(cid)
    p2 = s.render_total_power(cid)
    assert p2 is p1                              # the scene did not change: no new render
    s.mark_dirty()
    p3 = s.render_total_power(cid)
    assert p3 is not p1 and bool((p3 == p1).all())
    s.close()
