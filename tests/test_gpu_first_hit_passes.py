"""The first-hit passes renderPasses.save_velocity and save_triangle_size (passes.hpp:79-85,
computed at cpu_path_tracer.ipp:356-372) on the GPU against the oracle: two moving instances of a
DEM (one rotated and shifted, with its own velocity and angular rate) under a moving, rotating
camera.  Both passes are set once, at a pixel's first hit, from +, *, /, sqrt only, so they are
bit-identical to the oracle; pixels that never hit keep 0 velocity and +inf triangle size.  The
same planes come out of host films, the no-allocation render and the batched render."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

from helpers import gpu_render_host, oracle_render, same_bits, same_bits_or_nan
from vira_gb300 import FOUR_BAND, Mesh, Scene, capi, synthetic

pytestmark = pytest.mark.gpu

PASSES = ("velocity_global", "velocity_camera", "triangle_size")


def _scene(res=(70, 52)):
    h = synthetic.fbm_heights(65, 0.8, seed=2, lo=-80.0, hi=80.0)
    s = Scene(FOUR_BAND)
    m = s.add_mesh(Mesh.from_dem(h, 40.0, albedo=0.12, nbands=4))
    a = s.new_instance(m)
    b = s.new_instance(m)
    s[a].set_velocity([3.0, -1.5, 0.25])
    s[a].set_angular_rate([0.0, 0.0, 0.02])
    s[b].set_local_position(1500.0, 400.0, -30.0)
    th = math.radians(25.0)
    s[b].set_local_rotation([[math.cos(th), -math.sin(th), 0.0], [math.sin(th), math.cos(th), 0.0], [0.0, 0.0, 1.0]])
    s[b].set_velocity([-7.0, 2.0, 0.0])
    s[b].set_angular_rate([0.001, -0.002, 0.01])
    sun = s.new_sun(5778.0)
    s.set_sun_direction(sun, 30.0, 35.0)
    cid = s.new_camera()
    c = s[cid]
    c.set_resolution(*res)
    c.set_sensor_size(0.036)
    c.set_field_of_view(45.0)
    c.set_local_position(900.0, -2600.0, 1800.0)
    c.look_at((900.0, 300.0, 0.0))
    c.velocity = np.array([40.0, 5.0, -3.0])
    c.angular_rate = np.array([0.0, 0.01, 0.003])
    pt = s.pathtracer
    pt.options.samples = 2
    pt.options.deterministic_light = True
    pt.render_passes.simulate_lighting = True
    pt.render_passes.save_velocity = True
    pt.render_passes.save_triangle_size = True
    return s, cid


def test_first_hit_passes_match_oracle(gpu):
    s, cid = _scene()
    g = gpu_render_host(s, cid)
    rp = s.pathtracer.render_passes
    got = {k: getattr(rp, k).cpu().numpy() for k in PASSES}
    o, _ = oracle_render(s, cid)
    hit = o["triangle_id"] != capi.NO_HIT
    assert 0.3 < hit.mean() < 1.0   # sky pixels keep the initial values
    # the film's ids restart per instance (Interaction::tri_id is the instance's own triangle index)
    counts = [n for (_, _, n) in s.flat["tri_offsets"]]
    starts = np.cumsum([0] + counts[:-1])
    flat_id = o["triangle_id"][hit].astype(np.int64)
    k = np.searchsorted(starts, flat_id, side="right") - 1
    assert np.array_equal(g["triangle_id"][hit].astype(np.int64), flat_id - starts[k])
    assert np.all(g["triangle_id"][~hit] == capi.NO_HIT)
    assert set(k.tolist()) == {0, 1}
    for k in PASSES:
        assert same_bits_or_nan(got[k], o[k]), k
    assert np.all(np.isinf(got["triangle_size"][~hit])) and np.all(got["velocity_global"][:, ~hit] == 0)
    assert np.all(np.isfinite(got["triangle_size"][hit])) and (got["triangle_size"][hit] > 0).all()
    # both instances' motion shows up
    vg = got["velocity_global"][:, hit]
    assert np.unique(np.round(vg[0])).size > 2
    s.close()


def test_first_hit_passes_host_film_noalloc_and_batch(gpu):
    import torch

    from vira_gb300.scene import BatchFrame

    s, cid = _scene((48, 40))
    rp = s.pathtracer.render(s[cid], s)
    torch.cuda.synchronize()
    ref = {k: getattr(rp, k).cpu().numpy() for k in PASSES}
    lib = capi.load()
    ctx = s.context()
    cam = s[cid].to_c(s.origin, 4)
    lights, nl = s.c_lights()
    opts = s.pathtracer.c_options(s)
    H, W = cam.height, cam.width
    # host film
    host = {k: np.empty((3, H, W) if k != "triangle_size" else (H, W), np.float32) for k in PASSES}
    f = capi.Film()
    for k, v in host.items():
        setattr(f, k, v.ctypes.data)
    f.on_device = 0
    capi.check(lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)), ctx)
    for k in PASSES:
        assert same_bits(host[k], ref[k]), k
    # no-allocation render
    dev = {k: torch.full(v.shape, -3.0, device="cuda") for k, v in host.items()}
    f2 = capi.Film()
    for k, v in dev.items():
        setattr(f2, k, v.data_ptr())
    f2.on_device = 1
    capi.check(lib.vgb_render_noalloc(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f2)), ctx)
    torch.cuda.synchronize()
    for k in PASSES:
        assert same_bits(dev[k].cpu().numpy(), ref[k]), k
    # batched render of the same frame
    fr = BatchFrame(camera=s[cid], samples=s.pathtracer.options.samples, frame=s.pathtracer.options.frame,
                    light_positions=[L.position.copy() for L in s.lights])
    out = s.render_batch([fr], autotune=False, planes=("total_radiance",) + PASSES)
    torch.cuda.synchronize()
    for k in PASSES:
        assert same_bits(out[0][k].cpu().numpy(), ref[k]), k
    s.close()


def test_rasterizer_passes_match_oracle(gpu):
    """The rasterizer's passes (cpu_rasterizer.ipp:123-129, 211-218): the triangle size is the
    longest projected edge in pixels, the velocities those of the path tracer's first hit at the
    fragment's scene position; bit-identical to the oracle's sequential rasterizer, the same from
    a host film with every plane requested (all staged on the device)."""
    import torch

    from oracle import oracle

    s, cid = _scene()
    rr = s.rasterizer.render_passes
    rr.simulate_lighting = True
    rr.save_velocity = True
    rr.save_triangle_size = True
    rp = s.rasterizer.render(s[cid], s)
    torch.cuda.synchronize()
    got = {k: getattr(rp, k).cpu().numpy() for k in PASSES}
    B = s.bands.size
    cam = s[cid].to_c(s.origin, B)
    lights, nl = s.c_lights()
    omega = s.pixel_solid_angle(s[cid], cam).cpu().numpy()
    osc = oracle.OracleScene.from_flat(s.flat, B)
    ref = osc.rasterize(cam, s[cid].intrinsic_matrix(), lights, nl, True, s.smooth_shading(), omega, passes=True)
    osc.close()
    drawn = ref["triangle_id"] != 0xFFFFFFFF
    assert 0.3 < drawn.mean() < 1.0
    for k in PASSES:
        assert same_bits_or_nan(got[k], ref[k]), k
    assert np.all(np.isinf(got["triangle_size"][~drawn])) and np.all(got["velocity_camera"][:, ~drawn] == 0)
    assert np.all(got["triangle_size"][drawn] > 0)
    assert np.unique(np.round(got["velocity_global"][0][drawn])).size > 2
    # host film with every plane the rasterizer writes
    lib = capi.load()
    ctx = s.context()
    o = capi.RasterOptions()
    o.intrinsic[:] = [float(x) for x in s[cid].intrinsic_matrix()]
    o.simulate_lighting = 1
    o.nbands = B
    H, W = cam.height, cam.width
    host = {"depth": (H, W), "alpha": (H, W), "albedo": (B, H, W), "normal_global": (3, H, W),
            "total_radiance": (B, H, W), "direct_radiance": (B, H, W), "indirect_radiance": (B, H, W),
            "received_power": (B, H, W), "velocity_global": (3, H, W), "velocity_camera": (3, H, W),
            "triangle_size": (H, W)}
    host = {k: np.full(v, -5.0, np.float32) for k, v in host.items()}
    host["triangle_id"] = np.zeros((H, W), np.uint32)
    om = np.ascontiguousarray(omega, np.float32)
    f = capi.Film()
    for k, a in host.items():
        setattr(f, k, a.ctypes.data)
    f.pixel_solid_angle = om.ctypes.data
    f.on_device = 0
    capi.check(lib.vgb_rasterize(ctx, C.byref(cam), lights, nl, C.byref(o), C.byref(f)), ctx, "rasterize")
    for k in PASSES + ("depth", "total_radiance", "received_power", "albedo"):
        assert same_bits_or_nan(host[k], getattr(rp, k).cpu().numpy()), k
    assert np.all(host["direct_radiance"] == 0) and np.all(host["indirect_radiance"] == 0)
    s.close()
