"""vgb_render_noalloc: the render entry point that allocates no device memory.

It is meant for callers that cannot allocate once their scene is set up -- a frame loop held to
a fixed memory budget, or a host application whose own allocator owns the device -- since a
cudaMalloc inside a render call can synchronize the device or fail.  It runs the same launch
sequence as vgb_render with its scratch in a fixed array inside the library, so its planes must
equal vgb_render's bit for bit.  Two no-alloc calls run back to back with different frames, so
the second one also shows that what the first left in the shared array does not leak into its
result.

This file is named to be collected last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vira_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

PLANES = ("total_radiance", "direct_radiance", "indirect_radiance", "received_power", "albedo", "normal_global",
          "depth", "alpha", "triangle_id")


def _device_film(torch, B, H, W, dev, omega):
    planes = {}
    for name in PLANES:
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


def _same_bits(a, b):
    return a.shape == b.shape and np.array_equal(np.ascontiguousarray(a).view(np.uint32),
                                                 np.ascontiguousarray(b).view(np.uint32))


def test_noalloc_matches_render_on_two_calls_in_a_row(gpu):
    import torch

    scene, cam_id = workloads.path_traced(posts=65, tex=64, resolution=96, spp=4, bounces=2, rr_depth=2)
    s2 = scene.new_sphere_light(np.float32(5.0e5), 6.96e8)
    scene.set_sun_direction(s2, azimuth_deg=200.0, elevation_deg=40.0)
    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    camera = scene[cam_id]
    cam = camera.to_c(scene.origin, scene.bands.size)
    lights, nl = scene.c_lights()
    omega = scene.pixel_solid_angle(camera, cam)
    dev = omega.device
    B, H, W = scene.bands.size, cam.height, cam.width
    frames = [(4, 0, 11), (2, 3, 12)]  # (samples, frame, seed)

    def opts_for(spp, frame, seed):
        scene.pathtracer.options.samples = spp
        scene.pathtracer.options.frame = frame
        scene.pathtracer.options.seed = seed
        return scene.pathtracer.c_options(scene)

    refs = []
    for spp, frame, seed in frames:
        planes, f = _device_film(torch, B, H, W, dev, omega)
        o = opts_for(spp, frame, seed)
        capi.check(lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(o), C.byref(f)), ctx, "render")
        refs.append({k: v.cpu().numpy() for k, v in planes.items()})
    outs = []
    films = [_device_film(torch, B, H, W, dev, omega) for _ in frames]
    torch.cuda.synchronize()
    for (spp, frame, seed), (planes, f) in zip(frames, films):
        o = opts_for(spp, frame, seed)
        capi.check(lib.vgb_render_noalloc(ctx, C.byref(cam), lights, nl, C.byref(o), C.byref(f)), ctx,
                   "render_noalloc")
        st = capi.Stats()
        lib.vgb_get_stats(ctx, C.byref(st))
        assert st.rays_closest >= H * W * spp and st.rays_shadow > 0
        assert st.ms_last > 0 and st.nodes_visited == 0 and st.ms_trace == 0
        outs.append({k: v.cpu().numpy() for k, v in planes.items()})
    for ref, out in zip(refs, outs):
        for k in PLANES:
            assert _same_bits(out[k], ref[k]), k
    assert not np.array_equal(outs[0]["total_radiance"], outs[1]["total_radiance"])
    scene.close()


@pytest.mark.parametrize("nbands", [1, 4, 8])
@pytest.mark.parametrize("layout", [2, 8], ids=["bvh2", "bvh8"])
def test_noalloc_allocates_nothing(gpu, nbands, layout):
    """After one warm-up call for this band count and BVH layout (which may load their kernels
    under CUDA's lazy module loading), further calls leave the device's free memory unchanged."""
    import torch

    from vira_gb300 import Mesh, Scene, synthetic
    from vira_gb300.spectral import SpectralBands

    bands = SpectralBands.uniform(nbands, 400, 1000)
    scene = Scene(bands, device=0)
    h = synthetic.fbm_heights(65, hurst=0.8, seed=1, lo=-200.0, hi=200.0)
    scene.new_instance(scene.add_mesh(Mesh.from_dem(h, 80.0, albedo=0.12, nbands=nbands)))
    sun = scene.new_sun(temperature=5778.0)
    scene.set_sun_direction(sun, azimuth_deg=0.0, elevation_deg=30.0)
    cam_id = workloads._camera(scene, 72, 5000.0, 20.0)
    scene.pathtracer.render_passes.simulate_lighting = True
    scene.bvh_options.layout = layout
    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    camera = scene[cam_id]
    cam = camera.to_c(scene.origin, nbands)
    lights, nl = scene.c_lights()
    omega = scene.pixel_solid_angle(camera, cam)
    opts = scene.pathtracer.c_options(scene)
    planes, f = _device_film(torch, nbands, cam.height, cam.width, omega.device, omega)
    capi.check(lib.vgb_render_noalloc(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)), ctx)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(omega.device)[0]
    for _ in range(3):
        capi.check(lib.vgb_render_noalloc(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)), ctx)
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(omega.device)[0] == free0
    assert (planes["triangle_id"].cpu().numpy() != -1).any()
    scene.close()


def test_noalloc_rejects_oversized_frames(gpu):
    scene, cam_id = workloads.plain_direct(posts=65, resolution=128)
    scene.build_tlas()
    import torch

    lib = capi.load()
    ctx = scene.context()
    camera = scene[cam_id]
    cam = camera.to_c(scene.origin, scene.bands.size)
    lights, nl = scene.c_lights()
    omega = scene.pixel_solid_angle(camera, cam)
    opts = scene.pathtracer.c_options(scene)
    planes, f = _device_film(torch, 4, cam.height, cam.width, omega.device, omega)
    # a frame beyond the fixed array is refused with a message, before any device work
    big = camera.to_c(scene.origin, 4)
    big.width, big.height = 1024, 1024
    assert lib.vgb_render_noalloc(ctx, C.byref(big), lights, nl, C.byref(opts), C.byref(f)) == 1
    assert b"scratch" in lib.vgb_last_error(ctx)
    # sizes whose byte counts would wrap are refused by the pixel limit
    big.width, big.height = 2 ** 31 + 1, 2 ** 31 - 1
    assert lib.vgb_render_noalloc(ctx, C.byref(big), lights, nl, C.byref(opts), C.byref(f)) == 1
    assert b"resolution" in lib.vgb_last_error(ctx)
    # host films would need staging memory: refused
    hf = capi.Film()
    hf.on_device = 0
    assert lib.vgb_render_noalloc(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(hf)) == 1
    scene.close()
