"""vgb_render with host film planes: pageable planes are staged in device memory and copied back
after the render; pinned (cudaHostAlloc) planes are written by the kernels through their mapped
device address.  Both come out bit-identical to device planes, in any mix, with the pixel solid
angle read from pinned or pageable memory."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import same_bits_or_nan
from vira_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

PLANES = {"total_radiance": "B", "direct_radiance": "B", "received_power": "B", "albedo": "B",
          "normal_global": 3, "depth": 1, "velocity_global": 3, "triangle_size": 1, "triangle_id": 1}


def _shape(kind, B, H, W):
    if kind == "B":
        return (B, H, W)
    return (kind, H, W) if kind != 1 else (H, W)


def _render(lib, ctx, cam, lights, nl, opts, planes, omega, on_device):
    f = capi.Film()
    for k, t in planes.items():
        setattr(f, k, t.data_ptr())
    f.pixel_solid_angle = omega.data_ptr()
    f.on_device = 1 if on_device else 0
    capi.check(lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)), ctx, "render")


@pytest.mark.parametrize("mix", ["pinned", "pageable", "mixed"])
def test_host_film_pinned_and_pageable_equal_device(gpu, mix):
    import torch

    scene, cam_id = workloads.path_traced(posts=65, tex=64, resolution=72, spp=3, bounces=2, rr_depth=1, seed=4)
    scene.pathtracer.render_passes.save_velocity = True
    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    camera = scene[cam_id]
    cam = camera.to_c(scene.origin, scene.bands.size)
    cam.width, cam.height = 72, 40   # a frame that is not whole 8x4 tiles
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    B, H, W = scene.bands.size, cam.height, cam.width
    omega_d = torch.rand((H, W), device="cuda") * 1e-6
    dev = {k: torch.full(_shape(v, B, H, W), -9.0, device="cuda",
                         dtype=torch.int32 if k == "triangle_id" else torch.float32) for k, v in PLANES.items()}
    _render(lib, ctx, cam, lights, nl, opts, dev, omega_d, True)
    torch.cuda.synchronize()
    ref = {k: v.cpu().numpy() for k, v in dev.items()}
    host = {}
    for i, (k, t) in enumerate(dev.items()):
        pinned = mix == "pinned" or (mix == "mixed" and i % 2 == 0)
        host[k] = torch.full(t.shape, -7, dtype=t.dtype, pin_memory=pinned)
    omega_h = omega_d.cpu().pin_memory() if mix != "pageable" else omega_d.cpu()
    _render(lib, ctx, cam, lights, nl, opts, host, omega_h, False)
    for k in PLANES:
        got = host[k].numpy()
        if k == "triangle_id":
            assert np.array_equal(got, ref[k]), k
        else:
            assert same_bits_or_nan(got, ref[k]), k
    assert (ref["triangle_id"] != -1).mean() > 0.3
    scene.close()


@pytest.mark.parametrize("any_hit", [False, True], ids=["closest", "any"])
def test_trace_rays_pinned_and_pageable_buffers(gpu, any_hit):
    """vgb_trace_rays (the TLAS::intersect seam) reads pinned ray buffers and writes pinned result
    buffers through their mapped addresses, pageable ones through staging: same answers."""
    import torch

    scene, cam_id = workloads.plain_direct(posts=129, resolution=64)
    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    rng = np.random.default_rng(8)
    n = 5000
    o = np.zeros((n, 3), np.float32)
    o[:, :2] = rng.uniform(-400.0, 400.0, (n, 2))
    o[:, 2] = 3000.0
    d = rng.normal(size=(n, 3)).astype(np.float32)
    d[:, 2] = -np.abs(d[:, 2]) - 0.5
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    tm = np.full(n, 5000.0, np.float32)
    results = []
    for pinned in (False, True):
        buf = {"o": torch.from_numpy(o.copy()), "d": torch.from_numpy(d.copy()), "tm": torch.from_numpy(tm.copy()),
               "tri": torch.zeros(n, dtype=torch.int32), "t": torch.zeros(n), "w": torch.zeros((n, 3))}
        if pinned:
            buf = {k: v.pin_memory() for k, v in buf.items()}
        capi.check(lib.vgb_trace_rays(ctx, buf["o"].data_ptr(), buf["d"].data_ptr(), buf["tm"].data_ptr(), n,
                                      int(any_hit), buf["tri"].data_ptr(), buf["t"].data_ptr(), buf["w"].data_ptr(), 0),
                   ctx, "trace_rays")
        results.append({k: buf[k].numpy().copy() for k in ("tri", "t", "w")})
    a, b = results
    assert np.array_equal(a["tri"], b["tri"])
    assert np.array_equal(a["t"].view(np.uint32), b["t"].view(np.uint32))
    assert np.array_equal(a["w"].view(np.uint32), b["w"].view(np.uint32))
    assert (a["tri"] != -1).mean() > 0.3
    scene.close()
