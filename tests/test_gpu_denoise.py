"""EATWT denoiser (vgb_denoise and options.denoise) against the oracle's restatement of
denoiseSpectralRadianceEATWT.  The kernels form the same products and sums in the same order; the
exponentials (CUDA's expf against glibc's) differ by an ulp or two, so the bar is 1e-5 relative
on every pixel and band."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import gpu_render_host
from vira_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def _noisy_passes(res=48, spp=2):
    scene, cam_id = workloads.path_traced(posts=129, tex=64, resolution=res, spp=spp, bounces=2, rr_depth=1, seed=5)
    g = gpu_render_host(scene, cam_id)
    return scene, cam_id, g


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.nanmax(np.abs(a - b) / np.maximum(np.abs(b), 1e-30)))


def test_denoise_matches_oracle(gpu):
    from oracle import oracle

    scene, cam_id, g = _noisy_passes()
    lib = capi.load()
    ctx = scene.context()
    B, H, W = g["direct_radiance"].shape
    d = g["direct_radiance"].copy()
    i = g["indirect_radiance"].copy()
    capi.check(lib.vgb_denoise(ctx, capi.ptr(d), capi.ptr(i), capi.ptr(g["albedo"]), capi.ptr(g["depth"]),
                               capi.ptr(g["normal_global"]), W, H, B, None, 0), ctx, "denoise")
    od, oi = oracle.denoise(g["direct_radiance"], g["indirect_radiance"], g["albedo"], g["depth"], g["normal_global"])
    scene.close()
    assert np.array_equal(np.isnan(d), np.isnan(od))
    ok = ~np.isnan(od)
    print("direct max rel", _rel(d[ok], od[ok]), "indirect max rel", _rel(i[ok], oi[ok]))
    assert _rel(d[ok], od[ok]) <= 1e-5 and _rel(i[ok], oi[ok]) <= 1e-5
    # the filter changed the noisy planes
    assert not np.allclose(d[ok], g["direct_radiance"][ok])


def test_render_with_denoise_option(gpu):
    """options.denoise: the film's direct and indirect are the denoised planes, total is their sum
    and received power follows from it; the passes equal vgb_denoise on an undenoised render."""
    scene, cam_id, g = _noisy_passes()
    scene.pathtracer.options.denoise = True
    gd = gpu_render_host(scene, cam_id)
    lib = capi.load()
    ctx = scene.context()
    B, H, W = g["direct_radiance"].shape
    d = g["direct_radiance"].copy()
    i = g["indirect_radiance"].copy()
    capi.check(lib.vgb_denoise(ctx, capi.ptr(d), capi.ptr(i), capi.ptr(g["albedo"]), capi.ptr(g["depth"]),
                               capi.ptr(g["normal_global"]), W, H, B, None, 0), ctx, "denoise")
    scene.close()
    same = lambda a, b: np.array_equal(np.ascontiguousarray(a).view(np.uint32), np.ascontiguousarray(b).view(np.uint32))
    assert same(gd["direct_radiance"], d) and same(gd["indirect_radiance"], i)
    assert same(gd["total_radiance"], (d + i).astype(np.float32))
    for k in ("albedo", "depth", "normal_global", "alpha"):
        assert same(gd[k], g[k]), k
    assert np.array_equal(gd["triangle_id"], g["triangle_id"])


def test_denoise_in_batch_equals_per_frame(gpu):
    import torch

    scene, frames = workloads.trajectory(nframes=4, posts=129, resolutions=(32,), spps=(3,), seed=6,
                                         alt_top=3000.0, alt_bottom=900.0)
    scene.pathtracer.options.denoise = True
    planes = ("total_radiance", "direct_radiance", "indirect_radiance", "albedo", "depth", "normal_global",
              "received_power")
    batch = scene.render_batch(frames, autotune=False, use_graph=False, planes=planes)
    torch.cuda.synchronize()
    pt = scene.pathtracer
    for fr, b in zip(frames, batch):
        scene.lights[0].position = np.asarray(fr.light_positions[0], np.float64)
        pt.options.samples = fr.samples
        pt.options.frame = fr.frame
        rp = pt.render(fr.camera, scene)
        torch.cuda.synchronize()
        for k in planes:
            assert np.array_equal(b[k].cpu().numpy().view(np.uint32), getattr(rp, k).cpu().numpy().view(np.uint32)), k
    scene.close()
