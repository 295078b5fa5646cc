"""Normal maps (row a12: Material::getNormal, materials/material.ipp:129-143, applied in
processIntersection at cpu_path_tracer.ipp:316-329 and in the rasterizer at
cpu_rasterizer.ipp:177-191) on the GPU against the oracle.

The map's sample (wrap + bilinear at uv x resolution) is taken to the scene frame by the tangent
frame of the geometric shading normal; the result drives next-event estimation, MIS and the film's
normal, while the continuation direction is sampled in the frame built before the map.  Direct
lighting with deterministic light sampling is bit-identical to the oracle; path tracing agrees
sample for sample up to CUDA's and glibc's transcendentals; the rasterizer is bit-identical.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import gpu_render_host, oracle_render, rel_err, same_bits, same_bits_or_nan
from vira_gb300 import capi, synthetic, workloads

pytestmark = pytest.mark.gpu


def bumpy_normal_map(n=64, seed=11, slope=0.35):
    """A seeded tangent-space normal map: unit vectors tilted by up to `slope` from +z."""
    rng = np.random.default_rng(seed)
    g = rng.standard_normal((n, n, 2)).astype(np.float32)
    k = np.ones((5, 5), np.float32) / 25.0   # smooth the tilts over a few texels
    sm = np.empty_like(g)
    for c in range(2):
        p = np.pad(g[:, :, c], 2, mode="wrap")
        sm[:, :, c] = sum(p[i:i + n, j:j + n] * k[i, j] for i in range(5) for j in range(5))
    sm *= slope / max(1e-6, float(np.abs(sm).max()))
    v = np.concatenate([sm, np.ones((n, n, 1), np.float32)], 2)
    return (v / np.linalg.norm(v, axis=2, keepdims=True)).astype(np.float32)


def _scene(kind="direct", **kw):
    if kind == "direct":
        scene, cam_id = workloads.plain_direct(posts=129, resolution=kw.get("resolution", 64))
        posts = 129
    else:
        scene, cam_id = workloads.path_traced(posts=65, tex=64, resolution=kw.get("resolution", 48), spp=4,
                                              bounces=2, rr_depth=0, seed=5)
        posts = 65
    m = scene.meshes[0]
    if m.uv is None:
        m.uv = synthetic.grid_uvs(posts, posts, 8)
    m.normal_map = bumpy_normal_map()
    scene.mark_dirty()
    return scene, cam_id


@pytest.mark.parametrize("smooth", [False, True])
def test_direct_render_with_normal_map_bit_exact(gpu, smooth):
    scene, cam_id = _scene()
    scene.meshes[0].set_smooth_shading(smooth)
    g = gpu_render_host(scene, cam_id)
    o, _ = oracle_render(scene, cam_id)
    assert np.array_equal(g["triangle_id"], o["triangle_id"])
    for k in ("total_radiance", "direct_radiance", "albedo", "normal_global", "depth", "alpha"):
        assert same_bits_or_nan(g[k], o[k]), k
    # the map does change the shading
    scene.meshes[0].normal_map = None
    scene.mark_dirty()
    flat = gpu_render_host(scene, cam_id)
    hit = g["triangle_id"] != capi.NO_HIT
    assert float(rel_err(g["total_radiance"][:, hit], flat["total_radiance"][:, hit]).mean()) > 1e-2
    assert np.array_equal(flat["triangle_id"], g["triangle_id"])
    scene.close()


def test_path_traced_with_normal_map_matches_oracle(gpu):
    scene, cam_id = _scene("path")
    g = gpu_render_host(scene, cam_id)
    o, _ = oracle_render(scene, cam_id)
    assert np.array_equal(g["triangle_id"], o["triangle_id"])
    close = rel_err(g["total_radiance"], o["total_radiance"]) <= 1e-4
    assert close.mean() >= 0.98, close.mean()
    assert same_bits_or_nan(g["normal_global"], o["normal_global"])
    assert g["indirect_radiance"].mean() > 0
    scene.close()


def test_rasterizer_with_normal_map(gpu):
    from test_gpu_raster import _compare, _dem_scene

    for smooth in (False, True):
        s, cid = _dem_scene(smooth=smooth, res=72)
        s.meshes[0].normal_map = bumpy_normal_map(48, seed=3)
        s.mark_dirty()
        covered, _ = _compare(s, cid, f"normal map, smooth={smooth}")
        assert covered > 0.5
        s.close()


def test_adjoint_rejects_a_normal_map(gpu):
    scene, views = workloads.inversion(posts=65, tex=32, resolution=16, nviews=1, spp=1, bounces=0)
    scene.meshes[0].normal_map = bumpy_normal_map(16)
    scene.mark_dirty()
    scene.build_tlas()
    v = views[0]
    cam = v.camera.to_c(scene.origin, scene.bands.size)
    from vira_gb300.autograd import _lights_for

    lights = _lights_for(scene, v)
    opts = scene.pathtracer.c_options(scene)
    dl = np.ones((scene.bands.size, 16, 16), np.float32)
    gt = np.zeros(scene.meshes[0].albedo_map.shape, np.float32)
    lib = capi.load()
    ctx = scene.context()
    assert lib.vgb_adjoint(ctx, C.byref(cam), lights, 1, C.byref(opts), capi.ptr(dl), capi.ptr(gt), None, 0) == 1
    assert b"normal map" in lib.vgb_last_error(ctx)
    scene.close()


@pytest.mark.parametrize("bounces", [0, 2], ids=["direct", "path"])
def test_batch_with_normal_map_equals_per_frame(gpu, bounces):
    """The batched trajectory kernels shade through the same normal map: the lean direct kernel
    (which builds the tangent frame only for the map) and the general one with bounces."""
    import torch

    scene, frames = workloads.trajectory(nframes=3, posts=129, resolutions=(40, 56), spps=(1, 3), seed=7,
                                         alt_top=5000.0, alt_bottom=2500.0)
    m = scene.meshes[0]
    if m.uv is None:
        m.uv = synthetic.grid_uvs(129, 129, 8)
    m.normal_map = bumpy_normal_map()
    scene.mark_dirty()
    scene.pathtracer.options.bounces = bounces
    scene.pathtracer.options.rr_depth = 0
    planes = ("total_radiance", "normal_global", "triangle_id", "depth")
    batch = scene.render_batch(frames, autotune=False, use_graph=False, planes=planes)
    torch.cuda.synchronize()
    pt = scene.pathtracer
    for fr, b in zip(frames, batch):
        for k, L in enumerate(scene.lights):
            L.position = np.asarray(fr.light_positions[k], np.float64)
        pt.options.samples = fr.samples
        pt.options.frame = fr.frame
        rp = pt.render(fr.camera, scene)
        torch.cuda.synchronize()
        for k in planes:
            got, want = b[k].cpu().numpy(), getattr(rp, k).cpu().numpy()
            if k == "triangle_id":
                assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
            else:
                assert same_bits_or_nan(got, want), k
    scene.close()
