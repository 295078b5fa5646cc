"""Parity at the benchmark configurations (the workloads bench.py times), not only at reduced
sizes:

  * plain direct lighting at full size (513^2 fBm DEM, 0.52M triangles, 1024^2, 4 bands, 1 spp +
    1 shadow ray): triangle ids bit-exact, hit distances within 1e-5 relative, every band within
    1e-4 relative; the edge-grazing count against the reference's own triangle test is printed;
  * path tracing on the crater terrain with the full 4096^2 lognormal texture at 64 spp, 3 bounces
    and Russian roulette after bounce 2 (DEM at 2049^2 posts, 8.4M triangles, 1024^2 image, so the
    oracle's CPU BVH builds in seconds): a band of rows rendered by the oracle at full spp against
    the GPU frame, same-seed paths equal to 1e-4 almost everywhere and image means within 3 sigma;
  * the adjoint on the full inversion scene (1025^2 crater DEM, 2.1M triangles, 1024^2 texture,
    512^2 view, 16 spp, 2 bounces): 64 random parameters (32 albedo texels, 32 vertex heights)
    against the FP64 oracle on the same sampled paths, and the albedo ones against central finite
    differences at a step of 1e-3, with dL/dI on a 64x64 pixel window.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import gpu_render_host, oracle_render, primary_rays, rel_err
from vira_gb300 import capi, workloads

pytestmark = pytest.mark.gpu


def test_plain_direct_full_size(gpu):
    from oracle import oracle

    scene, cam_id = workloads.plain_direct()
    scene.build_tlas()
    cam = scene[cam_id].to_c(scene.origin, 4)
    assert (cam.width, cam.height) == (1024, 1024) and scene.flat["indices"].shape[0] == 524288
    g = gpu_render_host(scene, cam_id)
    omega = scene.pixel_solid_angle(scene[cam_id], cam).cpu().numpy()
    o, counts = oracle_render(scene, cam_id, omega=omega)
    assert np.array_equal(g["triangle_id"], o["triangle_id"])
    hit = o["triangle_id"] != capi.NO_HIT
    assert hit.mean() > 0.5   # the far part of the view looks past the DEM's edge
    assert float(rel_err(g["depth"][hit], o["depth"][hit]).max()) <= 1e-5
    for k in ("total_radiance", "direct_radiance", "received_power", "albedo"):
        assert float(rel_err(g[k], o[k]).max()) <= 1e-4, k
    st = scene.pathtracer.last_stats
    assert (st.rays_closest, st.rays_shadow) == counts
    # primary rays: distances from the ray queries, edge-grazing count against the reference test
    org, dirs = primary_rays(cam)
    tri_g, t_g, _ = scene.intersect(org, dirs)
    osc = oracle.OracleScene.from_flat(scene.flat, 4)
    tri_o, t_o, _ = osc.trace(org, dirs)
    tri_r, _, _ = osc.trace(org, dirs, mode=1)
    osc.close()
    assert np.array_equal(tri_g, tri_o)
    h = tri_o != capi.NO_HIT
    assert float(rel_err(t_g[h], t_o[h]).max()) <= 1e-5
    grazing = int(np.count_nonzero(tri_r != tri_o))
    print(f"edge-grazing rays at full size: {grazing} of {tri_o.size}")
    assert grazing <= tri_o.size // 100
    scene.close()


def test_path_traced_config_rows_statistical(gpu):
    scene, cam_id = workloads.path_traced(posts=2049, tex=4096, resolution=1024, spp=64, bounces=3, rr_depth=2)
    g = gpu_render_host(scene, cam_id)
    H = scene[cam_id].resolution[1]
    r0, r1 = H // 2 - 8, H // 2 + 8
    o, counts = oracle_render(scene, cam_id, rows=(r0, r1))
    scene.pathtracer.options.seed = 8
    g8 = gpu_render_host(scene, cam_id)
    scene.close()
    a = g["total_radiance"][:, r0:r1]
    b = o["total_radiance"][:, r0:r1]
    c = g8["total_radiance"][:, r0:r1]
    assert np.array_equal(g["triangle_id"][r0:r1], o["triangle_id"][r0:r1])
    close = rel_err(a, b) <= 1e-4
    print(f"same-seed pixels within 1e-4: {close.mean():.4f}")
    assert close.mean() >= 0.98
    sig = np.sqrt(np.maximum(np.var(a - c, axis=(1, 2)) / 2.0, 1e-30))
    n = a.shape[1] * a.shape[2]
    dm = np.abs(a.mean(axis=(1, 2)) - b.mean(axis=(1, 2)))
    assert np.all(dm <= 3 * sig * np.sqrt(2.0 / n) + 1e-6), (dm, sig)
    assert g["indirect_radiance"][:, r0:r1].mean() > 0


def test_inversion_gradients_full_scene(gpu):
    import torch

    from oracle import oracle
    from vira_gb300.autograd import _lights_for

    scene, views = workloads.inversion()
    scene.build_tlas()
    v = views[0]
    mesh = scene.meshes[0]
    cam = v.camera.to_c(scene.origin, 4)
    W, H = v.camera.resolution
    lights = _lights_for(scene, v)
    opts = scene.pathtracer.c_options(scene)
    opts.frame = v.frame
    rng = np.random.default_rng(64)
    dl = np.zeros((4, H, W), np.float32)
    y0, x0 = H // 2 - 32, W // 2 - 32
    dl[:, y0:y0 + 64, x0:x0 + 64] = rng.standard_normal((4, 64, 64)).astype(np.float32)
    lib = capi.load()
    ctx = scene.context()
    gt = np.zeros(mesh.albedo_map.shape, np.float32)
    gz = np.zeros(mesh.positions.shape[0], np.float32)
    capi.check(lib.vgb_adjoint(ctx, C.byref(cam), lights, 1, C.byref(opts), capi.ptr(dl), capi.ptr(gt), capi.ptr(gz), 0),
               ctx, "adjoint")
    osc = oracle.OracleScene.from_flat(scene.flat, 4)
    ot, oz = osc.adjoint(cam, lights, 1, opts, dl, tex_shape=gt.shape, nverts=gz.shape[0])
    osc.close()
    g_tex = gt.sum(axis=2)
    o_tex = ot.sum(axis=2)
    tex_c = np.argwhere(np.abs(o_tex) > 1e-3 * np.abs(o_tex).max())
    z_c = np.nonzero(np.abs(oz) > 1e-3 * np.abs(oz).max())[0]
    pt = tex_c[rng.choice(len(tex_c), 32, replace=False)]
    pz = rng.choice(z_c, 32, replace=False)
    e_tex = np.abs(g_tex[pt[:, 0], pt[:, 1]] - o_tex[pt[:, 0], pt[:, 1]]) / np.abs(o_tex[pt[:, 0], pt[:, 1]])
    e_z = np.abs(gz[pz] - oz[pz]) / np.abs(oz[pz])
    print(f"FP64 oracle: albedo max rel {e_tex.max():.2e}, height max rel {e_z.max():.2e}")
    assert e_tex.max() <= 1e-3 and np.median(e_z) <= 1e-3 and np.mean(e_z <= 1e-2) >= 0.95
    # central finite differences of L = sum(dL/dI * I) for the albedo texels (linear in each)
    base = mesh.albedo_map.copy()
    film = torch.empty((4, H, W), dtype=torch.float32, device="cuda")
    f = capi.Film()
    f.total_radiance = film.data_ptr()
    f.on_device = 1
    dlt = torch.tensor(dl, device="cuda", dtype=torch.float64)

    def loss():
        capi.check(lib.vgb_render(ctx, C.byref(cam), lights, 1, C.byref(opts), C.byref(f)), ctx, "render")
        torch.cuda.synchronize()
        return float((film.double() * dlt).sum())

    step = 1e-3
    errs = []
    for (y, x) in pt:
        vals = []
        for sgn in (+1, -1):
            t = base.copy()
            t[y, x, :] += sgn * step
            capi.check(lib.vgb_texture_update(ctx, capi.ptr(np.ascontiguousarray(t)), t.shape[1], t.shape[0]), ctx)
            vals.append(loss())
        fd = (vals[0] - vals[1]) / (2 * step)
        errs.append(abs(fd - g_tex[y, x]) / max(abs(fd), 1e-12))
    capi.check(lib.vgb_texture_update(ctx, capi.ptr(np.ascontiguousarray(base)), base.shape[1], base.shape[0]), ctx)
    scene.close()
    errs = np.array(errs)
    print("albedo FD relative errors:", np.round(np.sort(errs), 6))
    assert np.median(errs) <= 1e-3 and np.mean(errs <= 1e-2) >= 0.9
