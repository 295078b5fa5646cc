"""Adjoint (vgb_adjoint) against central finite differences of the rendered L2 loss.

Albedo texels are checked through 2 bounces (every contribution is linear in the albedo of each
path vertex, so the path-replay gradient is exact) at a step of 1e-3.  Heights are checked with
direct lighting: the gradient goes through the face normals and the hit-point motion;
visibility edges are excluded by design, so a parameter whose finite difference moves a
silhouette is skipped.  The height step is 1e-2 m: at 1e-3 m the radiance change (~1e-4) sits
at the FP32 rounding floor of the renders and the finite differences scatter by ~5e-3, while
at 1e-2 m they agree to ~5e-4.  The FP64 oracle, on the same sampled paths, is the tight check.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vira_gb300 import FOUR_BAND, Mesh, Scene, capi, synthetic

pytestmark = pytest.mark.gpu


def _scene(bounces, posts=65, tex=64, res=48, seed=4):
    h = synthetic.fbm_heights(posts, 0.8, seed=seed, lo=-60.0, hi=60.0)
    h = synthetic.add_crater_field(h, 2000.0 / (posts - 1), seed=seed + 1, dmin=40, dmax=400)
    alb = synthetic.lognormal_albedo(tex, 0.12, 0.3, seed=seed + 2)
    s = Scene(FOUR_BAND)
    m = Mesh.from_dem(h, 2000.0 / (posts - 1), albedo=1.0, nbands=4)
    m.uv = synthetic.grid_uvs(posts, posts, posts - 1)
    m.albedo_map = np.ascontiguousarray(np.repeat(alb[:, :, None], 4, axis=2))
    s.add_mesh(m)
    s.new_instance(("mesh", 0))
    sun = s.new_sun(5778.0)
    s.set_sun_direction(sun, 30.0, 35.0)
    cid = s.new_camera()
    c = s[cid]
    c.set_resolution(res, res)
    c.set_sensor_size(0.036)
    c.set_field_of_view(30.0)
    c.set_local_position(100.0, -200.0, 2500.0)
    c.look_at((0.0, 0.0, 0.0))
    pt = s.pathtracer
    pt.options.samples = 4
    pt.options.bounces = bounces
    pt.options.deterministic_light = False
    pt.options.seed = 11
    pt.render_passes.simulate_lighting = True
    return s, cid


def _render(s, cid):
    import torch

    rp = s.pathtracer.render(s[cid], s)
    torch.cuda.synchronize()
    return rp.total_radiance.cpu().numpy().astype(np.float64)


def _adjoint(s, cid, dl, tex=True, height=True):
    lib = capi.load()
    ctx = s.context()
    cam = s[cid].to_c(s.origin, 4)
    lights, nl = s.c_lights()
    opts = s.pathtracer.c_options(s)
    m = s.meshes[0]
    gt = np.zeros(m.albedo_map.shape, np.float32) if tex else None
    gh = np.zeros(m.positions.shape[0], np.float32) if height else None
    d = np.ascontiguousarray(dl, np.float32)
    capi.check(lib.vgb_adjoint(ctx, C.byref(cam), lights, nl, C.byref(opts), capi.ptr(d), capi.ptr(gt), capi.ptr(gh), 0),
               ctx, "adjoint")
    return gt, gh


def _loss(img, target):
    return float(np.sum((img - target) ** 2))


def test_albedo_gradient_matches_finite_differences(gpu):
    s, cid = _scene(bounces=2)
    m = s.meshes[0]
    base = m.albedo_map.copy()
    rng = np.random.default_rng(0)
    target_tex = (base * (1 + 0.05 * rng.standard_normal(base.shape[:2]))[:, :, None]).astype(np.float32)
    m.albedo_map = target_tex
    s.mark_dirty()
    target = _render(s, cid)
    m.albedo_map = base
    s.mark_dirty()
    img = _render(s, cid)
    gt, _ = _adjoint(s, cid, 2.0 * (img - target), tex=True, height=False)
    g_texel = gt.sum(axis=2)  # one scalar parameter per texel, replicated over the bands
    cand = np.argwhere(np.abs(g_texel) > np.percentile(np.abs(g_texel), 90))
    pick = cand[rng.choice(len(cand), size=min(12, len(cand)), replace=False)]
    lib = capi.load()
    ctx = s.context()
    errs = []
    step = 1e-3
    for (y, x) in pick:
        vals = []
        for sgn in (+1, -1):
            t = base.copy()
            t[y, x, :] += sgn * step
            capi.check(lib.vgb_texture_update(ctx, capi.ptr(np.ascontiguousarray(t)), t.shape[1], t.shape[0]), ctx)
            vals.append(_loss(_render(s, cid), target))
        fd = (vals[0] - vals[1]) / (2 * step)
        errs.append(abs(fd - g_texel[y, x]) / max(abs(fd), 1e-12))
    capi.check(lib.vgb_texture_update(ctx, capi.ptr(np.ascontiguousarray(base)), base.shape[1], base.shape[0]), ctx)
    s.close()
    errs = np.array(errs)
    print("albedo FD relative errors:", np.round(errs, 6))
    assert np.median(errs) <= 1e-3 and np.mean(errs <= 1e-2) >= 0.9


def test_height_gradient_matches_finite_differences(gpu):
    s, cid = _scene(bounces=0)
    m = s.meshes[0]
    base = m.positions.copy()
    rng = np.random.default_rng(1)
    m.positions = base + np.stack([np.zeros(len(base)), np.zeros(len(base)), rng.normal(0, 0.5, len(base))], 1).astype(np.float32)
    m.normals = None
    s.mark_dirty()
    target = _render(s, cid)
    m.positions = base.copy()
    m.normals = None
    s.mark_dirty()
    img = _render(s, cid)
    tri0 = s.pathtracer.render_passes.triangle_id.cpu().numpy().copy()
    _, gh = _adjoint(s, cid, 2.0 * (img - target), tex=False, height=True)
    cand = np.nonzero(np.abs(gh) > np.percentile(np.abs(gh), 95))[0]
    pick = rng.choice(cand, size=min(12, len(cand)), replace=False)
    errs = []
    step = 1e-2
    for v in pick:
        vals = []
        flipped = False
        for sgn in (+1, -1):
            p = base.copy()
            p[v, 2] += sgn * step
            m.positions = p
            m.normals = None
            s.mark_dirty()
            vals.append(_loss(_render(s, cid), target))
            st = s.pathtracer.last_stats
            flipped |= not np.array_equal(s.pathtracer.render_passes.triangle_id.cpu().numpy(), tri0)
        if flipped:
            continue  # a silhouette moved across a sample: a visibility edge, excluded
        fd = (vals[0] - vals[1]) / (2 * step)
        errs.append(abs(fd - gh[v]) / max(abs(fd), 1e-12))
    m.positions = base
    s.close()
    errs = np.array(errs)
    print("height FD relative errors:", np.round(errs, 6))
    assert len(errs) >= 6
    assert np.median(errs) <= 1e-3 and np.mean(errs <= 1e-2) >= 0.8


@pytest.mark.parametrize("bounces,kind", [(2, "albedo"), (0, "height")])
def test_gradients_match_fp64_oracle_on_the_same_paths(gpu, bounces, kind):
    from oracle import oracle

    s, cid = _scene(bounces=bounces, res=40)
    img = _render(s, cid)
    rng = np.random.default_rng(3)
    dl = rng.standard_normal(img.shape).astype(np.float32)
    gt, gh = _adjoint(s, cid, dl, tex=kind == "albedo", height=kind == "height")
    cam = s[cid].to_c(s.origin, 4)
    lights, nl = s.c_lights()
    opts = s.pathtracer.c_options(s)
    osc = oracle.OracleScene.from_flat(s.flat, 4)
    ot, oh = osc.adjoint(cam, lights, nl, opts, dl, tex_shape=s.flat["texture"].shape if kind == "albedo" else None,
                         nverts=s.flat["positions"].shape[0] if kind == "height" else None)
    osc.close()
    s.close()
    a, b = (gt, ot) if kind == "albedo" else (gh, oh)
    a = a.astype(np.float64).ravel()
    b = b.ravel()
    rel = np.linalg.norm(a - b) / np.linalg.norm(b)
    big = np.abs(b) > 1e-2 * np.abs(b).max()
    comp = np.abs(a[big] - b[big]) / np.abs(b[big])
    print(f"{kind}: relative L2 error {rel:.2e}, max component error {comp.max():.2e} over {big.sum()} components")
    assert rel <= 1e-3
    assert np.quantile(comp, 0.99) <= 1e-3


def test_autograd_function_matches_adjoint_and_descends(gpu):
    import torch

    from vira_gb300 import workloads
    from vira_gb300.autograd import RenderViews, _apply_parameters, forward_views

    scene, views = workloads.inversion(posts=129, tex=128, resolution=40, nviews=3, spp=4, bounces=1)
    mesh = scene.meshes[0]
    base_tex = torch.tensor(mesh.albedo_map.copy())
    base_z = torch.tensor(mesh.positions[:, 2].copy())
    rng = np.random.default_rng(7)
    tgt_tex = base_tex * torch.tensor(1.0 + 0.05 * rng.standard_normal(base_tex.shape[:2]), dtype=torch.float32)[:, :, None]
    _apply_parameters(scene, tgt_tex, base_z)
    dev = torch.device("cuda", 0)
    target = torch.stack(forward_views(scene, views, dev))
    tex = base_tex.clone().to(dev).requires_grad_(True)
    z = base_z.clone().to(dev).requires_grad_(True)
    img = RenderViews.apply(tex, z, scene, views)
    loss = ((img - target) ** 2).sum()
    loss.backward()
    assert tex.grad is not None and z.grad is not None
    assert float(tex.grad.abs().sum()) > 0
    # a small step against the texture gradient lowers the loss
    with torch.no_grad():
        g = tex.grad
        step = 0.2 * float(loss) / float((g * g).sum())
        tex2 = (tex - step * g).detach()
    img2 = RenderViews.apply(tex2, z.detach(), scene, views)
    loss2 = float(((img2 - target) ** 2).sum())
    print(f"loss {float(loss):.6g} -> {loss2:.6g}")
    assert loss2 < float(loss)
    scene.close()
