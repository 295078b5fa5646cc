"""Differentiable rendering for inversion: torch.autograd.Functions over the adjoint kernels.

``RenderViews.apply(texture, heights, scene, views)`` renders the total-radiance planes of
several views ([V][B][H][W]) of a one-mesh scene whose albedo texture ([th][tw][B]) and
per-vertex heights (z of the mesh's vertices) are the parameters; ``RenderViewsPositions``
takes the vertex positions ([nverts][3]) instead, so that any per-vertex offset field (radial
offsets of an asteroid, for instance) is differentiated by torch through positions =
base + offsets * directions.  Their backward replays every path on the GPU (vgb_adjoint /
vgb_adjoint_positions).  Position gradients go through the shading normal (face normal with
flat shading, interpolated vertex normals with smooth shading) and the hit-point motion;
visibility edges are excluded.

``render_adjoint_batch(scene, views, targets)`` is the fused form: one persistent launch
renders every view, forms the L2 loss against the targets and back-propagates it
(vgb_render_adjoint_batch).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from .scene import Camera, Scene


@dataclass
class View:
    """A camera and the sun position (FP64, scene frame) it is rendered with; `samples` (per
    pixel) defaults to the scene's path-tracer options."""

    camera: Camera
    sun_position: np.ndarray
    frame: int = 0
    samples: int | None = None


def _apply_parameters(scene: Scene, texture, heights):
    """Puts the parameters into the scene: the texture through vgb_texture_update, the heights
    by moving the mesh's vertices (device update and BVH refit when they changed)."""
    mesh = scene.meshes[0]
    tex = None if texture is None else texture.detach().float().contiguous().cpu().numpy()
    z = heights.detach().float().contiguous().cpu().numpy()
    scene.build_tlas()
    if not np.array_equal(mesh.positions[:, 2], z):
        p = mesh.positions.copy()
        p[:, 2] = z
        scene.update_positions(0, p)
    if tex is not None and not np.array_equal(mesh.albedo_map, tex):
        mesh.albedo_map = tex
        scene.build_tlas()
        lib = capi.load()
        ctx = scene.context()
        capi.check(lib.vgb_texture_update(ctx, capi.ptr(tex), tex.shape[1], tex.shape[0]), ctx, "texture_update")
    scene.build_tlas()


def _apply_positions(scene: Scene, texture, positions):
    """Puts texture and vertex positions ([nverts][3]) into the scene (device update and BVH
    refit when the positions changed)."""
    mesh = scene.meshes[0]
    p = positions.detach().float().contiguous().cpu().numpy()
    scene.build_tlas()
    if not np.array_equal(mesh.positions, p):
        scene.update_positions(0, p)
    _apply_parameters(scene, texture, positions.detach()[:, 2])


def _lights_for(scene: Scene, view: View):
    arr = (capi.Light * 1)()
    L = scene.lights[0]
    p = (np.asarray(view.sun_position, np.float64) - scene.origin).astype(np.float32)
    for a in range(3):
        arr[0].position[a] = float(p[a])
    arr[0].radius = float(L.radius)
    for b in range(scene.bands.size):
        arr[0].radiance[b] = float(L.radiance[b])
    return arr


def forward_views(scene: Scene, views: list, device):
    """Renders every view; returns a list of [B][H][W] total-radiance tensors."""
    import torch

    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    B = scene.bands.size
    out = []
    for v in views:
        cam = v.camera.to_c(scene.origin, B)
        lights = _lights_for(scene, v)
        opts = scene.pathtracer.c_options(scene)
        opts.frame = v.frame
        if v.samples:
            opts.samples = v.samples
        W, H = v.camera.resolution
        img = torch.empty((B, H, W), dtype=torch.float32, device=device)
        f = capi.Film()
        f.total_radiance = img.data_ptr()
        f.on_device = 1
        torch.cuda.current_stream(device).synchronize()
        capi.check(lib.vgb_render(ctx, C.byref(cam), lights, 1, C.byref(opts), C.byref(f)), ctx, "render")
        out.append(img)
    return out


def adjoint_views(scene: Scene, views: list, grads: list, device, want_texture=True, want_heights=True,
                  positions=False):
    """Sums the adjoint of every view: returns (d_texture [th][tw][B], d_heights [nverts]), or
    (d_texture, d_positions [nverts][3]) with positions=True."""
    import torch

    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    B = scene.bands.size
    mesh = scene.meshes[0]
    nv = mesh.positions.shape[0]
    want_texture = want_texture and mesh.albedo_map is not None
    gt = torch.zeros(mesh.albedo_map.shape, dtype=torch.float32, device=device) if want_texture else None
    gz = None
    if want_heights:
        gz = torch.zeros((nv, 3) if positions else (nv,), dtype=torch.float32, device=device)
    fn = lib.vgb_adjoint_positions if positions else lib.vgb_adjoint
    for v, g in zip(views, grads):
        cam = v.camera.to_c(scene.origin, B)
        lights = _lights_for(scene, v)
        opts = scene.pathtracer.c_options(scene)
        opts.frame = v.frame
        if v.samples:
            opts.samples = v.samples
        gc = g.detach().float().contiguous()
        torch.cuda.current_stream(device).synchronize()
        capi.check(fn(ctx, C.byref(cam), lights, 1, C.byref(opts), capi.ptr(gc), capi.ptr(gt), capi.ptr(gz), 1), ctx,
                   "adjoint")
    return gt, gz


def render_adjoint_batch(scene: Scene, views: list, targets: list, device, want_texture=True, want_positions=True,
                         keep_radiance=True):
    """The fused forward + adjoint of every view in one persistent launch (vgb_render_adjoint_batch).
    targets: one [B][H][W] CUDA tensor per view.  Returns (loss, radiance planes or None per view,
    d_texture [th][tw][B] or None, d_positions [nverts][3] or None)."""
    import torch

    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    B = scene.bands.size
    mesh = scene.meshes[0]
    arr = (capi.View * len(views))()
    keep = []
    rads = []
    for i, (v, t) in enumerate(zip(views, targets)):
        f = arr[i]
        f.camera = v.camera.to_c(scene.origin, B)
        f.lights[0] = _lights_for(scene, v)[0]
        f.nlights = 1
        f.samples = v.samples or scene.pathtracer.options.samples
        f.frame = v.frame
        tc = t.detach().float().contiguous()
        keep.append(tc)
        f.target = tc.data_ptr()
        r = torch.empty_like(tc) if keep_radiance else None
        rads.append(r)
        f.radiance = r.data_ptr() if r is not None else None
    opts = scene.pathtracer.c_options(scene)
    want_texture = want_texture and mesh.albedo_map is not None
    gt = torch.zeros(mesh.albedo_map.shape, dtype=torch.float32, device=device) if want_texture else None
    gp = torch.zeros((mesh.positions.shape[0], 3), dtype=torch.float32, device=device) if want_positions else None
    loss = C.c_double(0.0)
    torch.cuda.current_stream(device).synchronize()
    capi.check(lib.vgb_render_adjoint_batch(ctx, arr, len(views), C.byref(opts), capi.ptr(gt), capi.ptr(gp),
                                            C.byref(loss)), ctx, "render_adjoint_batch")
    return loss.value, rads, gt, gp


class RenderViews:
    """``RenderViews.apply(texture, heights, scene, views)`` -> [V][B][H][W] radiance."""

    @staticmethod
    def apply(texture, heights, scene: Scene, views: list):
        import torch

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, tex, z):
                _apply_parameters(scene, tex, z)
                imgs = forward_views(scene, views, tex.device if tex.is_cuda else torch.device("cuda", scene.device))
                return torch.stack(imgs)

            @staticmethod
            def backward(ctx, grad):
                dev = grad.device
                gt, gz = adjoint_views(scene, views, list(grad.unbind(0)), dev, ctx.needs_input_grad[0],
                                       ctx.needs_input_grad[1])
                return gt, gz

        return _Fn.apply(texture, heights)


class RenderViewsPositions:
    """``RenderViewsPositions.apply(texture, positions, scene, views)`` -> [V][B][H][W] radiance,
    differentiable in the texture and the vertex positions ([nverts][3])."""

    @staticmethod
    def apply(texture, positions, scene: Scene, views: list):
        import torch

        class _Fn(torch.autograd.Function):
            @staticmethod
            def forward(ctx, tex, pos):
                _apply_positions(scene, tex, pos)
                imgs = forward_views(scene, views, pos.device if pos.is_cuda else torch.device("cuda", scene.device))
                return torch.stack(imgs)

            @staticmethod
            def backward(ctx, grad):
                gt, gp = adjoint_views(scene, views, list(grad.unbind(0)), grad.device,
                                       ctx.needs_input_grad[0] and texture is not None, ctx.needs_input_grad[1],
                                       positions=True)
                return gt, gp

        return _Fn.apply(texture, positions)
