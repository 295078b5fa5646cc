"""Differentiable rendering for inversion: a torch.autograd.Function over the adjoint kernel.

``render_views(texture, heights, scene, views)`` renders the total-radiance planes of several
views ([V][B][H][W]) of a one-DEM scene whose albedo texture ([th][tw][B]) and per-vertex
heights (z of the mesh's vertices) are the parameters.  Its backward replays every path on the
GPU (vgb_adjoint) and returns d loss / d texture and d loss / d heights.  Height gradients go
through face normals and hit-point motion (flat shading); visibility edges are excluded.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import capi
from .scene import Camera, Scene


@dataclass
class View:
    """A camera and the sun position (FP64, scene frame) it is rendered with."""

    camera: Camera
    sun_position: np.ndarray
    frame: int = 0


def _apply_parameters(scene: Scene, texture, heights):
    """Puts the parameters into the scene: the texture through vgb_texture_update, the heights
    by moving the mesh's vertices (re-upload and BVH rebuild when they changed)."""
    mesh = scene.meshes[0]
    tex = texture.detach().float().contiguous().cpu().numpy()
    z = heights.detach().float().contiguous().cpu().numpy()
    if not np.array_equal(mesh.positions[:, 2], z):
        p = mesh.positions.copy()
        p[:, 2] = z
        mesh.positions = p
        mesh.normals = None
        mesh.albedo_map = tex
        scene.mark_dirty()
        scene.build_tlas()
    elif not np.array_equal(mesh.albedo_map, tex):
        mesh.albedo_map = tex
        scene.build_tlas()
        lib = capi.load()
        ctx = scene.context()
        capi.check(lib.vgb_texture_update(ctx, capi.ptr(tex), tex.shape[1], tex.shape[0]), ctx, "texture_update")
    scene.build_tlas()


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
        W, H = v.camera.resolution
        img = torch.empty((B, H, W), dtype=torch.float32, device=device)
        f = capi.Film()
        f.total_radiance = img.data_ptr()
        f.on_device = 1
        torch.cuda.current_stream(device).synchronize()
        capi.check(lib.vgb_render(ctx, C.byref(cam), lights, 1, C.byref(opts), C.byref(f)), ctx, "render")
        out.append(img)
    return out


def adjoint_views(scene: Scene, views: list, grads: list, device, want_texture=True, want_heights=True):
    """Sums the adjoint of every view: returns (d_texture [th][tw][B], d_heights [nverts])."""
    import torch

    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    B = scene.bands.size
    mesh = scene.meshes[0]
    gt = torch.zeros(mesh.albedo_map.shape, dtype=torch.float32, device=device) if want_texture else None
    gz = torch.zeros(mesh.positions.shape[0], dtype=torch.float32, device=device) if want_heights else None
    for v, g in zip(views, grads):
        cam = v.camera.to_c(scene.origin, B)
        lights = _lights_for(scene, v)
        opts = scene.pathtracer.c_options(scene)
        opts.frame = v.frame
        gc = g.detach().float().contiguous()
        torch.cuda.current_stream(device).synchronize()
        capi.check(lib.vgb_adjoint(ctx, C.byref(cam), lights, 1, C.byref(opts), capi.ptr(gc), capi.ptr(gt),
                                   capi.ptr(gz), 1), ctx, "adjoint")
    return gt, gz


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
