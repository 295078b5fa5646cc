"""The traversal step limit on the GPU: a ray that exceeds it stops, the kernel records the limit
in the device error word and returns, and the call reports VGB_ERR_DEVICE_LIMIT.  The limit is
made to run out on a healthy scene (vgb_set_traversal_limit(ctx, 1): every ray that visits more
than one node gives up), not by faulting anything; afterwards the same context renders the
frame exactly as before."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from helpers import same_bits
from vira_gb300 import capi, workloads

pytestmark = pytest.mark.gpu

DEVICE_LIMIT = 5


def _host_render(lib, ctx, cam, lights, nl, opts, fn="vgb_render"):
    W, H = cam.width, cam.height
    tot = np.full((4, H, W), -1.0, np.float32)
    tri = np.zeros((H, W), np.uint32)
    f = capi.Film()
    f.total_radiance = tot.ctypes.data
    f.triangle_id = tri.ctypes.data
    f.on_device = 0
    return getattr(lib, fn)(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)), tot, tri


@pytest.mark.parametrize("layout", [2, 8], ids=["bvh2", "bvh8"])
def test_step_limit_reports_and_context_recovers(gpu, layout):
    scene, cam_id = workloads.plain_direct(posts=65, resolution=48)
    scene.bvh_options.layout = layout
    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    cam = scene[cam_id].to_c(scene.origin, 4)
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    rc, tot0, tri0 = _host_render(lib, ctx, cam, lights, nl, opts)
    assert rc == 0 and (tri0 != capi.NO_HIT).mean() > 0.5
    capi.check(lib.vgb_set_traversal_limit(ctx, 1), ctx)
    rc, _, _ = _host_render(lib, ctx, cam, lights, nl, opts)
    assert rc == DEVICE_LIMIT
    assert b"iterations" in lib.vgb_last_error(ctx)
    st = capi.Stats()
    lib.vgb_get_stats(ctx, C.byref(st))
    assert st.device_error & 2
    # the other entry points that traverse report the same way
    o = np.zeros((4, 3), np.float32)
    o[:, 2] = 3000.0
    d = np.tile(np.array([0.0, 0.0, -1.0], np.float32), (4, 1))
    tri = np.zeros(4, np.uint32)
    assert lib.vgb_trace_rays(ctx, capi.ptr(o), capi.ptr(d), None, 4, 0, capi.ptr(tri), None, None, 0) == DEVICE_LIMIT
    # back to the default limit: the context renders the same frame bit for bit
    capi.check(lib.vgb_set_traversal_limit(ctx, 0), ctx)
    rc, tot1, tri1 = _host_render(lib, ctx, cam, lights, nl, opts)
    assert rc == 0
    assert np.array_equal(tri1, tri0) and same_bits(tot1, tot0)
    lib.vgb_get_stats(ctx, C.byref(st))
    assert st.device_error == 0
    scene.close()


def test_step_limit_in_batch_and_noalloc(gpu):
    """The persistent batch kernel and the no-allocation render stop the same way."""
    import torch

    scene, frames = workloads.trajectory(nframes=2, posts=65, resolutions=(32,), spps=(1,), seed=2,
                                         alt_top=5000.0, alt_bottom=3000.0)
    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    ok = scene.render_batch(frames, autotune=False)
    torch.cuda.synchronize()
    capi.check(lib.vgb_set_traversal_limit(ctx, 1), ctx)
    with pytest.raises(RuntimeError, match="limit"):
        scene.render_batch(frames, autotune=False)
    cam_c = frames[0].camera.to_c(scene.origin, scene.bands.size)
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    W, H = cam_c.width, cam_c.height
    tot = torch.zeros((scene.bands.size, H, W), dtype=torch.float32, device="cuda")
    f = capi.Film()
    f.total_radiance = tot.data_ptr()
    f.on_device = 1
    assert lib.vgb_render_noalloc(ctx, C.byref(cam_c), lights, nl, C.byref(opts), C.byref(f)) == DEVICE_LIMIT
    capi.check(lib.vgb_set_traversal_limit(ctx, 0), ctx)
    again = scene.render_batch(frames, autotune=False)
    torch.cuda.synchronize()
    for a, b in zip(ok, again):
        assert torch.equal(a["total_radiance"], b["total_radiance"])
        assert torch.equal(a["triangle_id"], b["triangle_id"])
    scene.close()
