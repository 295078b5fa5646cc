"""Batched trajectory rendering (vgb_render_batch) against per-frame vgb_render calls: same
frames, same random streams, so every plane must be bit-identical."""
from __future__ import annotations

import numpy as np
import pytest

from vira_gb300 import workloads

pytestmark = pytest.mark.gpu


def _per_frame(scene, frames):
    import torch

    out = []
    pt = scene.pathtracer
    saved = [L.position.copy() for L in scene.lights]
    for fr in frames:
        for k, L in enumerate(scene.lights):
            L.position = np.asarray(fr.light_positions[k], np.float64)
        pt.options.samples = fr.samples
        pt.options.frame = fr.frame
        rp = pt.render(fr.camera, scene)
        torch.cuda.synchronize()
        out.append({"total_radiance": rp.total_radiance.cpu().numpy(), "received_power": rp.received_power.cpu().numpy(),
                    "triangle_id": rp.triangle_id.cpu().numpy(), "depth": rp.depth.cpu().numpy()})
    for k, L in enumerate(scene.lights):
        L.position = saved[k]
    return out


@pytest.mark.parametrize("bounces,graph", [(0, False), (0, True), (2, True)], ids=["direct", "direct-graph", "path-graph"])
def test_batch_equals_per_frame(gpu, bounces, graph):
    import torch

    scene, frames = workloads.trajectory(nframes=14, posts=129, resolutions=(24, 40, 64), spps=(1, 2, 5), seed=9,
                                         alt_top=8000.0, alt_bottom=400.0)
    scene.pathtracer.options.bounces = bounces
    scene.pathtracer.options.rr_depth = 1 if bounces else 0
    batch = scene.render_batch(frames, autotune=True, use_graph=graph)
    torch.cuda.synchronize()
    st = scene.pathtracer.last_stats
    assert st.rays_closest >= sum(f.camera.resolution[0] ** 2 * f.samples for f in frames)
    ref = _per_frame(scene, frames)
    for i, (b, r) in enumerate(zip(batch, ref)):
        for k in r:
            bb = b[k].cpu().numpy()
            assert bb.shape == r[k].shape
            assert np.array_equal(bb.view(np.uint32), r[k].view(np.uint32)), (i, k)
    hits = sum(int((r["triangle_id"] != -1).sum()) for r in ref)
    assert hits > 0
    scene.close()


def test_batch_graph_replay_picks_up_new_frames(gpu):
    import torch

    scene, frames = workloads.trajectory(nframes=6, posts=65, resolutions=(32,), spps=(2,), seed=4, alt_top=6000.0,
                                         alt_bottom=800.0)
    a = scene.render_batch(frames, autotune=False, use_graph=True)
    first = [x["total_radiance"].clone() for x in a]
    for fr in frames:
        fr.frame += 100  # new random streams, same shapes: the captured graph is replayed
    b = scene.render_batch(frames, autotune=False, use_graph=True)
    torch.cuda.synchronize()
    ref = _per_frame(scene, frames)
    for x, r, f0 in zip(b, ref, first):
        assert np.array_equal(x["total_radiance"].cpu().numpy(), r["total_radiance"])
    assert any(not torch.equal(x["total_radiance"], f0) for x, f0 in zip(b, first))
    scene.close()


@pytest.mark.parametrize("bounces", [0, 1])
def test_adaptive_batch_equals_per_frame(gpu, bounces):
    """Adaptive sampling (cpu_path_tracer.ipp:198-226): the persistent kernel stops each pixel at
    the same sample as the wavefront renderer and divides by the same count."""
    import torch

    scene, frames = workloads.trajectory(nframes=6, posts=129, resolutions=(24, 40), spps=(24, 33), seed=4,
                                         alt_top=3000.0, alt_bottom=800.0)
    opt = scene.pathtracer.options
    opt.bounces = bounces
    opt.adaptive_sampling = True
    opt.samples_per_batch = 4
    opt.samples_to_detect_miss = 6
    opt.sampling_tolerance = 0.2
    batch = scene.render_batch(frames, autotune=False, use_graph=False)
    torch.cuda.synchronize()
    ref = _per_frame(scene, frames)
    for i, (b, r) in enumerate(zip(batch, ref)):
        for k in r:
            assert np.array_equal(b[k].cpu().numpy().view(np.uint32), r[k].view(np.uint32)), (i, k)
    opt.adaptive_sampling = False
    full = _per_frame(scene, frames)
    changed = sum(int((~np.isclose(r["total_radiance"], f["total_radiance"], rtol=0, atol=0)).any(axis=0).sum())
                  for r, f in zip(ref, full))
    assert changed > 0, "no pixel stopped early"
    scene.close()
