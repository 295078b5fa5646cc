"""The GPU BVH builder (vgb_bvh_options.builder = 1: linear BVH in Morton order, built on the device)
against the host binned-SAH builder.  The closest hit does not depend on the BVH and occlusion is
a yes/no answer, so every render pass and every ray batch must come out identical with either
tree -- a missing triangle, a wrong box or a broken link shows up as a different hit.  Also: leaf
sizes 1..8, a refit on top of a GPU-built tree, and a scene small enough to be one leaf.
"""
from __future__ import annotations

import numpy as np
import pytest

from vira_gb300 import FOUR_BAND, Mesh, Scene, capi, synthetic

pytestmark = pytest.mark.gpu


def _scene(mesh_list, builder, leaf=0, cam_pos=(150.0, -300.0, 900.0), res=64, bounces=2, smooth=False):
    s = Scene(FOUR_BAND)
    s.bvh_options = capi.BvhOptions(leaf, builder, 0, 2)
    for k, m in enumerate(mesh_list):
        mm = Mesh(positions=m.positions.copy(), indices=m.indices.copy(),
                  albedo=None if m.albedo is None else m.albedo.copy(), uv=None if m.uv is None else m.uv.copy(),
                  albedo_map=m.albedo_map, smooth_shading=smooth)
        s.add_mesh(mm)
        s.new_instance(("mesh", k))
    sun = s.new_sun(5778.0)
    s.set_sun_direction(sun, 30.0, 35.0)
    cid = s.new_camera()
    c = s[cid]
    c.set_resolution(res, res)
    c.set_sensor_size(0.036)
    c.set_field_of_view(40.0)
    c.set_local_position(*cam_pos)
    c.look_at((0.0, 0.0, 0.0))
    pt = s.pathtracer
    pt.options.samples = 3
    pt.options.bounces = bounces
    pt.options.seed = 9
    pt.render_passes.simulate_lighting = True
    return s, cid


def _dem(posts=129, holes=False, seed=3):
    h = synthetic.fbm_heights(posts, 0.8, seed=seed, lo=-60.0, hi=60.0)
    h = synthetic.add_crater_field(h, 1000.0 / (posts - 1), seed=seed + 1, dmin=40, dmax=300)
    h = np.ascontiguousarray(h, np.float32)
    if holes:
        h[10:20, 30:45] = np.inf
    m = Mesh.from_dem(h, 1000.0 / (posts - 1), albedo=np.array([0.1, 0.12, 0.14, 0.2], np.float32), nbands=4)
    m.uv = synthetic.grid_uvs(posts, posts, posts - 1)
    return m


def _render(s, cid):
    import torch

    rp = s.pathtracer.render(s[cid], s)
    torch.cuda.synchronize()
    return {k: getattr(rp, k).cpu().numpy().copy() for k in ("total_radiance", "triangle_id", "depth", "normal_global")}


def _rays(n, seed, spread):
    rng = np.random.default_rng(seed)
    o = rng.normal(0.0, spread, (n, 3)).astype(np.float32)
    o[:, 2] = np.abs(o[:, 2]) + 200.0
    d = rng.normal(0.0, 0.3 * spread, (n, 3)) - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def _same(meshes, leaf=0, smooth=False, cam_pos=(150.0, -300.0, 900.0), nrays=8192, spread=500.0):
    a, ca = _scene(meshes, 0, leaf, cam_pos, smooth=smooth)
    b, cb = _scene(meshes, 1, leaf, cam_pos, smooth=smooth)
    ra, rb = _render(a, ca), _render(b, cb)
    for k in ra:
        assert np.array_equal(ra[k], rb[k], equal_nan=True), f"{k} differs at {np.sum(ra[k] != rb[k])} values"
    o, d = _rays(nrays, 5, spread)
    for any_hit in (False, True):
        tm = np.full(nrays, 3000.0, np.float32) if any_hit else None
        x, y = a.intersect(o, d, any_hit, tm), b.intersect(o, d, any_hit, tm)
        if any_hit:
            assert np.array_equal(x[0] != 0xFFFFFFFF, y[0] != 0xFFFFFFFF)
        else:
            assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
    stats = b.pathtracer.last_stats
    a.close()
    b.close()
    return stats


@pytest.mark.parametrize("leaf", [1, 4, 8])
def test_dem_renders_like_the_sah_build(gpu, leaf):
    st = _same([_dem()], leaf=leaf)
    assert st.bvh_nodes > 0


def test_dem_with_holes_smooth(gpu):
    _same([_dem(holes=True)], smooth=True)


def test_icosphere_and_coplanar_instances(gpu):
    dirs, faces = synthetic.icosphere(5)
    ico = Mesh(positions=(dirs * 250.0).astype(np.float32), indices=faces,
               albedo=np.full((dirs.shape[0], 4), 0.3, np.float32))
    _same([ico], cam_pos=(900.0, 300.0, 200.0), spread=300.0)
    m = _dem(posts=65)
    _same([m, m])           # two identical instances: duplicate Morton codes, equal-distance ties


def test_large_dem_rays(gpu):
    m = _dem(posts=1025, seed=7)
    a, _ = _scene([m], 0)
    b, _ = _scene([m], 1)
    a.build_tlas()
    b.build_tlas()
    o, d = _rays(200_000, 11, 400.0)
    x, y = a.intersect(o, d), b.intersect(o, d)
    assert np.array_equal(x[0], y[0]) and np.array_equal(x[1], y[1])
    assert (x[0] != 0xFFFFFFFF).mean() > 0.5
    a.close()
    b.close()


def test_refit_on_a_gpu_built_tree(gpu):
    m = _dem(posts=65)
    s, cid = _scene([m], 1)
    _render(s, cid)
    moved = m.positions.copy()
    moved[:, 2] += np.random.default_rng(2).normal(0.0, 20.0, moved.shape[0]).astype(np.float32)
    s.update_positions(0, moved)
    got = _render(s, cid)
    mm = Mesh(positions=moved, indices=m.indices, albedo=m.albedo, uv=m.uv)
    r, cr = _scene([mm], 0)
    want = _render(r, cr)
    for k in got:
        assert np.array_equal(got[k], want[k], equal_nan=True), k
    s.close()
    r.close()


def test_tiny_scene_takes_one_leaf(gpu):
    p = np.array([[0, 0, 0], [100, 0, 0], [0, 100, 0], [100, 100, 5]], np.float32)
    i = np.array([[0, 1, 2], [1, 3, 2]], np.uint32)
    _same([Mesh(positions=p, indices=i)], cam_pos=(50.0, 40.0, 300.0), nrays=512, spread=60.0)


def test_gpu_builder_arguments(gpu):
    import ctypes as C

    s, _ = _scene([_dem(posts=17)], 0)
    s.build_tlas()
    lib = capi.load()
    ctx = s.context()
    assert lib.vgb_bvh_build(ctx, C.byref(capi.BvhOptions(0, 1, 0, 8))) != 0     # binary layout only
    assert b"binary" in lib.vgb_last_error(ctx)
    assert lib.vgb_bvh_build(ctx, C.byref(capi.BvhOptions(9, 1, 0, 2))) != 0     # leaf size <= 8
    assert lib.vgb_bvh_build(ctx, C.byref(capi.BvhOptions(0, 2, 0, 2))) != 0     # unknown builder
    capi.check(lib.vgb_bvh_build(ctx, C.byref(capi.BvhOptions(2, 1, 0, 2))), ctx, "bvh_build")
    s.close()
