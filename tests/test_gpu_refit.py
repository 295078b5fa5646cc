"""Moving the vertices of an uploaded scene (vgb_scene_update_positions): the binary BVH is
refitted on the device, the 8-wide one rebuilt.

The closest hit is independent of the BVH (watertight test, (t, triangle id) tie-break) and the
occlusion test is a yes/no answer, so a correct refit renders exactly what a scene built from
scratch at the moved positions renders: every pass bit-identical, every closest-hit ray of a
batch hitting the same triangle at the same distance, every occlusion query answering the same.  A refit whose boxes missed a moved triangle
shows up as a different hit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vira_gb300 import FOUR_BAND, Mesh, Scene, capi, synthetic

pytestmark = pytest.mark.gpu


def _dem_mesh(posts=129, seed=3):
    h = synthetic.fbm_heights(posts, 0.8, seed=seed, lo=-60.0, hi=60.0)
    h = synthetic.add_crater_field(h, 2000.0 / (posts - 1), seed=seed + 1, dmin=40, dmax=400)
    m = Mesh.from_dem(h, 2000.0 / (posts - 1), albedo=1.0, nbands=4)
    m.uv = synthetic.grid_uvs(posts, posts, posts - 1)
    alb = synthetic.lognormal_albedo(64, 0.12, 0.3, seed=seed + 2)
    m.albedo_map = np.ascontiguousarray(np.repeat(alb[:, :, None], 4, axis=2))
    m.set_smooth_shading(True)
    return m


def _asteroid_mesh(subdivisions=4, seed=9):
    dirs, faces = synthetic.icosphere(subdivisions)
    relief = synthetic.real_sh_noise(dirs, 8, seed=seed)
    relief *= 20.0 / max(1e-12, float(np.sqrt(np.mean(relief * relief))))
    pos = (dirs * (250.0 + relief)[:, None]).astype(np.float32)
    m = Mesh(positions=pos, indices=faces, albedo=np.full((pos.shape[0], 4), 0.2, np.float32))
    m.set_smooth_shading(True)
    return m, dirs.astype(np.float32)


def _scene(mesh, layout=2, cam_pos=(100.0, -200.0, 2500.0), res=64):
    s = Scene(FOUR_BAND)
    s.bvh_options = capi.BvhOptions(0, 0, 0, layout)
    s.add_mesh(mesh)
    s.new_instance(("mesh", 0))
    sun = s.new_sun(5778.0)
    s.set_sun_direction(sun, 30.0, 35.0)
    cid = s.new_camera()
    c = s[cid]
    c.set_resolution(res, res)
    c.set_sensor_size(0.036)
    c.set_field_of_view(30.0)
    c.set_local_position(*cam_pos)
    c.look_at((0.0, 0.0, 0.0))
    pt = s.pathtracer
    pt.options.samples = 4
    pt.options.bounces = 2
    pt.options.seed = 5
    pt.render_passes.simulate_lighting = True
    return s, cid


def _copy(mesh, positions):
    return Mesh(positions=np.ascontiguousarray(positions, np.float32), indices=mesh.indices.copy(),
                albedo=None if mesh.albedo is None else mesh.albedo.copy(),
                uv=None if mesh.uv is None else mesh.uv.copy(),
                albedo_map=None if mesh.albedo_map is None else mesh.albedo_map.copy(),
                smooth_shading=mesh.smooth_shading)


def _passes(s, cid):
    import torch

    rp = s.pathtracer.render(s[cid], s)
    torch.cuda.synchronize()
    return {k: getattr(rp, k).cpu().numpy().copy() for k in ("total_radiance", "triangle_id", "depth", "normal_global")}


def _rays(n, seed, center, spread):
    rng = np.random.default_rng(seed)
    o = (center + rng.normal(0.0, spread, (n, 3))).astype(np.float32)
    tgt = rng.normal(0.0, 0.3 * spread, (n, 3))
    d = tgt - o
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def _assert_same(a, b, what):
    for k in a:
        nan = a[k].dtype.kind == "f"
        assert np.array_equal(a[k], b[k], equal_nan=nan), f"{what}: pass {k} differs ({np.sum(a[k] != b[k])} values)"


def _check_against_fresh(s, cid, mesh, moved, layout, cam_pos, rays):
    """Refitted scene vs a scene built from scratch at `moved`: passes and ray batches."""
    got = _passes(s, cid)
    ref_s, ref_cid = _scene(_copy(mesh, moved), layout, cam_pos)
    ref = _passes(ref_s, ref_cid)
    _assert_same(got, ref, f"layout {layout}")
    o, d = rays
    for any_hit in (False, True):
        tm = np.full(o.shape[0], 2000.0, np.float32) if any_hit else None
        a = s.intersect(o, d, any_hit, tm)
        b = ref_s.intersect(o, d, any_hit, tm)
        if any_hit:
            # which occluder an occlusion query reports depends on the traversal order: compare
            # the yes/no answer
            assert np.array_equal(a[0] != 0xFFFFFFFF, b[0] != 0xFFFFFFFF), "occlusion answers differ"
        else:
            assert np.array_equal(a[0], b[0]), "closest-hit triangle ids differ"
            hit = a[0] != 0xFFFFFFFF
            assert hit.sum() > o.shape[0] // 8, "too few rays hit the surface to test anything"
            assert np.array_equal(a[1], b[1]) and np.array_equal(a[2][hit], b[2][hit])
    ref_s.close()


@pytest.mark.parametrize("layout", [2, 8])
def test_dem_heights_moved_render_like_a_rebuild(gpu, layout):
    mesh = _dem_mesh()
    s, cid = _scene(_copy(mesh, mesh.positions), layout)
    _passes(s, cid)                       # uploaded and built at the original heights
    rng = np.random.default_rng(7)
    moved = mesh.positions.copy()
    moved[:, 2] += rng.normal(0.0, 25.0, moved.shape[0]).astype(np.float32)   # far beyond the old boxes
    s.update_positions(0, moved)
    assert not s._dirty, "the update should have been done in place"
    rays = _rays(4096, 1, np.array([0.0, 0.0, 800.0]), 600.0)
    _check_against_fresh(s, cid, mesh, moved, layout, (100.0, -200.0, 2500.0), rays)
    s.close()


def test_repeated_refits_of_an_asteroid(gpu):
    mesh, dirs = _asteroid_mesh()
    cam = (1500.0, -900.0, 700.0)
    s, cid = _scene(_copy(mesh, mesh.positions), 2, cam)
    _passes(s, cid)
    rng = np.random.default_rng(11)
    rays = _rays(4096, 2, np.array([0.0, 0.0, 0.0]), 900.0)
    for it in range(3):
        off = rng.normal(0.0, 8.0 * (it + 1), dirs.shape[0]).astype(np.float32)
        moved = (mesh.positions + off[:, None] * dirs).astype(np.float32)
        s.update_positions(0, moved)
        _check_against_fresh(s, cid, mesh, moved, 2, cam, rays)
    s.close()


def test_unchanged_positions_render_identically(gpu):
    mesh = _dem_mesh(posts=65)
    s, cid = _scene(_copy(mesh, mesh.positions), 2)
    before = _passes(s, cid)
    s.update_positions(0, mesh.positions)
    _assert_same(before, _passes(s, cid), "refit with the same positions")
    s.close()


def test_device_update_then_rebuild(gpu):
    """Positions handed over in device memory; a later vgb_bvh_build reads them back."""
    import torch

    mesh = _dem_mesh(posts=65)
    s, cid = _scene(_copy(mesh, mesh.positions), 2)
    _passes(s, cid)
    moved = mesh.positions.copy()
    moved[:, 2] *= np.float32(1.7)
    dev = torch.tensor(moved, device="cuda")
    lib = capi.load()
    ctx = s.context()
    torch.cuda.synchronize()
    capi.check(lib.vgb_scene_update_positions(ctx, capi.ptr(dev), None, 1), ctx, "scene_update_positions")
    s.meshes[0].positions = moved.copy()
    s.meshes[0].normals = None
    refit = _passes(s, cid)
    capi.check(lib.vgb_bvh_build(ctx, C.byref(s.bvh_options)), ctx, "bvh_build")
    rebuilt = _passes(s, cid)
    _assert_same(refit, rebuilt, "device update: refit vs rebuild from the read-back positions")
    ref_s, ref_cid = _scene(_copy(mesh, moved), 2)
    _assert_same(rebuilt, _passes(ref_s, ref_cid), "device update vs fresh scene")
    ref_s.close()
    s.close()


def test_update_positions_rejects_a_scene_without_mesh(gpu):
    lib = capi.load()
    h = C.c_void_p()
    capi.check(lib.vgb_context_create(C.byref(h), 0))
    p = np.zeros((3, 3), np.float32)
    assert lib.vgb_scene_update_positions(h, capi.ptr(p), None, 0) != 0
    lib.vgb_context_destroy(h)
