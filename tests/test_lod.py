"""The level-of-detail manager on the CPU (vira_gb300/lod.py, lod_manager.ipp:33-216) with a stand-in
for the Quipu reader that records which GSD each mesh asks for: visibility by normal cone and
frustum, the target GSD from Camera::calculateGSD, the keep-while-within-2x rule, the reload to
the default GSD of meshes with an invisible instance (only when another mesh needs a reload),
and the geometry helpers (oriented-box frustum test, shadow frustums)."""
from __future__ import annotations

import math

import numpy as np

from vira_gb300 import FOUR_BAND, Mesh, Scene
from vira_gb300.lod import (OBB, LevelOfDetailOptions, aabb_to_obb, calculate_gsd, camera_frustum,
                            intersects_frustum, make_shadow_frustum)


class FakeQuipu:
    """The reader interface Mesh.update_gsd and the manager use, with the readBuffers LoD rule."""

    def __init__(self, positions, indices, gsds=(1.0, 2.0, 4.0, 8.0, 16.0), default=16.0):
        self.gsds = list(gsds)
        self.default_gsd = default
        self.current_gsd = float(default)
        self.normal = np.array([0.0, 0.0, 1.0], np.float32)
        self.cone_angle = 0.2
        self.nbands = 4
        self.requests = []
        self._m = (positions, indices)

    def read_buffers(self, required_gsd=None, gpu=0, nbands=None):
        self.requests.append(required_gsd)
        lod = 0
        for i in range(1, len(self.gsds)):
            if self.gsds[i] <= required_gsd:
                lod = i
            else:
                break
        g = float(np.float32(self.gsds[lod]))
        if g == self.current_gsd:
            return None
        self.current_gsd = g
        return Mesh(self._m[0].copy(), self._m[1].copy())


def _scene(n_meshes=1):
    s = Scene(FOUR_BAND)
    h = np.zeros((33, 33), np.float32)
    for k in range(n_meshes):
        m = Mesh.from_dem(h, 10.0)
        m.quipu = FakeQuipu(m.positions, m.indices)
        s.add_mesh(m)
        inst = s.new_instance(("mesh", k))
        s[inst].position = np.array([1000.0 * k, 0.0, 0.0])
    sun = s.new_sun(5778.0)
    s.set_sun_direction(sun, 0.0, 60.0)
    cid = s.new_camera()
    c = s[cid]
    c.set_resolution(512, 512)
    c.set_sensor_size(0.036)
    c.set_field_of_view(30.0)
    return s, cid


def _place(cam, height, target=(0.0, 0.0, 0.0)):
    cam.set_local_position(0.0, -0.1 * height, height)
    cam.look_at(target)


def test_calculate_gsd():
    s, cid = _scene()
    c = s[cid]
    d = 1234.5
    want = min(d * float(c.sensor_size[0]) / (float(c.focal_length) * 512), d * float(c.sensor_size[1]) / (float(c.focal_length) * 512))
    assert calculate_gsd(c, d) == want


def test_gsd_selection_and_hysteresis():
    s, cid = _scene()
    c = s[cid]
    q = s.meshes[0].quipu
    s.lod_manager.options = LevelOfDetailOptions(target_triangle_size=2.0)

    def target(height):
        _place(c, height)
        return float(np.float32(2.0 * np.float32(calculate_gsd(c, float(np.linalg.norm(c.position))))))

    # the default LoD (16 m) is coarser than a 3 km view needs: reload to the 4 m LoD
    t = target(3000.0)
    assert 4.0 <= t < 8.0, t
    assert s.update_level_of_detail(cid) == 1 and q.requests[-1] == t and q.current_gsd == 4.0
    assert s.instances[0].visible
    # a little farther: the target grows but stays below twice the loaded GSD -> no reload
    t = target(3400.0)
    assert 4.0 < t < 8.0
    n = len(q.requests)
    assert s.update_level_of_detail(cid) == 0 and len(q.requests) == n and q.current_gsd == 4.0
    # close: finer than loaded -> the finest LoD below the target
    t = target(700.0)
    assert 1.0 <= t < 2.0
    assert s.update_level_of_detail(cid) == 1 and q.current_gsd == 1.0
    # very far: more than twice the loaded GSD -> the coarsest LoD
    t = target(20000.0)
    assert t > 16.0
    assert s.update_level_of_detail(cid) == 1 and q.current_gsd == 16.0


def test_invisible_meshes_return_to_the_default_gsd():
    s, cid = _scene(n_meshes=2)
    c = s[cid]
    q0, q1 = s.meshes[0].quipu, s.meshes[1].quipu
    for q in (q0, q1):
        q.current_gsd = 1.0
    # look at mesh 0 from close by; mesh 1 (1 km away along x) is outside the 30 degree view
    _place(c, 400.0)
    s.update_level_of_detail(cid)
    assert s.instances[0].visible and not s.instances[1].visible
    assert q1.requests and math.isinf(s.meshes[1].target_gsd) and q1.current_gsd == 16.0   # default
    assert q0.current_gsd == 1.0 or q0.requests   # mesh 0 decided by its own target
    # from below the DEMs (outside their normal cones) nothing is visible and nothing needs a
    # reload, so nothing is reloaded: the reference only calls updateMeshLoDs when a visible mesh
    # needs one.  (The box test alone would not reject a box behind the camera: with only the four
    # side planes it is conservative near the apex.)
    c.set_local_position(0.0, 0.0, -400.0)
    c.look_in_direction((0.0, 0.0, 1.0))
    n0, n1 = len(q0.requests), len(q1.requests)
    assert s.update_level_of_detail(cid) == 0
    assert not s.instances[0].visible and len(q0.requests) == n0 and len(q1.requests) == n1


def test_frustum_and_shadow_geometry():
    s, cid = _scene()
    c = s[cid]
    _place(c, 500.0)
    planes = camera_frustum(c)
    ahead = OBB(np.array([0.0, 0.0, 300.0]), np.array([5.0, 5.0, 5.0]), np.eye(3))
    aside = OBB(np.array([900.0, 0.0, 300.0]), np.array([5.0, 5.0, 5.0]), np.eye(3))
    behind = OBB(-(c.rotation.T @ np.array([0.0, 0.0, 0.0]) + np.array([0.0, 0.0, 300.0])), np.array([5.0, 5.0, 5.0]),
                 np.eye(3))
    assert intersects_frustum(ahead, planes)
    assert not intersects_frustum(aside, planes)
    assert len(planes) == 4
    # the four side planes pass through the camera centre, so a box straddling it intersects
    assert intersects_frustum(OBB(np.zeros(3), np.ones(3), np.eye(3)), planes)
    assert not intersects_frustum(behind, planes)   # small box 300 m behind: separated
    box = aabb_to_obb(np.array([-1.0, -1.0, -1.0]), np.array([1.0, 1.0, 1.0]), np.eye(3), np.array([0.0, 0.0, 50.0]), 2.0)
    assert np.allclose(box.center, [0, 0, 50]) and np.allclose(box.half, [2, 2, 2])
    fr = make_shadow_frustum(box, np.array([0.0, 0.0, 1.0e6]))
    assert 2 <= len(fr) <= 6
    corners = box.corners()
    assert len(corners) == 8 and np.allclose(np.mean(corners, axis=0), box.center)
