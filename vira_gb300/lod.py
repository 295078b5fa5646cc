"""Level-of-detail selection for meshes backed by DEM Quipu pyramids.

``LevelOfDetailManager.update(camera, scene)`` restates vira::scene::LevelOfDetailManager::
updateByMapping (include/implementation/scene/lod_manager.ipp:33-216) on the host: per instance a
normal-cone test against the view direction, an oriented-box test against the camera's four side
planes, and (with check_shadows) the shadow frustums of the visible boxes for instances that may
cast a shadow into view; per mesh the target GSD target_triangle_size x Camera::calculateGSD of
the nearest visible instance, with the reference's hysteresis (a finer mesh is kept while its
GSD is more than half the target); then Scene::updateMeshLoDs / Mesh::updateGSD
(scene.ipp:615-665, mesh.ipp:86-113), whose LoD reads run through DEMQuipu.read_buffers -- LZ4
decode on the host, mesh build on the GPU.

The decisions follow the reference line by line, including its quirks: the shadow test compares
an angle in radians with 90, so any lit instance counts as a possible shadow caster; the box
centre is scaled but not rotated into the camera frame (AABB::toOBB, aabb.ipp:131-141); shadow
frustums mix the camera-frame box with the light's scene-frame position; and an invisible
instance sends its mesh back to the default GSD.  Arithmetic is FP64 (the reference's TFloat
geometry in FP32 can differ on borderline cases only).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np


@dataclass
class LevelOfDetailOptions:
    """LevelOfDetailOptions (lod_manager.hpp:14-23)."""

    target_triangle_size: float = 2.0
    cone_angle: float = 0.0          # degrees; 0 = the mesh's own normal cone
    max_view_angle: float = 90.0     # degrees
    check_shadows: bool = True
    parallel_update: bool = True


def _normalize(v):
    with np.errstate(invalid="ignore", divide="ignore"):   # a zero vector gives NaN, as glm's does
        return v / np.linalg.norm(v)


class Plane:
    """rendering::Plane (frustum.ipp:10-26): normal n and distance d = dot(n, p1); a point is
    inside when dot(n, p) + d <= 0."""

    def __init__(self, normal, distance):
        self.normal = np.asarray(normal, np.float64)
        self.distance = float(distance)

    @staticmethod
    def through(p1, p2, p3) -> "Plane":
        n = _normalize(np.cross(p2 - p1, p3 - p1))
        return Plane(n, float(n @ p1))


class OBB:
    """rendering::OBB: centre, half sizes and axes (columns)."""

    def __init__(self, center, half, axes):
        self.center = np.asarray(center, np.float64)
        self.half = np.asarray(half, np.float64)
        self.axes = np.asarray(axes, np.float64)   # axes[:, j] is axis j

    def corners(self):
        """OBB::getCorners (obb.ipp:26-39): corner i takes +half along axis j when bit j of i is set."""
        out = []
        for i in range(8):
            c = self.center.copy()
            for j in range(3):
                sign = 1.0 if (i & (1 << j)) else -1.0
                c = c + sign * self.half[j] * self.axes[:, j]
            out.append(c)
        return out

    EDGES = ((0, 1), (1, 3), (3, 2), (2, 0), (4, 5), (5, 7), (7, 6), (6, 4), (0, 4), (1, 5), (2, 6), (3, 7))


def aabb_to_obb(lo, hi, rotation, position, scale) -> OBB:
    """AABB::toOBB (aabb.ipp:131-141) for a transformation split into position, rotation and scale:
    the centre is position + scale * (box centre) -- scaled, not rotated, as in the reference."""
    center = (np.asarray(lo, np.float64) + np.asarray(hi, np.float64)) / 2.0
    extent = np.asarray(hi, np.float64) - np.asarray(lo, np.float64)
    return OBB(position + scale * center, scale * (extent / 2.0), rotation)


def intersects_frustum(obb: OBB, planes) -> bool:
    """intersectsFrustum(OBB) (frustum.ipp:55-80)."""
    for p in planes:
        radius = sum(abs(obb.half[i] * float(p.normal @ obb.axes[:, i])) for i in range(3))
        if float(p.normal @ obb.center) + p.distance > radius:
            return False
    return True


def make_shadow_frustum(obb: OBB, light_position) -> list:
    """makeShadowFrustum (frustum.ipp:82-160): near and far planes along the light direction and up
    to four side planes through the light and the box's silhouette edges."""
    lp = np.asarray(light_position, np.float64)
    corners = obb.corners()
    dists = [float(np.linalg.norm(c - lp)) for c in corners]
    furthest = 0
    for i in range(1, 8):
        if dists[i] > dists[furthest]:
            furthest = i
    light_dir = _normalize(obb.center - lp)
    planes = [Plane(-light_dir, float(-light_dir @ corners[furthest])), Plane(light_dir, float(light_dir @ lp))]
    for a, b in OBB.EDGES:
        v1, v2 = corners[a], corners[b]
        to_v1 = _normalize(v1 - lp)
        n = _normalize(np.cross(v2 - v1, to_v1))
        side, established, silhouette = 0.0, False, True
        for j in range(8):
            if j in (a, b):
                continue
            d = float(n @ (corners[j] - v1))
            if not established:
                side, established = d, True
            elif math.copysign(1.0, d) != math.copysign(1.0, side):
                silhouette = False
                break
        if silhouette and len(planes) < 6:
            planes.append(Plane(n, float(n @ v1)))
    return planes


def camera_frustum(camera) -> list:
    """Camera::precomputeFrustum (camera.ipp:1710-1729): the four side planes through the corner
    pixels' directions, in the camera frame."""
    W, H = camera.resolution
    kinv = camera.kinv().astype(np.float64)
    zd = float(camera.z_dir)

    def direction(x, y):
        u = kinv[0] * x + kinv[2] * y + kinv[4]
        v = kinv[1] * x + kinv[3] * y + kinv[5]
        return _normalize(np.array([u, zd * v, zd]))

    c = [direction(0, 0), direction(W - 1, 0), direction(W - 1, H - 1), direction(0, H - 1)]
    c += [10.0 * x for x in c]
    return [Plane.through(c[0], c[4], c[3]), Plane.through(c[1], c[2], c[5]),
            Plane.through(c[0], c[1], c[4]), Plane.through(c[3], c[7], c[2])]


def calculate_gsd(camera, distance: float) -> float:
    """Camera::calculateGSD (camera.ipp:1408-1414)."""
    W, H = camera.resolution
    gx = distance * float(camera.sensor_size[0]) / (float(camera.focal_length) * W)
    gy = distance * float(camera.sensor_size[1]) / (float(camera.focal_length) * H)
    return min(gx, gy)


class LevelOfDetailManager:
    """vira::scene::LevelOfDetailManager (lod_manager.hpp:25-41)."""

    def __init__(self, options: LevelOfDetailOptions | None = None):
        self.options = options or LevelOfDetailOptions()
        self.last_updates = 0

    def update(self, camera, scene, gpu: int | None = None) -> int:
        """Sets every instance's visibility and every mesh's target GSD, then reloads the meshes
        whose LoD changes.  Returns the number of meshes reloaded."""
        opt = self.options
        Rc = np.asarray(camera.rotation, np.float64)
        Oc = np.asarray(camera.position, np.float64) - scene.origin
        planes = camera_frustum(camera)
        max_view = math.radians(opt.max_view_angle)
        lights = [np.asarray(L.position, np.float64) - scene.origin for L in scene.lights]
        inst_of = {}
        for k, inst in enumerate(scene.instances):
            inst_of.setdefault(inst.mesh, []).append(k)
        vis = [False] * len(scene.instances)
        casting = [False] * len(scene.instances)
        boxes = [None] * len(scene.instances)
        shadow_frustums = []

        def camera_obb(mesh, inst):
            lo, hi = mesh.aabb()
            R = Rc.T @ np.asarray(inst.rotation, np.float64)
            pos = Rc.T @ (np.asarray(inst.position, np.float64) - scene.origin - Oc)
            return aabb_to_obb(lo, hi, R, pos, float(inst.scale))

        # direct visibility (lod_manager.ipp:56-119)
        for m_i, mesh in enumerate(scene.meshes):
            cone = math.radians(opt.cone_angle)
            if cone == 0:
                cone = mesh.cone_angle()
            n_local = mesh.normal()
            for k in inst_of.get(m_i, []):
                inst = scene.instances[k]
                ipos = np.asarray(inst.position, np.float64) - scene.origin
                v = _normalize(Oc - ipos)
                n = np.asarray(inst.rotation, np.float64) @ n_local
                if opt.check_shadows:
                    for lp in lights:
                        lv = _normalize(ipos - lp)
                        if math.acos(max(-1.0, min(1.0, float(lv @ n)))) - cone < 90:   # radians against 90
                            casting[k] = True
                            break
                if math.acos(max(-1.0, min(1.0, float(v @ n)))) - cone >= max_view:
                    continue
                obb = camera_obb(mesh, inst)
                boxes[k] = obb
                if not intersects_frustum(obb, planes):
                    continue
                vis[k] = True
                if opt.check_shadows:
                    for lp in lights:
                        shadow_frustums.append(make_shadow_frustum(obb, lp))
        # shadow visibility (lod_manager.ipp:121-147)
        if opt.check_shadows:
            for m_i, mesh in enumerate(scene.meshes):
                for k in inst_of.get(m_i, []):
                    if vis[k] or not casting[k]:
                        continue
                    obb = boxes[k] or camera_obb(mesh, scene.instances[k])
                    if any(intersects_frustum(obb, fr) for fr in shadow_frustums):
                        vis[k] = True
        # target GSDs (lod_manager.ipp:149-196)
        to_update = 0
        for m_i, mesh in enumerate(scene.meshes):
            dist = math.inf
            for k in inst_of.get(m_i, []):
                if vis[k]:
                    d = float(np.linalg.norm(Oc - (np.asarray(scene.instances[k].position, np.float64) - scene.origin)))
                    dist = min(dist, d)
            if math.isinf(dist):
                continue
            mesh.target_gsd = float(np.float32(opt.target_triangle_size * np.float32(calculate_gsd(camera, dist))))
            cur = mesh.gsd()
            if cur > mesh.target_gsd:
                to_update += 1
                continue
            if cur < mesh.target_gsd:
                if cur * 2.0 > mesh.target_gsd:
                    mesh.target_gsd = cur
                else:
                    to_update += 1
        # meshes with an invisible instance go back to their default GSD (lod_manager.ipp:198-205)
        for m_i, mesh in enumerate(scene.meshes):
            if any(not vis[k] for k in inst_of.get(m_i, [])):
                mesh.target_gsd = math.inf
        for k, inst in enumerate(scene.instances):
            inst.visible = vis[k]
        scene.mark_dirty()
        # Scene::updateMeshLoDs (scene.ipp:615-665)
        updated = 0
        if to_update:
            for mesh in scene.meshes:
                if mesh.update_gsd(mesh.target_gsd, gpu=scene.device if gpu is None else gpu):
                    updated += 1
        self.last_updates = updated
        return updated
