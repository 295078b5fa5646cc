"""The benchmark scenes, built from seeded synthetic terrain.

``plain_direct``   513^2 fBm DEM (Hurst 0.8, 10 m posts, +-200 m), albedo 0.12, sun at 30 deg
                   elevation (5778 K blackbody, 4 bands 450/550/650/850 nm), 1024^2 pinhole camera,
                   30 deg FOV, 5 km altitude, 20 deg off nadir; 1 spp, no bounces.
``path_traced``    4097^2 fBm DEM plus a Poisson crater field (20 m - 2 km, exponent -2.5), 4096^2
                   lognormal albedo texture (median 0.12, sigma_log 0.3), 8 bands 400-1000 nm,
                   2048^2 image, 3 bounces with sun NEE, 64 spp, Russian roulette after bounce 2.
Both take a ``scale`` that shrinks posts and pixels together (same footprint) for tests.
"""
from __future__ import annotations

import math

import numpy as np

from . import synthetic
from .scene import Mesh, Scene
from .spectral import EIGHT_BAND, FOUR_BAND

DEM_EXTENT_M = 5120.0        # 512 intervals of 10 m
PT_EXTENT_M = 40960.0        # 4096 intervals of 10 m


def _camera(scene: Scene, res: int, altitude: float, off_nadir_deg: float, fov_deg: float = 30.0):
    cam_id = scene.new_camera()
    cam = scene[cam_id]
    cam.set_resolution(res, res)
    cam.set_sensor_size(36.0 / 1000.0)
    cam.set_field_of_view(fov_deg)
    cam.set_local_position(0.0, 0.0, altitude)
    a = math.radians(off_nadir_deg)
    cam.look_in_direction((math.sin(a), 0.0, -math.cos(a)), up=(0.0, 0.0, 1.0))
    return cam_id


def plain_direct(posts: int = 513, resolution: int = 1024, seed: int = 1, device: int = 0,
                 deterministic: bool = True):
    posting = DEM_EXTENT_M / (posts - 1)
    h = synthetic.fbm_heights(posts, hurst=0.8, seed=seed, lo=-200.0, hi=200.0)
    scene = Scene(FOUR_BAND, device=device)
    mesh = scene.add_mesh(Mesh.from_dem(h, posting, albedo=0.12, nbands=FOUR_BAND.size))
    scene.new_instance(mesh)
    sun = scene.new_sun(temperature=5778.0)
    scene.set_sun_direction(sun, azimuth_deg=0.0, elevation_deg=30.0)
    cam_id = _camera(scene, resolution, 5000.0, 20.0)
    pt = scene.pathtracer
    pt.options.samples = 1
    pt.options.bounces = 0
    pt.options.deterministic_light = deterministic
    pt.options.seed = seed
    pt.render_passes.simulate_lighting = True
    return scene, cam_id


def path_traced(posts: int = 4097, tex: int = 4096, resolution: int = 2048, spp: int = 64, bounces: int = 3,
                rr_depth: int = 2, seed: int = 7, device: int = 0, altitude: float = 12000.0):
    posting = PT_EXTENT_M / (posts - 1)
    h = synthetic.fbm_heights(posts, hurst=0.8, seed=seed, lo=-200.0, hi=200.0)
    h = synthetic.add_crater_field(h, posting, seed=seed + 1, dmin=20.0, dmax=2000.0, exponent=-2.5)
    alb = synthetic.lognormal_albedo(tex, 0.12, 0.3, seed=seed + 2)
    B = EIGHT_BAND.size
    scene = Scene(EIGHT_BAND, device=device)
    mesh = Mesh.from_dem(h, posting, albedo=1.0, nbands=B)
    mesh.uv = synthetic.grid_uvs(posts, posts, tex)
    mesh.albedo_map = np.ascontiguousarray(np.repeat(alb[:, :, None], B, axis=2))
    mid = scene.add_mesh(mesh)
    scene.new_instance(mid)
    sun = scene.new_sun(temperature=5778.0)
    scene.set_sun_direction(sun, azimuth_deg=30.0, elevation_deg=30.0)
    cam_id = _camera(scene, resolution, altitude, 20.0)
    pt = scene.pathtracer
    pt.options.samples = spp
    pt.options.bounces = bounces
    pt.options.rr_depth = rr_depth
    pt.options.seed = seed
    pt.render_passes.simulate_lighting = True
    return scene, cam_id
