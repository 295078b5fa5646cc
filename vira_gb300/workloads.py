"""The benchmark scenes, built from seeded synthetic terrain.

``plain_direct``   513^2 fBm DEM (Hurst 0.8, 10 m posts, +-200 m), albedo 0.12, sun at 30 deg
                   elevation (5778 K blackbody, 4 bands 450/550/650/850 nm), 1024^2 pinhole camera,
                   30 deg FOV, 5 km altitude, 20 deg off nadir; 1 spp, no bounces.
``path_traced``    4097^2 fBm DEM plus a Poisson crater field (20 m - 2 km, exponent -2.5), 4096^2
                   lognormal albedo texture (median 0.12, sigma_log 0.3), 8 bands 400-1000 nm,
                   2048^2 image, 3 bounces with sun NEE, 64 spp, Russian roulette after bounce 2.
``inversion``      1025^2 crater DEM (2.1M triangles), 1024^2 lognormal albedo texture and per-vertex
                   heights as parameters; 16 views of 512^2 (30 deg FOV, 2 km altitude, sun
                   elevation 10-60 deg); 2 bounces, 16 spp, 4 bands; flat shading.
``trajectory``     256 camera poses on a seeded descent arc from 50 km to 100 m altitude over the
                   plain_direct terrain; per-frame resolution drawn from {256^2, 512^2, 1024^2,
                   2048^2} and spp from {1, 4, 16, 64}; the sun slews 0.1 deg per frame; 8 bands;
                   direct lighting.
``asteroid``       icosphere subdivision 9 (5.2M triangles) with radial spherical-harmonic relief
                   up to degree 32 (amplitude ~ l^-2, 20 m RMS, mean radius 250 m), uniform albedo
                   0.05, smooth shading; 64 views of 256^2-1024^2 at 1-3 km range under phase
                   angles 0-90 deg; 4 bands, 8 spp, direct lighting; per-vertex radial offsets are
                   the parameters (fused forward + adjoint of every view in one launch).
Each takes sizes that shrink posts, pixels or frames for tests.
"""
from __future__ import annotations

import math

import numpy as np

from . import synthetic
from .scene import BatchFrame, Camera, Mesh, Scene
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
                 deterministic: bool = True, mesher=None):
    """`mesher(heights, posting, albedo, nbands) -> Mesh` triangulates the DEM (default
    Mesh.from_dem); every other step is numpy."""
    mesher = mesher or Mesh.from_dem
    posting = DEM_EXTENT_M / (posts - 1)
    h = synthetic.fbm_heights(posts, hurst=0.8, seed=seed, lo=-200.0, hi=200.0)
    scene = Scene(FOUR_BAND, device=device)
    mesh = scene.add_mesh(mesher(h, posting, albedo=0.12, nbands=FOUR_BAND.size))
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
                rr_depth: int = 2, seed: int = 7, device: int = 0, altitude: float = 12000.0, mesher=None):
    """`mesher` as for plain_direct."""
    mesher = mesher or Mesh.from_dem
    posting = PT_EXTENT_M / (posts - 1)
    h = synthetic.fbm_heights(posts, hurst=0.8, seed=seed, lo=-200.0, hi=200.0)
    h = synthetic.add_crater_field(h, posting, seed=seed + 1, dmin=20.0, dmax=2000.0, exponent=-2.5)
    alb = synthetic.lognormal_albedo(tex, 0.12, 0.3, seed=seed + 2)
    B = EIGHT_BAND.size
    scene = Scene(EIGHT_BAND, device=device)
    mesh = mesher(h, posting, albedo=1.0, nbands=B)
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


def trajectory(nframes: int = 256, posts: int = 513, seed: int = 3, resolutions=(256, 512, 1024, 2048),
               spps=(1, 4, 16, 64), device: int = 0, alt_top: float = 50000.0, alt_bottom: float = 100.0):
    """The batched trajectory workload: returns (scene, frames)."""
    posting = DEM_EXTENT_M / (posts - 1)
    h = synthetic.fbm_heights(posts, hurst=0.8, seed=1, lo=-200.0, hi=200.0)
    scene = Scene(EIGHT_BAND, device=device)
    mid = scene.add_mesh(Mesh.from_dem(h, posting, albedo=0.12, nbands=EIGHT_BAND.size))
    scene.new_instance(mid)
    sun = scene.new_sun(temperature=5778.0)
    scene.set_sun_direction(sun, azimuth_deg=0.0, elevation_deg=30.0)
    pt = scene.pathtracer
    pt.options.bounces = 0
    pt.options.seed = seed
    pt.render_passes.simulate_lighting = True
    rng = np.random.default_rng(seed)
    frames = []
    az0 = rng.uniform(0.0, 360.0)
    for i in range(nframes):
        s = i / max(1, nframes - 1)
        alt = alt_top * (alt_bottom / alt_top) ** s                       # logarithmic descent
        rng_h = alt * 0.6 * (1.0 - s) + rng.normal(0.0, 0.01 * alt)          # ground range shrinks
        az = math.radians(az0 + 40.0 * s)
        pos = np.array([rng_h * math.cos(az), rng_h * math.sin(az), alt + 200.0])
        target = np.array([rng.normal(0.0, 100.0), rng.normal(0.0, 100.0), 0.0])
        cam = Camera()
        res = int(rng.choice(resolutions))
        cam.set_resolution(res, res)
        cam.set_sensor_size(36.0 / 1000.0)
        cam.set_field_of_view(30.0)
        cam.set_local_position(pos)
        cam.look_at(target)
        spp = int(rng.choice(spps))
        sun_az = 0.1 * i
        el = math.radians(30.0)
        d = np.array([math.cos(el) * math.cos(math.radians(sun_az)), math.cos(el) * math.sin(math.radians(sun_az)),
                      math.sin(el)])
        frames.append(BatchFrame(camera=cam, samples=spp, frame=i, light_positions=[scene.origin + 149597870700.0 * d]))
    return scene, frames


def inversion(posts: int = 1025, tex: int = 1024, resolution: int = 512, nviews: int = 16, spp: int = 16,
              bounces: int = 2, seed: int = 4, device: int = 0):
    """The adjoint inversion workload: returns (scene, views)."""
    from .autograd import View

    posting = 10.0 * 1024 / (posts - 1)
    h = synthetic.fbm_heights(posts, hurst=0.8, seed=seed, lo=-100.0, hi=100.0)
    h = synthetic.add_crater_field(h, posting, seed=seed + 1, dmin=20.0, dmax=1000.0, exponent=-2.5)
    alb = synthetic.lognormal_albedo(tex, 0.12, 0.3, seed=seed + 2)
    B = FOUR_BAND.size
    scene = Scene(FOUR_BAND, device=device)
    mesh = Mesh.from_dem(h, posting, albedo=1.0, nbands=B)
    mesh.uv = synthetic.grid_uvs(posts, posts, tex)
    mesh.albedo_map = np.ascontiguousarray(np.repeat(alb[:, :, None], B, axis=2))
    scene.add_mesh(mesh)
    scene.new_instance(("mesh", 0))
    scene.new_sun(temperature=5778.0)
    rng = np.random.default_rng(seed)
    views = []
    for v in range(nviews):
        cam = Camera()
        cam.set_resolution(resolution, resolution)
        cam.set_sensor_size(36.0 / 1000.0)
        cam.set_field_of_view(30.0)
        az = 2 * math.pi * v / nviews
        rr = rng.uniform(200.0, 800.0)
        cam.set_local_position(rr * math.cos(az), rr * math.sin(az), 2000.0)
        cam.look_at((rng.normal(0, 200.0), rng.normal(0, 200.0), 0.0))
        el = math.radians(10.0 + 50.0 * v / max(1, nviews - 1))
        saz = rng.uniform(0, 2 * math.pi)
        d = np.array([math.cos(el) * math.cos(saz), math.cos(el) * math.sin(saz), math.sin(el)])
        views.append(View(camera=cam, sun_position=scene.origin + 149597870700.0 * d, frame=v))
    pt = scene.pathtracer
    pt.options.samples = spp
    pt.options.bounces = bounces
    pt.options.seed = seed
    pt.render_passes.simulate_lighting = True
    return scene, views


def asteroid(subdivisions: int = 9, lmax: int = 32, nviews: int = 64, resolutions=(256, 512, 1024), spp: int = 8,
             bounces: int = 0, seed: int = 9, device: int = 0, radius: float = 250.0, relief_rms: float = 20.0):
    """The batched-adjoint asteroid workload: returns (scene, views, radial_dirs [nverts][3] float32).
    Vertex v sits at radial_dirs[v] * (radius + relief_v); an offset field o moves it to
    radial_dirs[v] * (radius + relief_v + o_v)."""
    from .autograd import View

    dirs, faces = synthetic.icosphere(subdivisions)
    relief = synthetic.real_sh_noise(dirs, lmax, seed=seed)
    relief *= relief_rms / max(1e-12, float(np.sqrt(np.mean(relief * relief))))
    pos = (dirs * (radius + relief)[:, None]).astype(np.float32)
    B = FOUR_BAND.size
    scene = Scene(FOUR_BAND, device=device)
    mesh = Mesh(positions=pos, indices=faces, albedo=np.full((pos.shape[0], B), 0.05, np.float32))
    mesh.set_smooth_shading(True)
    scene.add_mesh(mesh)
    scene.new_instance(("mesh", 0))
    scene.new_sun(temperature=5778.0)
    rng = np.random.default_rng(seed + 1)
    views = []
    for v in range(nviews):
        res = int(rng.choice(resolutions))
        cam = Camera()
        cam.set_resolution(res, res)
        cam.set_sensor_size(36.0 / 1000.0)
        cam.set_field_of_view(30.0)
        d = rng.standard_normal(3)
        d /= np.linalg.norm(d)
        rr = rng.uniform(1000.0, 3000.0)
        cam.set_local_position(*(rr * d))
        cam.look_at((0.0, 0.0, 0.0))
        # sun direction at phase angle alpha from the view direction (seen from the body)
        alpha = math.radians(rng.uniform(0.0, 90.0))
        a = rng.standard_normal(3)
        a -= d * float(a @ d)
        a /= np.linalg.norm(a)
        s_dir = math.cos(alpha) * d + math.sin(alpha) * a
        views.append(View(camera=cam, sun_position=scene.origin + 149597870700.0 * s_dir, frame=v, samples=spp))
    pt = scene.pathtracer
    pt.options.samples = spp
    pt.options.bounces = bounces
    pt.options.seed = seed
    pt.render_passes.simulate_lighting = True
    return scene, views, dirs.astype(np.float32)
