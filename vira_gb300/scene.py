"""Host side of the hot path, mirroring Vira's scene / camera / path-tracer API.

Names follow the reference (``Scene.new_camera``, ``scene[cam].set_resolution``,
``scene.pathtracer.options.samples``, ``scene.pathtracer.render_passes.simulate_lighting``,
``scene.pathtrace_render(cam)``), as its Python example uses them
(examples/virapy_examples/pyvira_orex.py:52-110).  Poses, the sun ephemeris and the rebasing of
everything into a local scene frame are FP64 on the host; the device sees FP32 in that frame.
Rendering goes through the C ABI of include/vgb.h (libvgb.so); film planes are torch CUDA
tensors (PyTorch provides device memory only).
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .spectral import AU_TO_M, SOLAR_RADIUS, SpectralBands, black_body_radiance

PI_F = np.float32(3.14159265358979323846)


# ============================================================================ camera
class Camera:
    """Pinhole camera: Camera (include/vira/cameras/camera.hpp); `sensor` holds the sensor chain.

    Defaults follow camera.hpp:220-235: focal length 50 mm, sensor 36 x 20.25 mm,
    resolution 1920 x 1080, f-stop 2.8, optical efficiency 1, principal point at the centre.
    """

    def __init__(self):
        self.focal_length = np.float32(50.0 / 1000.0)
        self.resolution = (1920, 1080)
        self.sensor_size = (np.float32(36.0 / 1000.0), np.float32(20.25 / 1000.0))
        self.square_pixel = True
        self.f_stop = np.float32(2.8)
        self.aperture_diameter = np.float32(self.focal_length / self.f_stop)
        self.optical_efficiency = 1.0
        self.principal_point = (np.float32(np.inf), np.float32(np.inf))
        self.skew = (np.float32(0.0), np.float32(0.0))
        self.blender_frame = False
        self.position = np.zeros(3, np.float64)          # FP64, scene (global) frame
        self.rotation = np.eye(3, dtype=np.float64)       # FP64, columns = camera axes
        self._kinv = None
        # lens distortion: (capi distortion model, FP32 coefficients) or None; with interpolation
        # (the reference's default) ray directions come from the table of integer-pixel directions
        self.distortion = None
        self.interpolate_distortion_directions = True
        # depth of field (off by default, as in the reference); +inf focus keeps pinhole directions
        self.depth_of_field = False
        self.focus_distance = np.float32(np.inf)
        # motion (global frame) for the velocity pass
        self.velocity = np.zeros(3, np.float64)
        self.angular_rate = np.zeros(3, np.float64)
        # the sensor chain after the film (exposure, photosite, noise model, PSF, filter mosaic)
        from .sensor import SensorModel

        self.sensor = SensorModel()
        self._psf_kernel = None

    def psf_kernel(self, bands):
        """The PSF kernel the render convolves with (built once per PSF, size and bands)."""
        key = (id(self.sensor.psf), self.sensor.psf_kernel_size, bands.size)
        if self._psf_kernel is None or self._psf_kernel[0] != key:
            self._psf_kernel = (key, self.sensor.psf.make_kernel(bands, self.sensor.psf_kernel_size, 20))
        return self._psf_kernel[1]

    # --- setters (camera.ipp:235-470)
    def set_focal_length(self, f: float):
        if not f > 0:
            raise ValueError("Focal Length must be positive")
        self.focal_length = np.float32(f)
        self.f_stop = np.float32(np.float32(f) / self.aperture_diameter)

    def set_f_stop(self, f_stop: float):
        if not f_stop > 0:
            raise ValueError("F-Stop must be positive")
        self.f_stop = np.float32(f_stop)
        self.aperture_diameter = np.float32(self.focal_length / self.f_stop)

    def set_resolution(self, x: int, y: int):
        self.resolution = (int(x), int(y))
        if self.square_pixel:
            self.set_sensor_size(float(self.sensor_size[0]))

    def set_sensor_size(self, x: float, y: float | None = None):
        if y is None:
            yy = float(self.resolution[1]) * (float(x) / float(self.resolution[0]))
            self.sensor_size = (np.float32(x), np.float32(yy))
            self.square_pixel = True
        else:
            self.sensor_size = (np.float32(x), np.float32(y))
            self.square_pixel = False

    def set_field_of_view(self, fov_deg: float):
        """Focal length giving the horizontal field of view for the current sensor width."""
        self.set_focal_length(float(self.sensor_size[0]) / 2.0 / math.tan(math.radians(fov_deg) / 2.0))

    # --- lens distortion and depth of field (camera.ipp:183-206, 420-428, 795-840)
    def set_brown_distortion_coefficients(self, k1=0.0, k2=0.0, k3=0.0, p1=0.0, p2=0.0):
        self.distortion = (capi.DISTORTION_BROWN, np.array([k1, k2, k3, p1, p2], np.float32))

    def set_opencv_distortion_coefficients(self, k1=0.0, k2=0.0, k3=0.0, k4=0.0, k5=0.0, k6=0.0, p1=0.0, p2=0.0,
                                           s1=0.0, s2=0.0, s3=0.0, s4=0.0):
        self.distortion = (capi.DISTORTION_OPENCV,
                           np.array([k1, k2, k3, k4, k5, k6, p1, p2, s1, s2, s3, s4], np.float32))

    def set_owen_distortion_coefficients(self, e1=0.0, e2=0.0, e3=0.0, e4=0.0, e5=0.0, e6=0.0):
        self.distortion = (capi.DISTORTION_OWEN, np.array([e1, e2, e3, e4, e5, e6], np.float32))

    def clear_distortion(self):
        self.distortion = None

    def has_distortion(self) -> bool:
        return self.distortion is not None

    def enable_distortion_interpolation(self, interpolation: bool = True):
        self.interpolate_distortion_directions = bool(interpolation)

    def enable_depth_of_field(self, depth_of_field: bool = True):
        self.depth_of_field = bool(depth_of_field)

    def set_focus_distance(self, focus_distance: float):
        if math.isnan(focus_distance):
            raise ValueError("Focus Distance must not be NaN")
        self.focus_distance = np.float32(focus_distance)

    def aperture_radius(self) -> np.float32:
        """CircularAperture radius after Camera::initialize: (focal_length / f_stop) / 2 in FP32."""
        return np.float32(np.float32(self.focal_length / self.f_stop) / np.float32(2.0))

    def set_optical_efficiency(self, eff):
        self.optical_efficiency = eff

    def enable_blender_frame(self):
        self.blender_frame = True

    def set_local_position(self, x, y=None, z=None):
        self.position = np.array([x, y, z] if y is not None else x, np.float64).reshape(3)

    def set_local_rotation(self, matrix):
        self.rotation = np.array(matrix, np.float64).reshape(3, 3)

    def look_at(self, target, up=(0.0, 0.0, 1.0)):
        self.look_in_direction(np.asarray(target, np.float64) - self.position, up)

    def look_in_direction(self, direction, up=(0.0, 0.0, 1.0)):
        """Camera::lookInDirection (camera.ipp:1455-1500), evaluated in FP64."""
        up = np.asarray(up, np.float64)
        up = up / np.linalg.norm(up)
        d = np.asarray(direction, np.float64)
        d = d / np.linalg.norm(d)
        if abs(float(d @ up)) > 0.999:
            for cand in ((0.0, 1.0, 0.0), (0.0, 0.0, 1.0), (1.0, 0.0, 0.0)):
                if abs(float(d @ np.array(cand))) < 0.999:
                    up = np.array(cand)
                    break
        if self.blender_frame:
            y_axis, z_axis = up, -d
        else:
            y_axis, z_axis = -up, d
        x_axis = np.cross(y_axis, z_axis)
        x_axis /= np.linalg.norm(x_axis)
        y_axis = np.cross(z_axis, x_axis)
        y_axis /= np.linalg.norm(y_axis)
        self.rotation = np.stack([x_axis, y_axis, z_axis / np.linalg.norm(z_axis)], axis=1)

    # --- derived constants
    @property
    def z_dir(self) -> np.float32:
        return np.float32(-1.0 if self.blender_frame else 1.0)

    @property
    def intrinsics_z_dir(self) -> np.float32:
        """The z_dir the intrinsic matrices are built with: Camera::initialize computes them before
        it switches z_dir to -1 for the Blender frame (camera.ipp:131-138), so a camera initialized
        once carries +1 in K and K^-1 and -1 only in its ray directions, behind test and mirror."""
        return np.float32(1.0)

    def kinv(self) -> np.ndarray:
        """Inverse intrinsic matrix, FP32, through the C ABI (camera.ipp:1526-1568)."""
        lib = capi.load()
        out = (C.c_float * 6)()
        W, H = self.resolution
        capi.check(lib.vgb_camera_intrinsics(self.focal_length, self.sensor_size[0], self.sensor_size[1], W, H,
                                             self.principal_point[0], self.principal_point[1], self.skew[0],
                                             self.skew[1], self.intrinsics_z_dir, out), what="camera_intrinsics")
        return np.array(out[:], np.float32)

    def intrinsic_matrix(self) -> np.ndarray:
        """The rows of K, FP32 (camera.ipp:1526-1556): fx, kxy, px, kyx, fy, py with z_dir folded in."""
        f32 = np.float32
        W, H = self.resolution
        kx = f32(f32(W) / f32(self.sensor_size[0]))
        ky0 = f32(f32(H) / f32(self.sensor_size[1]))
        px = f32(f32(W) / f32(2)) if np.isinf(self.principal_point[0]) else f32(self.principal_point[0])
        py = f32(f32(H) / f32(2)) if np.isinf(self.principal_point[1]) else f32(self.principal_point[1])
        zd = self.intrinsics_z_dir
        ky = f32(zd * ky0)
        fx = f32(f32(self.focal_length) * kx)
        fy = f32(f32(self.focal_length) * ky)
        return np.array([fx, f32(zd * f32(self.skew[0])), f32(zd * px), f32(zd * f32(self.skew[1])), fy,
                         f32(zd * py)], np.float32)

    def aperture_area(self) -> np.float32:
        """CircularAperture::getArea after Camera::initialize (aperture.ipp:25-31)."""
        d = np.float32(self.focal_length / self.f_stop)
        r = np.float32(d / np.float32(2.0))
        return np.float32(np.float32(PI_F * r) * r)

    def to_c(self, scene_origin: np.ndarray, nbands: int, kinv=None) -> capi.Camera:
        """The C-ABI camera: FP64 pose rebased on `scene_origin`, then FP32.  `kinv`: the six
        FP32 entries of K^-1 when the caller has them (default: vgb_camera_intrinsics)."""
        c = capi.Camera()
        c.width, c.height = self.resolution
        o = (self.position - scene_origin).astype(np.float32)    # FP64 rebasing, then FP32
        for k in range(3):
            c.origin[k] = float(o[k])
        R = self.rotation.astype(np.float32)
        for col in range(3):
            for row in range(3):
                c.rotation[3 * col + row] = float(R[row, col])
        kinv = self.kinv() if kinv is None else np.asarray(kinv, np.float32)
        for k in range(6):
            c.kinv[k] = float(kinv[k])
        c.z_dir = float(self.z_dir)
        eff = np.broadcast_to(np.asarray(self.optical_efficiency, np.float32), (nbands,))
        area = self.aperture_area()
        for k in range(nbands):
            c.power_scale[k] = float(np.float32(eff[k] * area))
        if self.distortion is not None:
            c.distortion = int(self.distortion[0])
            for k, v in enumerate(self.distortion[1]):
                c.distortion_coeffs[k] = float(v)
        c.interpolate_directions = int(bool(self.interpolate_distortion_directions))
        c.depth_of_field = int(bool(self.depth_of_field))
        c.aperture_radius = float(self.aperture_radius())
        c.focal_length = float(self.focal_length)
        c.focus_distance = float(self.focus_distance)
        c.sensor_size[0], c.sensor_size[1] = float(self.sensor_size[0]), float(self.sensor_size[1])
        ro = (self.rotation @ np.asarray(scene_origin, np.float64)).astype(np.float32)
        for k in range(3):
            c.velocity[k] = float(np.float32(self.velocity[k]))
            c.angular_rate[k] = float(np.float32(self.angular_rate[k]))
            c.rot_origin[k] = float(ro[k])
        return c


# ============================================================================ assets
@dataclass
class Mesh:
    """Mesh (include/vira/geometry/mesh.hpp): FP32 vertices in the mesh frame."""

    positions: np.ndarray                  # (n, 3) float32
    indices: np.ndarray                    # (t, 3) uint32
    albedo: np.ndarray | None = None       # (n, B) float32 per-vertex albedo (Vertex::albedo)
    uv: np.ndarray | None = None           # (n, 2) float32
    normals: np.ndarray | None = None      # (n, 3) float32; computed by Mesh::init when absent
    albedo_map: np.ndarray | None = None   # (h, w, B) float32 material albedo texture
    normal_map: np.ndarray | None = None   # (h, w, 3) float32 tangent-space normals (Material::setNormalMap)
    smooth_shading: bool = False
    quipu: object = None                   # DEMQuipu the mesh's LoDs come from (Mesh::hasQuipu_)
    target_gsd: float = math.inf           # set by the level-of-detail manager

    # --- level of detail (mesh.ipp:86-113 and the queries lod_manager.ipp reads)
    @staticmethod
    def from_quipu(path, nbands: int = 1, options=None, required_gsd: float | None = None,
                   gpu: int = 0) -> "Mesh":
        """A mesh whose vertices come from a DEM Quipu file: the LoD for `required_gsd` (the
        reader's default GSD when None), read into a mesh on GPU `gpu`."""
        from .quipu import DEMQuipu

        q = DEMQuipu(path, options, nbands=nbands)
        m = q.read_buffers(required_gsd, gpu=gpu, nbands=nbands)
        m.quipu = q
        return m

    def gsd(self) -> float:
        """Mesh::getGSD: the GSD of the loaded LoD (0 without a Quipu)."""
        return float(self.quipu.current_gsd) if self.quipu is not None else 0.0

    def normal(self) -> np.ndarray:
        """Mesh::getNormal: the Quipu's normal cone axis (+z without one)."""
        if self.quipu is not None:
            return np.asarray(self.quipu.normal, np.float64)
        return np.array([0.0, 0.0, 1.0])

    def cone_angle(self) -> float:
        return float(self.quipu.cone_angle) if self.quipu is not None else math.pi

    def aabb(self):
        """Mesh::getAABB over the finite vertices."""
        p = self.positions[np.isfinite(self.positions).all(axis=1)]
        return p.min(axis=0).astype(np.float64), p.max(axis=0).astype(np.float64)

    def update_gsd(self, target_gsd: float, gpu: int = 0) -> bool:
        """Mesh::updateGSD: reloads the vertices from the Quipu LoD for the target GSD (the default
        GSD for +inf).  Returns whether the mesh changed."""
        q = self.quipu
        if q is None:
            return False
        t = q.default_gsd if math.isinf(target_gsd) else target_gsd
        if t == q.current_gsd:
            return False
        m = q.read_buffers(t, gpu=gpu, nbands=q.nbands)
        if m is None:
            return False
        self.positions, self.indices, self.albedo, self.normals = m.positions, m.indices, m.albedo, m.normals
        self.uv = None
        return True

    def set_smooth_shading(self, on: bool):
        self.smooth_shading = bool(on)

    def compute_normals(self, gpu: int | None = None) -> np.ndarray:
        """Mesh::calculateNormals (mesh.ipp:199-233); with `gpu` by vgb_compute_vertex_normals_gpu,
        which gives the same normals."""
        if self.normals is None:
            lib = capi.load()
            p = np.ascontiguousarray(self.positions, np.float32)
            i = np.ascontiguousarray(self.indices, np.uint32)
            n = np.empty_like(p)
            if gpu is None:
                capi.check(lib.vgb_compute_vertex_normals(capi.ptr(p), p.shape[0], capi.ptr(i), i.shape[0], capi.ptr(n)),
                           what="compute_vertex_normals")
            else:
                ctx = _mesh_context(gpu)
                capi.check(lib.vgb_compute_vertex_normals_gpu(ctx, capi.ptr(p), p.shape[0], capi.ptr(i), i.shape[0],
                                                              capi.ptr(n), 0), ctx, "compute_vertex_normals_gpu")
            self.normals = n
        return self.normals

    @staticmethod
    def from_dem(heights: np.ndarray, posting: float, albedo=None, nbands: int = 1, gpu: int | None = None) -> "Mesh":
        """DEM::makeMesh with the non-OGR projection (dem.ipp:138-211).  With `gpu` (a device index)
        the grid is triangulated by vgb_dem_triangulate_gpu, which gives the same arrays."""
        lib = capi.load()
        h = np.ascontiguousarray(heights, np.float32)
        H, W = h.shape
        pos = np.empty((H * W, 3), np.float32)
        idx = np.empty((2 * (W - 1) * (H - 1), 3), np.uint32)
        nt = C.c_uint32(0)
        if gpu is None:
            capi.check(lib.vgb_dem_triangulate(capi.ptr(h), W, H, float(posting), float(posting), capi.ptr(pos),
                                               capi.ptr(idx), C.byref(nt)), what="dem_triangulate")
        else:
            ctx = _mesh_context(gpu)
            capi.check(lib.vgb_dem_triangulate_gpu(ctx, capi.ptr(h), W, H, float(posting), float(posting), capi.ptr(pos),
                                                   capi.ptr(idx), C.byref(nt), 0), ctx, "dem_triangulate_gpu")
        alb = None
        if albedo is not None:
            a = np.asarray(albedo, np.float32)
            if a.ndim == 0 or a.size == nbands:
                alb = np.broadcast_to(a.reshape(1, -1) if a.ndim else a, (H * W, nbands)).astype(np.float32)
            else:
                alb = a.reshape(H * W, -1).astype(np.float32)
        return Mesh(pos, idx[: nt.value].copy(), albedo=alb)


_MESH_CONTEXTS: dict = {}


def _mesh_context(device: int):
    """A context per device for the mesh helpers (triangulation, normals)."""
    if device not in _MESH_CONTEXTS:
        lib = capi.load()
        h = C.c_void_p()
        capi.check(lib.vgb_context_create(C.byref(h), int(device)), what="context_create (is a GPU present?)")
        _MESH_CONTEXTS[device] = h
    return _MESH_CONTEXTS[device]


@dataclass
class Instance:
    mesh: int
    position: np.ndarray = field(default_factory=lambda: np.zeros(3))   # FP64
    rotation: np.ndarray = field(default_factory=lambda: np.eye(3))     # FP64
    scale: float = 1.0
    visible: bool = True
    velocity: np.ndarray = field(default_factory=lambda: np.zeros(3))      # global frame, m/s
    angular_rate: np.ndarray = field(default_factory=lambda: np.zeros(3))  # global frame, rad/s

    def set_local_position(self, x, y=None, z=None):
        self.position = np.array([x, y, z] if y is not None else x, np.float64).reshape(3)

    def set_local_rotation(self, matrix):
        self.rotation = np.array(matrix, np.float64).reshape(3, 3)

    def set_velocity(self, v):
        self.velocity = np.array(v, np.float64).reshape(3)

    def set_angular_rate(self, w):
        self.angular_rate = np.array(w, np.float64).reshape(3)


@dataclass
class SphereLight:
    """SphereLight (include/implementation/lights/sphere_light.ipp:17-28)."""

    radiance: np.ndarray        # FP32 per band
    radius: np.float32
    position: np.ndarray = field(default_factory=lambda: np.zeros(3))   # FP64

    def set_local_position(self, x, y=None, z=None):
        self.position = np.array([x, y, z] if y is not None else x, np.float64).reshape(3)


# ============================================================================ path tracer
@dataclass
class EATWTOptions:
    """EATWTOptions (include/vira/rendering/cpu_denoise.hpp:10-19)."""

    max_levels_direct: int = 5
    max_levels_indirect: int = 5
    depth_threshold: float = 0.2
    normal_threshold: float = 0.5
    min_normal_weight: float = 0.3
    epsilon: float = 1e-6

    def to_c(self) -> capi.DenoiseOptions:
        return capi.DenoiseOptions(int(self.max_levels_direct), int(self.max_levels_indirect),
                                   float(self.depth_threshold), float(self.normal_threshold),
                                   float(self.min_normal_weight), float(self.epsilon))


@dataclass
class PathTracerOptions:
    """CPUPathTracerOptions (include/vira/rendering/cpu_path_tracer.hpp:30-43) plus the
    counter-based RNG key and the two additions (deterministic light sampling, Russian roulette)."""

    samples: int = 1
    bounces: int = 0
    show_background: bool = False
    denoise: bool = False
    seed: int = 0
    frame: int = 0
    deterministic_light: bool = False
    rr_depth: int = 0
    adaptive_sampling: bool = False
    samples_per_batch: int = 30
    sampling_tolerance: float = 0.05
    samples_to_detect_miss: int = 30


@dataclass
class RenderPasses:
    """RenderPasses (include/vira/rendering/passes.hpp:51-95): planes are torch CUDA tensors
    [B][H][W] / [3][H][W] / [H][W] after a render."""

    simulate_lighting: bool = False
    depth: object = None
    alpha: object = None
    albedo: object = None
    normal_global: object = None
    triangle_id: object = None
    received_power: object = None
    total_radiance: object = None
    direct_radiance: object = None
    indirect_radiance: object = None
    # first-hit ids (passes.ipp:96-101; -1 where nothing was hit): the instance, its mesh and the
    # material (0: the default material, the only one this path shades with); normal_camera is
    # the normal in the camera frame, which only the rasterizer fills (zeros from the path tracer,
    # as the reference's)
    instance_id: object = None
    mesh_id: object = None
    material_id: object = None
    normal_camera: object = None
    # first-hit passes (passes.hpp:79-85), filled by the path tracer when requested
    save_velocity: bool = False
    velocity_global: object = None
    velocity_camera: object = None
    save_triangle_size: bool = False
    triangle_size: object = None


def _id_passes(rp: "RenderPasses", scene: "Scene", camera: "Camera", first: int, raster: bool):
    """Turns the device's triangle ids (index in the flattened scene, + `first`) into the reference's
    per-instance ids and derives instance_id, mesh_id, material_id and normal_camera."""
    import torch

    dev = rp.triangle_id.device
    tid = rp.triangle_id.to(torch.int64)
    hit = tid != -1
    fi = (tid - first).clamp(min=0)
    offs = scene.flat["tri_offsets"]
    counts = [n for (_, _, n) in offs]
    starts = torch.tensor(np.cumsum([0] + counts[:-1]), dtype=torch.int64, device=dev)
    k = (torch.searchsorted(starts, fi, right=True) - 1).clamp(min=0)
    inst = torch.tensor([ii for (ii, _, _) in offs], dtype=torch.int64, device=dev)
    mesh = torch.tensor([scene.instances[ii].mesh for (ii, _, _) in offs], dtype=torch.int64, device=dev)
    none = torch.full_like(tid, -1)
    rp.triangle_id = torch.where(hit, fi - starts[k] + first, none).to(torch.int32)
    rp.instance_id = torch.where(hit, inst[k], none).to(torch.int32)
    rp.mesh_id = torch.where(hit, mesh[k], none).to(torch.int32)
    rp.material_id = torch.where(hit, torch.zeros_like(tid), none).to(torch.int32)
    n = rp.normal_global
    if raster:
        # Camera::getViewNormalMatrix (the inverse rotation) times the normal, glm's row sums
        R = np.asarray(camera.rotation, np.float64).astype(np.float32)
        rows = []
        for r in range(3):
            a, b, c = (float(R[0, r]), float(R[1, r]), float(R[2, r]))
            rows.append((n[0] * a + n[1] * b) + n[2] * c)
        rp.normal_camera = torch.stack(rows)
    else:
        rp.normal_camera = torch.zeros_like(n)


class PathTracer:
    """GPU replacement of CPUPathTracer: same ``render(camera, scene)``, ``options``,
    ``render_passes`` (cpu_path_tracer.hpp:46-58)."""

    def __init__(self):
        self.options = PathTracerOptions()
        self.denoiser_options = EATWTOptions()   # CPUPathTracer::denoiserOptions
        self.render_passes = RenderPasses()
        self.last_stats = None

    def c_options(self, scene: "Scene") -> capi.PtOptions:
        o = capi.PtOptions()
        opt = self.options
        if opt.samples < 1:
            raise ValueError("options.samples must be >= 1")
        o.samples, o.bounces = int(opt.samples), int(opt.bounces)
        o.show_background = int(bool(opt.show_background))
        o.simulate_lighting = int(bool(self.render_passes.simulate_lighting))
        o.smooth_shading = int(scene.smooth_shading())
        o.deterministic_light = int(bool(opt.deterministic_light))
        o.rr_depth = int(opt.rr_depth)
        o.seed, o.frame = int(opt.seed), int(opt.frame)
        o.nbands = scene.bands.size
        o.adaptive_sampling = int(bool(opt.adaptive_sampling))
        o.samples_per_batch = int(opt.samples_per_batch)
        o.sampling_tolerance = float(opt.sampling_tolerance)
        o.samples_to_detect_miss = int(opt.samples_to_detect_miss)
        o.denoise = int(bool(opt.denoise))
        o.denoiser = self.denoiser_options.to_c()
        if scene.ambient is not None:
            o.has_ambient = 1
            for k in range(scene.bands.size):
                o.ambient[k] = float(scene.ambient[k])
        for k in range(scene.bands.size):
            o.background[k] = float(scene.background[k])
        return o

    def render(self, camera: Camera, scene: "Scene"):
        import torch

        scene.build_tlas()
        ctx = scene.context()
        lib = capi.load()
        W, H = camera.resolution
        B = scene.bands.size
        dev = torch.device("cuda", scene.device)
        cam = camera.to_c(scene.origin, B)
        lights, nl = scene.c_lights()
        opts = self.c_options(scene)
        rp = self.render_passes
        omega = scene.pixel_solid_angle(camera, cam)
        rp.depth = torch.empty((H, W), dtype=torch.float32, device=dev)
        rp.alpha = torch.empty((H, W), dtype=torch.float32, device=dev)
        rp.albedo = torch.empty((B, H, W), dtype=torch.float32, device=dev)
        rp.normal_global = torch.empty((3, H, W), dtype=torch.float32, device=dev)
        rp.triangle_id = torch.empty((H, W), dtype=torch.int32, device=dev)
        if rp.simulate_lighting:
            rp.total_radiance = torch.empty((B, H, W), dtype=torch.float32, device=dev)
            rp.direct_radiance = torch.empty((B, H, W), dtype=torch.float32, device=dev)
            rp.indirect_radiance = torch.empty((B, H, W), dtype=torch.float32, device=dev)
            rp.received_power = torch.empty((B, H, W), dtype=torch.float32, device=dev)
        else:
            rp.total_radiance = rp.direct_radiance = rp.indirect_radiance = rp.received_power = None
        if rp.save_velocity:
            rp.velocity_global = torch.empty((3, H, W), dtype=torch.float32, device=dev)
            rp.velocity_camera = torch.empty((3, H, W), dtype=torch.float32, device=dev)
        else:
            rp.velocity_global = rp.velocity_camera = None
        rp.triangle_size = torch.empty((H, W), dtype=torch.float32, device=dev) if rp.save_triangle_size else None
        f = capi.Film()
        for name in ("total_radiance", "direct_radiance", "indirect_radiance", "received_power", "albedo",
                     "normal_global", "depth", "alpha", "triangle_id", "velocity_global", "velocity_camera",
                     "triangle_size"):
            setattr(f, name, capi.ptr(getattr(rp, name)))
        f.pixel_solid_angle = capi.ptr(omega)
        f.on_device = 1
        torch.cuda.current_stream(dev).synchronize()
        capi.check(lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)), ctx, "render")
        st = capi.Stats()
        lib.vgb_get_stats(ctx, C.byref(st))
        self.last_stats = st
        _id_passes(rp, scene, camera, 0, raster=False)
        if rp.received_power is not None and camera.sensor.psf is not None:
            # CPUPathTracer::render convolves the received power with the camera's PSF
            # (cpu_path_tracer.ipp:150-158)
            from .sensor import psf_convolve

            psf_convolve(scene, rp.received_power, camera.psf_kernel(scene.bands))
        return rp


class Rasterizer:
    """GPU replacement of CPURasterizer (cpu_rasterizer.hpp:18-36): ``render(camera, scene)`` fills
    ``render_passes`` (torch CUDA planes) through vgb_rasterize.  triangle_id counts from 1 within
    each instance, as the reference's loop does; alpha is +inf where a triangle was drawn (the
    reference's count / sample with sample 0)."""

    def __init__(self):
        self.render_passes = RenderPasses()
        self.last_stats = None

    def render(self, camera: Camera, scene: "Scene"):
        import torch

        scene.build_tlas()
        ctx = scene.context()
        lib = capi.load()
        W, H = camera.resolution
        B = scene.bands.size
        dev = torch.device("cuda", scene.device)
        cam = camera.to_c(scene.origin, B)
        lights, nl = scene.c_lights()
        o = capi.RasterOptions()
        o.intrinsic[:] = [float(x) for x in camera.intrinsic_matrix()]
        rp = self.render_passes
        o.simulate_lighting = 1 if rp.simulate_lighting else 0
        o.smooth_shading = 1 if scene.smooth_shading() else 0
        o.nbands = B
        rp.depth = torch.empty((H, W), dtype=torch.float32, device=dev)
        rp.alpha = torch.empty((H, W), dtype=torch.float32, device=dev)
        rp.albedo = torch.empty((B, H, W), dtype=torch.float32, device=dev)
        rp.normal_global = torch.empty((3, H, W), dtype=torch.float32, device=dev)
        rp.triangle_id = torch.empty((H, W), dtype=torch.int32, device=dev)
        # the fragment's velocities and projected size (cpu_rasterizer.ipp:123-129, 211-218)
        if rp.save_velocity:
            rp.velocity_global = torch.empty((3, H, W), dtype=torch.float32, device=dev)
            rp.velocity_camera = torch.empty((3, H, W), dtype=torch.float32, device=dev)
        else:
            rp.velocity_global = rp.velocity_camera = None
        rp.triangle_size = torch.empty((H, W), dtype=torch.float32, device=dev) if rp.save_triangle_size else None
        omega = None
        if rp.simulate_lighting:
            omega = scene.pixel_solid_angle(camera, cam)
            for name in ("total_radiance", "direct_radiance", "indirect_radiance", "received_power"):
                setattr(rp, name, torch.empty((B, H, W), dtype=torch.float32, device=dev))
        else:
            rp.total_radiance = rp.direct_radiance = rp.indirect_radiance = rp.received_power = None
        f = capi.Film()
        for name in ("total_radiance", "direct_radiance", "indirect_radiance", "received_power", "albedo",
                     "normal_global", "depth", "alpha", "triangle_id", "velocity_global", "velocity_camera",
                     "triangle_size"):
            setattr(f, name, capi.ptr(getattr(rp, name)))
        f.pixel_solid_angle = capi.ptr(omega)
        f.on_device = 1
        torch.cuda.current_stream(dev).synchronize()
        capi.check(lib.vgb_rasterize(ctx, C.byref(cam), lights, nl, C.byref(o), C.byref(f)), ctx, "rasterize")
        st = capi.Stats()
        lib.vgb_get_stats(ctx, C.byref(st))
        self.last_stats = st
        # triangle ids restart at 1 for every instance (cpu_rasterizer.ipp:70-72)
        _id_passes(rp, scene, camera, 1, raster=True)
        if rp.received_power is not None and camera.sensor.psf is not None:
            from .sensor import psf_convolve

            psf_convolve(scene, rp.received_power, camera.psf_kernel(scene.bands))   # cpu_rasterizer.ipp:264-270
        return rp


@dataclass
class BatchFrame:
    """One frame of a batched render: its camera, samples per pixel, RNG frame key and, optionally,
    its own light positions (FP64, scene frame) in the order of Scene.lights."""

    camera: Camera
    samples: int = 1
    frame: int = 0
    light_positions: list | None = None


# ============================================================================ scene
class Scene:
    """Scene (include/vira/scene.hpp) reduced to what the path tracer reads.

    ``origin`` is the FP64 point of the global frame that becomes the local scene frame's
    origin on the device (rebasing); instances, lights and cameras are placed in FP64.
    """

    def __init__(self, bands: SpectralBands, device: int = 0):
        self.bands = bands
        self.device = device
        self.origin = np.zeros(3, np.float64)
        self.meshes: list[Mesh] = []
        self.instances: list[Instance] = []
        self.lights: list[SphereLight] = []
        self.cameras: list[Camera] = []
        self.ambient = None
        self.background = np.zeros(bands.size, np.float32)
        self.pathtracer = PathTracer()
        self.rasterizer = Rasterizer()
        from .lod import LevelOfDetailManager

        self.lod_manager = LevelOfDetailManager()
        self.bvh_options = capi.BvhOptions(0, 0, 0, 0)
        self._ctx = None
        self._dirty = True
        self._omega_cache = {}
        self.flat = None

    # --- graph (scene/group.hpp:88-133)
    def new_camera(self) -> int:
        self.cameras.append(Camera())
        return ("camera", len(self.cameras) - 1)

    def add_mesh(self, mesh: Mesh) -> tuple:
        self.meshes.append(mesh)
        self._dirty = True
        return ("mesh", len(self.meshes) - 1)

    def new_instance(self, mesh_id) -> tuple:
        self.instances.append(Instance(mesh=mesh_id[1]))
        self._dirty = True
        return ("instance", len(self.instances) - 1)

    def new_sphere_light(self, spectral_input, radius, is_power: bool = False) -> tuple:
        s = np.broadcast_to(np.asarray(spectral_input, np.float32), (self.bands.size,)).astype(np.float32)
        r = np.float32(radius)
        if is_power:
            s = (s / np.float32(np.float32(np.float32(np.float32(4) * PI_F) * np.float32(r * r)) * PI_F)).astype(np.float32)
        self.lights.append(SphereLight(s, r))
        return ("light", len(self.lights) - 1)

    def new_sun(self, temperature: float = 5800.0, steps: int = 1000) -> tuple:
        """Group::newSun (scene/group.ipp:585-591): blackbody sphere light of solar radius."""
        rad = black_body_radiance(self.bands, temperature, steps)
        return self.new_sphere_light(rad, SOLAR_RADIUS, False)

    def set_sun_direction(self, light_id, azimuth_deg: float, elevation_deg: float, distance: float = AU_TO_M):
        """Places a light at `distance` in the direction (azimuth, elevation) from the scene origin, FP64."""
        az, el = math.radians(azimuth_deg), math.radians(elevation_deg)
        d = np.array([math.cos(el) * math.cos(az), math.cos(el) * math.sin(az), math.sin(el)])
        self[light_id].position = self.origin + distance * d

    def set_ambient(self, ambient):
        self.ambient = np.broadcast_to(np.asarray(ambient, np.float32), (self.bands.size,)).astype(np.float32)

    def set_background_emission(self, bg):
        self.background = np.broadcast_to(np.asarray(bg, np.float32), (self.bands.size,)).astype(np.float32)

    def __getitem__(self, key):
        kind, i = key
        return {"camera": self.cameras, "mesh": self.meshes, "instance": self.instances, "light": self.lights}[kind][i]

    def mark_dirty(self):
        self._dirty = True

    def smooth_shading(self) -> bool:
        used = {inst.mesh for inst in self.instances if inst.visible}
        flags = {self.meshes[m].smooth_shading for m in used}
        if len(flags) > 1:
            raise ValueError("meshes with mixed smooth-shading flags are not supported in one scene")
        return flags.pop() if flags else False

    # --- device
    def context(self):
        if self._ctx is None:
            lib = capi.load()
            h = C.c_void_p()
            capi.check(lib.vgb_context_create(C.byref(h), self.device), what="context_create (is a GPU present?)")
            self._ctx = h
        return self._ctx

    def close(self):
        if self._ctx is not None:
            capi.load().vgb_context_destroy(self._ctx)
            self._ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def flatten(self):
        """Scene::processSceneGraph + buildTLAS input: every visible instance's mesh moved into
        the local scene frame in FP64 (rotation, scale, translation, minus `origin`), then FP32."""
        B = self.bands.size
        pos, idx, alb, uv, nrm = [], [], [], [], []
        tex = None
        nmap = None
        moving = []
        base = 0
        tri_offsets = []
        for ii, inst in enumerate(self.instances):
            if not inst.visible:
                continue
            m = self.meshes[inst.mesh]
            n = m.compute_normals()
            p64 = m.positions.astype(np.float64)
            if not (np.array_equal(inst.rotation, np.eye(3)) and inst.scale == 1.0 and not inst.position.any()
                    and not self.origin.any()):
                p64 = (p64 * inst.scale) @ inst.rotation.T + (inst.position - self.origin)
                n = (n.astype(np.float64) @ inst.rotation.T).astype(np.float32)
            pos.append(p64.astype(np.float32))
            nrm.append(n.astype(np.float32))
            idx.append(m.indices.astype(np.uint32) + np.uint32(base))
            a = m.albedo if m.albedo is not None else np.ones((m.positions.shape[0], B), np.float32)
            alb.append(np.broadcast_to(a, (m.positions.shape[0], B)).astype(np.float32))
            uv.append(m.uv if m.uv is not None else np.zeros((m.positions.shape[0], 2), np.float32))
            if m.albedo_map is not None:
                if tex is not None and tex is not m.albedo_map:
                    raise ValueError("one albedo texture per scene is supported")
                tex = m.albedo_map
            if m.normal_map is not None:
                if nmap is not None and nmap is not m.normal_map:
                    raise ValueError("one normal map per scene is supported")
                nmap = m.normal_map
            tri_offsets.append((ii, base, int(m.indices.shape[0])))
            moving.append(bool(inst.velocity.any() or inst.angular_rate.any()))
            base += m.positions.shape[0]
        if not pos:
            raise ValueError("scene has no visible instances")
        self.flat = dict(
            positions=np.ascontiguousarray(np.concatenate(pos)),
            indices=np.ascontiguousarray(np.concatenate(idx)),
            albedo=np.ascontiguousarray(np.concatenate(alb)),
            uv=np.ascontiguousarray(np.concatenate(uv)),
            normals=np.ascontiguousarray(np.concatenate(nrm)),
            texture=None if tex is None else np.ascontiguousarray(tex, np.float32),
            normal_map=None if nmap is None else np.ascontiguousarray(nmap, np.float32).reshape(nmap.shape[0], nmap.shape[1], 3),
            tri_offsets=tri_offsets,
            motion=self._motion_table(tri_offsets) if any(moving) else None,
        )
        return self.flat

    def _motion_table(self, tri_offsets):
        """The instances' motion for the velocity pass: (first triangle in the flattened mesh,
        velocity, angular rate, position rebased on the scene origin in FP64, then FP32)."""
        arr = (capi.InstanceMotion * len(tri_offsets))()
        first = 0
        for k, (ii, _, ntri) in enumerate(tri_offsets):
            inst = self.instances[ii]
            arr[k].first_triangle = first
            p = (inst.position - self.origin).astype(np.float32)
            for a in range(3):
                arr[k].velocity[a] = float(np.float32(inst.velocity[a]))
                arr[k].angular_rate[a] = float(np.float32(inst.angular_rate[a]))
                arr[k].position[a] = float(p[a])
            first += ntri
        return arr

    def build_tlas(self):
        """Scene::buildTLAS (scene.ipp:712-812): flatten, upload and build the BVH when dirty."""
        if not self._dirty:
            return
        f = self.flatten()
        lib = capi.load()
        ctx = self.context()
        tex = f["texture"]
        th, tw = (tex.shape[0], tex.shape[1]) if tex is not None else (0, 0)
        capi.check(lib.vgb_scene_upload(ctx, capi.ptr(f["positions"]), f["positions"].shape[0], capi.ptr(f["indices"]),
                                        f["indices"].shape[0], self.bands.size, capi.ptr(f["albedo"]),
                                        capi.ptr(f["normals"]), capi.ptr(f["uv"]), capi.ptr(tex), tw, th),
                   ctx, "scene_upload")
        if f["motion"] is not None:
            capi.check(lib.vgb_scene_motion(ctx, C.cast(f["motion"], C.c_void_p), len(f["motion"])), ctx, "scene_motion")
        nm = f["normal_map"]
        if nm is not None:
            capi.check(lib.vgb_scene_normal_map(ctx, capi.ptr(nm), nm.shape[1], nm.shape[0]), ctx, "scene_normal_map")
        capi.check(lib.vgb_bvh_build(ctx, C.byref(self.bvh_options)), ctx, "bvh_build")
        self._dirty = False

    def update_positions(self, mesh_index: int, positions) -> None:
        """Moves the vertices of mesh `mesh_index` (same triangles).  When the uploaded scene is
        that mesh alone, untransformed, the device vertices are replaced and the BVH refitted
        (vgb_scene_update_positions); otherwise the scene is flattened and rebuilt."""
        mesh = self.meshes[mesh_index]
        p = np.ascontiguousarray(positions, np.float32)
        if p.shape != mesh.positions.shape:
            raise ValueError("update_positions: shape differs from the mesh's vertices")
        mesh.positions = p.copy()
        mesh.normals = None
        vis = [inst for inst in self.instances if inst.visible]
        in_place = (not self._dirty and self._ctx is not None and len(vis) == 1 and vis[0].mesh == mesh_index
                    and np.array_equal(vis[0].rotation, np.eye(3)) and vis[0].scale == 1.0
                    and not vis[0].position.any() and not self.origin.any())
        if not in_place:
            self._dirty = True
            self.build_tlas()
            return
        ctx = self._ctx
        capi.check(capi.load().vgb_scene_update_positions(ctx, capi.ptr(mesh.positions), None, 0), ctx,
                   "scene_update_positions")
        self._flat_stale = True

    @property
    def flat(self):
        """The flattened scene arrays of the last upload (None before the first); recomputed on
        access after vertices were moved in place."""
        if self._flat is not None and self._flat_stale:
            self._flat_stale = False
            self.flatten()
        return self._flat

    @flat.setter
    def flat(self, value):
        self._flat = value
        self._flat_stale = False

    def c_lights(self):
        arr = (capi.Light * max(1, len(self.lights)))()
        for k, L in enumerate(self.lights):
            p = (L.position - self.origin).astype(np.float32)
            for a in range(3):
                arr[k].position[a] = float(p[a])
            arr[k].radius = float(L.radius)
            for b in range(self.bands.size):
                arr[k].radiance[b] = float(L.radiance[b])
        return arr, len(self.lights)

    def pixel_solid_angle(self, camera: Camera, cam_c: capi.Camera):
        """Camera::initializePixelSolidAngle (camera.ipp:1622-1666) on the device, FP64, cached."""
        import torch

        key = (camera.resolution, tuple(cam_c.kinv), float(cam_c.z_dir), int(cam_c.distortion),
               tuple(cam_c.distortion_coeffs))
        om = self._omega_cache.get(key)
        if om is None:
            W, H = camera.resolution
            om = torch.empty((H, W), dtype=torch.float32, device=torch.device("cuda", self.device))
            torch.cuda.current_stream(om.device).synchronize()
            ctx = self.context()
            capi.check(capi.load().vgb_pixel_solid_angle(ctx, C.byref(cam_c), capi.ptr(om), 1), ctx, "pixel_solid_angle")
            self._omega_cache = {key: om}
        return om

    # --- batched trajectory rendering
    def render_batch(self, frames: list, autotune: bool = True, use_graph: bool = False,
                     planes=("total_radiance", "received_power", "triangle_id", "depth")):
        """Renders many frames in one persistent launch (vgb_render_batch).  Returns one dict of
        torch CUDA planes per frame.  Per-pixel results equal those of rendering each frame with
        PathTracer.render and options.samples/frame set to the frame's values."""
        import torch

        self.build_tlas()
        ctx = self.context()
        lib = capi.load()
        B = self.bands.size
        dev = torch.device("cuda", self.device)
        arr = (capi.Frame * len(frames))()
        outs = []
        keep = []
        for i, fr in enumerate(frames):
            cam = fr.camera.to_c(self.origin, B)
            W, H = fr.camera.resolution
            omega = self._batch_omega(fr.camera, cam)
            keep.append(omega)
            out = {}
            for name in planes:
                if name in ("depth", "alpha", "triangle_size"):
                    out[name] = torch.empty((H, W), dtype=torch.float32, device=dev)
                elif name == "triangle_id":
                    out[name] = torch.empty((H, W), dtype=torch.int32, device=dev)
                elif name in ("normal_global", "velocity_global", "velocity_camera"):
                    out[name] = torch.empty((3, H, W), dtype=torch.float32, device=dev)
                else:
                    out[name] = torch.empty((B, H, W), dtype=torch.float32, device=dev)
            outs.append(out)
            f = arr[i]
            f.camera = cam
            pos = fr.light_positions if fr.light_positions is not None else [L.position for L in self.lights]
            for k, L in enumerate(self.lights):
                p = (np.asarray(pos[k], np.float64) - self.origin).astype(np.float32)
                for a in range(3):
                    f.lights[k].position[a] = float(p[a])
                f.lights[k].radius = float(L.radius)
                for b in range(B):
                    f.lights[k].radiance[b] = float(L.radiance[b])
            f.nlights = len(self.lights)
            f.samples = int(fr.samples)
            f.frame = int(fr.frame)
            for name, t in out.items():
                setattr(f.film, name, t.data_ptr())
            f.film.pixel_solid_angle = omega.data_ptr()
            f.film.on_device = 1
        opts = self.pathtracer.c_options(self)
        bo = capi.BatchOptions(int(autotune), int(use_graph), 0, 0, 0)
        torch.cuda.current_stream(dev).synchronize()
        capi.check(lib.vgb_render_batch(ctx, arr, len(frames), C.byref(opts), C.byref(bo)), ctx, "render_batch")
        st = capi.Stats()
        lib.vgb_get_stats(ctx, C.byref(st))
        self.pathtracer.last_stats = st
        return outs

    def _batch_omega(self, camera: Camera, cam_c):
        import torch

        key = (camera.resolution, tuple(cam_c.kinv), float(cam_c.z_dir), int(cam_c.distortion),
               tuple(cam_c.distortion_coeffs))
        cache = getattr(self, "_omega_batch", None)
        if cache is None:
            cache = self._omega_batch = {}
        om = cache.get(key)
        if om is None:
            W, H = camera.resolution
            om = torch.empty((H, W), dtype=torch.float32, device=torch.device("cuda", self.device))
            torch.cuda.current_stream(om.device).synchronize()
            ctx = self.context()
            capi.check(capi.load().vgb_pixel_solid_angle(ctx, C.byref(cam_c), capi.ptr(om), 1), ctx, "pixel_solid_angle")
            cache[key] = om
        return om

    # --- renders (scene.ipp:840-915)
    def render_total_power(self, camera_id):
        """Scene::renderTotalPower (scene.ipp:873-915): path-traces only when the scene changed since
        the last render (so several exposures reuse one render), then returns the received power.
        Unresolved objects (stars, unresolved bodies) are not rendered here, so the total power is
        the path tracer's received power."""
        rp = self.pathtracer.render_passes
        if self._dirty or rp.received_power is None:
            rp = self.pathtracer.render(self[camera_id], self)
        if rp.received_power is None:
            raise ValueError("render_total_power needs pathtracer.render_passes.simulate_lighting")
        return rp.received_power

    def update_level_of_detail(self, camera_id) -> int:
        """Scene::updateLevelOfDetail: the LoD manager's update for this camera (lod_manager.ipp:24-30)."""
        return self.lod_manager.update(self[camera_id], self)

    def rasterize_render(self, camera_id):
        """Scene::rasterizeRender (scene.ipp:857-862): rasterizes, then simulates the camera's
        sensor on the received power."""
        from .sensor import simulate_sensor

        cam = self[camera_id]
        rp = self.rasterizer.render(cam, self)
        if rp.received_power is None:
            raise ValueError("rasterize_render needs rasterizer.render_passes.simulate_lighting")
        return simulate_sensor(self, rp.received_power, cam.sensor)

    def pathtrace_render(self, camera_id):
        """Scene::pathtraceRender (scene.ipp:840-845): renders, then simulates the camera's sensor
        on the received power; returns the [H][W] image in 0..1 (torch CUDA tensor)."""
        from .sensor import simulate_sensor

        cam = self[camera_id]
        rp = self.pathtracer.render(cam, self)
        if rp.received_power is None:
            raise ValueError("pathtrace_render needs render_passes.simulate_lighting")
        return simulate_sensor(self, rp.received_power, cam.sensor, frame=self.pathtracer.options.frame)

    def pathtrace_render_rgb(self, camera_id):
        """Scene::pathtraceRenderRGB (scene.ipp:847-853): renders, then Camera::simulateSensorRGB
        on the received power; returns [3][H][W] (R, G, B; torch CUDA tensor)."""
        from .sensor import simulate_sensor_rgb

        cam = self[camera_id]
        rp = self.pathtracer.render(cam, self)
        if rp.received_power is None:
            raise ValueError("pathtrace_render_rgb needs render_passes.simulate_lighting")
        return simulate_sensor_rgb(self, rp.received_power, cam.sensor, frame=self.pathtracer.options.frame)

    def rasterize_render_rgb(self, camera_id):
        """Scene::rasterizeRenderRGB (scene.ipp:864-870)."""
        from .sensor import simulate_sensor_rgb

        cam = self[camera_id]
        rp = self.rasterizer.render(cam, self)
        if rp.received_power is None:
            raise ValueError("rasterize_render_rgb needs rasterizer.render_passes.simulate_lighting")
        return simulate_sensor_rgb(self, rp.received_power, cam.sensor)

    def intersect(self, origins: np.ndarray, directions: np.ndarray, any_hit: bool = False, tmax=None):
        """Scene::intersect / TLAS::intersect (scene.hpp:230) for a batch of rays (host arrays)."""
        self.build_tlas()
        lib = capi.load()
        ctx = self.context()
        o = np.ascontiguousarray(origins, np.float32)
        d = np.ascontiguousarray(directions, np.float32)
        n = o.shape[0]
        tri = np.empty(n, np.uint32)
        t = np.empty(n, np.float32)
        w = np.empty((n, 3), np.float32)
        tm = None if tmax is None else np.ascontiguousarray(tmax, np.float32)
        capi.check(lib.vgb_trace_rays(ctx, capi.ptr(o), capi.ptr(d), capi.ptr(tm), n, int(any_hit), capi.ptr(tri),
                                      capi.ptr(t), capi.ptr(w), 0), ctx, "trace_rays")
        return tri, t, w
