"""TEST INFRASTRUCTURE ONLY: ctypes wrapper of the oracle (oracle/vgb_oracle.cpp).

The oracle is a CPU restatement of Vira's CPU path tracer used as the parity checker and as
the timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline /
reference legs may use it.  Parity with the reference itself is unpinned (the reference
cannot be built here and ships no golden vectors); see the header of vgb_oracle.cpp.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

from vira_gb300 import capi

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libvgb_oracle.so"
_lib = None


def build(force: bool = False) -> Path:
    src = HERE / "vgb_oracle.cpp"
    hdr = HERE.parent / "include" / "vgb.h"
    if force or not LIB.exists() or LIB.stat().st_mtime < max(src.stat().st_mtime, hdr.stat().st_mtime):
        r = subprocess.run(["make", "-C", str(HERE), "-B" if force else "all"], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(str(LIB))
    P, U32 = C.c_void_p, C.c_uint32
    sig = {
        "oracle_philox": (None, [P, P, P]),
        "oracle_compute_normals": (C.c_int, [P, U32, P, U32, P]),
        "oracle_dem_triangulate": (C.c_int, [P, U32, U32, C.c_double, C.c_double, P, P, C.POINTER(U32)]),
        "oracle_intrinsics": (C.c_int, [C.c_float] * 3 + [U32, U32] + [C.c_float] * 5 + [P]),
        "oracle_pixel_solid_angle": (C.c_int, [C.POINTER(capi.Camera), P, C.c_int]),
        "oracle_distortion": (C.c_int, [C.POINTER(capi.Camera), P, U32, C.c_int, P]),
        "oracle_blackbody_band": (C.c_double, [C.c_double, C.c_float, C.c_float, U32]),
        "oracle_scene_create": (P, [P, U32, P, U32, U32, P, P, P, P, U32, U32]),
        "oracle_scene_destroy": (None, [P]),
        "oracle_scene_normal_map": (C.c_int, [P, P, U32, U32]),
        "oracle_scene_motion": (C.c_int, [P, P, U32]),
        "oracle_scene_bvh_nodes": (U32, [P]),
        "oracle_trace": (C.c_int, [P, P, P, P, U32, C.c_int, C.c_int, P, P, P, C.c_int, P, P]),
        "oracle_render": (C.c_int, [P, C.POINTER(capi.Camera), P, U32, C.POINTER(capi.PtOptions),
                                    C.POINTER(capi.Film), U32, U32, U32, C.c_int, P]),
        "oracle_adjoint": (C.c_int, [P, C.POINTER(capi.Camera), P, U32, C.POINTER(capi.PtOptions), P, P, P, C.c_int]),
        "oracle_sensor": (C.c_int, [P, P, U32, U32, U32, C.c_float, P, P, C.c_float, C.c_float, P]),
        "oracle_psf": (C.c_int, [P, U32, U32, U32, P, U32, U32, P]),
        "oracle_sensor_rgb": (C.c_int, [P, P, U32, U32, U32, P, P, P, C.c_float, C.c_float, C.c_float, P]),
        "oracle_denoise": (C.c_int, [P, P, P, P, P, U32, U32, U32, U32, U32, C.c_float, C.c_float, C.c_float,
                                     C.c_float]),
        "oracle_adjoint_positions": (C.c_int, [P, C.POINTER(capi.Camera), P, U32, C.POINTER(capi.PtOptions), P, P, P,
                                               C.c_int]),
        "oracle_lz4_decompress": (C.c_int64, [P, C.c_uint64, P, C.c_uint64]),
        "oracle_rasterize": (C.c_int, [P, C.POINTER(capi.Camera), P, P, U32, C.c_int, C.c_int, P, P, P, P, P, P, P, P,
                                       P, P, P]),
        "oracle_normal_cone": (C.c_int, [P, C.c_uint64, P]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def nthreads() -> int:
    return max(1, len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count() or 1)


def philox(ctr, key):
    c = np.array(ctr, np.uint32)
    k = np.array(key, np.uint32)
    out = np.zeros(4, np.uint32)
    load().oracle_philox(c.ctypes.data, k.ctypes.data, out.ctypes.data)
    return out


def compute_normals(pos, idx):
    p = np.ascontiguousarray(pos, np.float32)
    i = np.ascontiguousarray(idx, np.uint32)
    n = np.empty_like(p)
    assert load().oracle_compute_normals(p.ctypes.data, p.shape[0], i.ctypes.data, i.shape[0], n.ctypes.data) == 0
    return n


def dem_triangulate(heights, posting):
    h = np.ascontiguousarray(heights, np.float32)
    H, W = h.shape
    pos = np.empty((H * W, 3), np.float32)
    idx = np.empty((2 * (W - 1) * (H - 1), 3), np.uint32)
    nt = C.c_uint32(0)
    assert load().oracle_dem_triangulate(h.ctypes.data, W, H, posting, posting, pos.ctypes.data, idx.ctypes.data,
                                         C.byref(nt)) == 0
    return pos, idx[: nt.value].copy()


def intrinsics(focal, sx, sy, W, H, px=np.inf, py=np.inf, kxy=0.0, kyx=0.0, z_dir=1.0):
    out = (C.c_float * 6)()
    load().oracle_intrinsics(focal, sx, sy, W, H, px, py, kxy, kyx, z_dir, out)
    return np.array(out[:], np.float32)


def dem_mesh(heights, posting, albedo=None, nbands: int = 1):
    """A DEM mesh built entirely by the oracle (DEM::makeVertexBuffer / imageToIndexBuffer /
    Mesh::calculateNormals restated), for workload builders that must not load the product
    library: the same arrays as vira_gb300.Mesh.from_dem plus its vertex normals."""
    from vira_gb300.scene import Mesh

    pos, idx = dem_triangulate(heights, posting)
    n = pos.shape[0]
    alb = None
    if albedo is not None:
        a = np.asarray(albedo, np.float32)
        if a.ndim == 0 or a.size == nbands:
            alb = np.broadcast_to(a.reshape(1, -1) if a.ndim else a, (n, nbands)).astype(np.float32)
        else:
            alb = a.reshape(n, -1).astype(np.float32)
    return Mesh(pos, idx, albedo=alb, normals=compute_normals(pos, idx))


def camera_kinv(camera):
    """K^-1 of a vira_gb300 Camera by the oracle's restatement of initializeIntrinsicMatrix."""
    W, H = camera.resolution
    return intrinsics(camera.focal_length, camera.sensor_size[0], camera.sensor_size[1], W, H,
                      camera.principal_point[0], camera.principal_point[1], camera.skew[0], camera.skew[1],
                      camera.intrinsics_z_dir)


def distortion(cam: capi.Camera, xy, inverse: bool):
    """The camera's lens distortion applied to (n, 2) normalised image points (undistort when
    `inverse`), as the oracle's pixelToDirectionHelper / projectCameraPoint apply it."""
    p = np.ascontiguousarray(xy, np.float32).reshape(-1, 2)
    out = np.empty_like(p)
    assert load().oracle_distortion(C.byref(cam), p.ctypes.data, p.shape[0], int(inverse), out.ctypes.data) == 0
    return out


def pixel_solid_angle(cam: capi.Camera):
    out = np.empty((cam.height, cam.width), np.float32)
    assert load().oracle_pixel_solid_angle(C.byref(cam), out.ctypes.data, nthreads()) == 0
    return out


def blackbody_band(T, lmin_m, lmax_m, steps=1000):
    return load().oracle_blackbody_band(T, lmin_m, lmax_m, steps)


def sensor(power, exposure_time, photon_energy, qe, gain, max_adu, mosaic=None):
    """Noise-free sensor chain restated: [B][H][W] received power -> [H][W] image."""
    p = np.ascontiguousarray(power, np.float32)
    B, H, W = p.shape
    e = np.ascontiguousarray(np.asarray(photon_energy, np.float32)[:B])
    q = np.ascontiguousarray(np.asarray(qe, np.float32)[:B])
    m = None if mosaic is None else np.ascontiguousarray(mosaic, np.float32)
    out = np.empty((H, W), np.float32)
    rc = load().oracle_sensor(p.ctypes.data, None if m is None else m.ctypes.data, W, H, B, exposure_time,
                              e.ctypes.data, q.ctypes.data, gain, max_adu, out.ctypes.data)
    if rc != 0:
        raise ValueError("oracle_sensor rejected its arguments")
    return out


def sensor_rgb(power, band_min, band_max, rgb_min, rgb_max, rgb_bandwidth, rgb_photon_energy, rgb_qe, exposure_time,
               gain, max_adu, mosaic=None):
    """Noise-free RGB sensor restated: [B][H][W] received power -> [3][H][W] image."""
    p = np.ascontiguousarray(power, np.float32)
    B, H, W = p.shape
    bmin = np.ascontiguousarray(np.asarray(band_min, np.float32)[:B])
    bmax = np.ascontiguousarray(np.asarray(band_max, np.float32)[:B])
    rgb = np.ascontiguousarray(np.concatenate([np.asarray(a, np.float32).reshape(3) for a in
                                               (rgb_min, rgb_max, rgb_bandwidth, rgb_photon_energy, rgb_qe)]))
    m = None if mosaic is None else np.ascontiguousarray(mosaic, np.float32)
    out = np.empty((3, H, W), np.float32)
    rc = load().oracle_sensor_rgb(p.ctypes.data, None if m is None else m.ctypes.data, W, H, B, bmin.ctypes.data,
                                  bmax.ctypes.data, rgb.ctypes.data, exposure_time, gain, max_adu, out.ctypes.data)
    if rc != 0:
        raise ValueError("oracle_sensor_rgb rejected its arguments")
    return out


def psf(image, kernel):
    """Spatial convolution restated: [B][H][W] with a [B][kh][kw] kernel, zero padding."""
    a = np.ascontiguousarray(image, np.float32)
    k = np.ascontiguousarray(kernel, np.float32)
    B, H, W = a.shape
    out = np.empty_like(a)
    assert load().oracle_psf(a.ctypes.data, W, H, B, k.ctypes.data, k.shape[2], k.shape[1], out.ctypes.data) == 0
    return out


def denoise(direct, indirect, albedo, depth, normal, levels_direct=5, levels_indirect=5, depth_threshold=0.2,
            normal_threshold=0.5, min_normal_weight=0.3, epsilon=1e-6):
    """EATWT denoiser restated (square images): returns filtered (direct, indirect) planes [B][H][W]."""
    d = np.array(direct, np.float32, order="C", copy=True)
    i = np.array(indirect, np.float32, order="C", copy=True)
    a = np.ascontiguousarray(albedo, np.float32)
    z = np.ascontiguousarray(depth, np.float32)
    n = np.ascontiguousarray(normal, np.float32)
    B, H, W = d.shape
    rc = load().oracle_denoise(d.ctypes.data, i.ctypes.data, a.ctypes.data, z.ctypes.data, n.ctypes.data, W, H, B,
                               levels_direct, levels_indirect, depth_threshold, normal_threshold, min_normal_weight,
                               epsilon)
    if rc != 0:
        raise ValueError("oracle_denoise rejected its arguments (square images only)")
    return d, i


class OracleScene:
    """A flattened scene on the CPU with the reference's own BVH (vira_blas.ipp)."""

    def __init__(self, positions, indices, nbands, albedo=None, normals=None, uv=None, texture=None, normal_map=None):
        self.keep = [np.ascontiguousarray(positions, np.float32), np.ascontiguousarray(indices, np.uint32)]
        p, i = self.keep
        opt = []
        for a in (albedo, normals, uv, texture):
            arr = None if a is None else np.ascontiguousarray(a, np.float32)
            opt.append(arr)
            self.keep.append(arr)
        tex = opt[3]
        th, tw = (tex.shape[0], tex.shape[1]) if tex is not None else (0, 0)
        ptrs = [None if a is None else a.ctypes.data for a in opt]
        self.h = load().oracle_scene_create(p.ctypes.data, p.shape[0], i.ctypes.data, i.shape[0], nbands,
                                            ptrs[0], ptrs[1], ptrs[2], ptrs[3], tw, th)
        if not self.h:
            raise ValueError("oracle_scene_create rejected the scene")
        self.nbands = nbands
        if normal_map is not None:
            nm = np.ascontiguousarray(normal_map, np.float32)
            self.keep.append(nm)
            assert load().oracle_scene_normal_map(self.h, nm.ctypes.data, nm.shape[1], nm.shape[0]) == 0

    def set_motion(self, motion):
        """The instance motion table (a ctypes array of capi.InstanceMotion, or None)."""
        self.keep.append(motion)
        n = 0 if motion is None else len(motion)
        assert load().oracle_scene_motion(self.h, C.cast(motion, C.c_void_p) if n else None, n) == 0

    @staticmethod
    def from_flat(flat, nbands):
        o = OracleScene(flat["positions"], flat["indices"], nbands, flat["albedo"], flat["normals"], flat["uv"],
                        flat["texture"], flat.get("normal_map"))
        if flat.get("motion") is not None:
            o.set_motion(flat["motion"])
        return o

    def close(self):
        if self.h:
            load().oracle_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def rasterize(self, cam: capi.Camera, K, lights, nlights: int, lighting: bool, smooth: bool, omega=None,
                  passes=False):
        """The CPURasterizer restatement: planes depth, alpha, albedo, normal_global, triangle_id
        (index + 1), total_radiance and received_power (with lighting); with `passes` also
        triangle_size, velocity_global and velocity_camera."""
        W, H, B = cam.width, cam.height, self.nbands
        k = np.ascontiguousarray(K, np.float32)
        out = dict(depth=np.empty((H, W), np.float32), alpha=np.empty((H, W), np.float32),
                   albedo=np.empty((B, H, W), np.float32), normal_global=np.empty((3, H, W), np.float32),
                   triangle_id=np.empty((H, W), np.uint32))
        if passes:
            out["triangle_size"] = np.empty((H, W), np.float32)
            out["velocity_global"] = np.empty((3, H, W), np.float32)
            out["velocity_camera"] = np.empty((3, H, W), np.float32)
        if lighting:
            out["total_radiance"] = np.empty((B, H, W), np.float32)
            out["received_power"] = np.empty((B, H, W), np.float32)
        om = None if omega is None else np.ascontiguousarray(omega, np.float32)
        p = lambda a: None if a is None else a.ctypes.data  # noqa: E731
        assert load().oracle_rasterize(self.h, C.byref(cam), k.ctypes.data, lights, nlights, int(lighting), int(smooth),
                                       p(out["depth"]), p(out["alpha"]), p(out["albedo"]), p(out["normal_global"]),
                                       p(out["triangle_id"]), p(out.get("total_radiance")), p(out.get("received_power")),
                                       p(om), p(out.get("triangle_size")), p(out.get("velocity_global")),
                                       p(out.get("velocity_camera"))) == 0
        return out

    def trace(self, origins, dirs, any_hit=False, tmax=None, mode=0, threads=None):
        o = np.ascontiguousarray(origins, np.float32)
        d = np.ascontiguousarray(dirs, np.float32)
        n = o.shape[0]
        tri = np.empty(n, np.uint32)
        t = np.empty(n, np.float32)
        w = np.empty((n, 3), np.float32)
        tm = None if tmax is None else np.ascontiguousarray(tmax, np.float32)
        nodes = C.c_uint64(0)
        tris = C.c_uint64(0)
        assert load().oracle_trace(self.h, o.ctypes.data, d.ctypes.data, None if tm is None else tm.ctypes.data, n,
                                   int(any_hit), mode, tri.ctypes.data, t.ctypes.data, w.ctypes.data,
                                   threads or nthreads(), C.byref(nodes), C.byref(tris)) == 0
        return tri, t, w

    def adjoint(self, cam: capi.Camera, lights, nlights: int, opts: capi.PtOptions, dldi, tex_shape=None,
                nverts=None, threads=None):
        """FP64 gradients of sum(dL/dI * I): (d_texture [th][tw][B] or None, d_height [nverts] or None)."""
        d = np.ascontiguousarray(dldi, np.float32)
        gt = np.zeros(tex_shape, np.float64) if tex_shape is not None else None
        gz = np.zeros(nverts, np.float64) if nverts is not None else None
        rc = load().oracle_adjoint(self.h, C.byref(cam), C.cast(lights, C.c_void_p) if nlights else None, nlights,
                                   C.byref(opts), d.ctypes.data, None if gt is None else gt.ctypes.data,
                                   None if gz is None else gz.ctypes.data, threads or nthreads())
        if rc != 0:
            raise ValueError("oracle_adjoint rejected its arguments")
        return gt, gz

    def adjoint_positions(self, cam: capi.Camera, lights, nlights: int, opts: capi.PtOptions, dldi, tex_shape=None,
                          nverts=None, threads=None):
        """FP64 gradients of sum(dL/dI * I): (d_texture [th][tw][B] or None, d_position [nverts][3] or None)."""
        d = np.ascontiguousarray(dldi, np.float32)
        gt = np.zeros(tex_shape, np.float64) if tex_shape is not None else None
        gp = np.zeros((nverts, 3), np.float64) if nverts is not None else None
        rc = load().oracle_adjoint_positions(self.h, C.byref(cam), C.cast(lights, C.c_void_p) if nlights else None,
                                             nlights, C.byref(opts), d.ctypes.data,
                                             None if gt is None else gt.ctypes.data,
                                             None if gp is None else gp.ctypes.data, threads or nthreads())
        if rc != 0:
            raise ValueError("oracle_adjoint_positions rejected its arguments")
        return gt, gp

    PLANES = ("total_radiance", "direct_radiance", "indirect_radiance", "albedo", "normal_global", "depth", "alpha",
              "triangle_id", "velocity_global", "velocity_camera", "triangle_size")

    def render(self, cam: capi.Camera, lights, nlights: int, opts: capi.PtOptions, omega=None, rows=None,
               threads=None, outputs=None, fill=True):
        """Renders rows [r0, r1) (all rows by default; `rows=(r0, r1, step)` takes every step-th
        row from r0) into host planes; returns (planes, ray_counts).
        `outputs`: the planes to write (default all; received_power too when omega is given);
        `fill=False` leaves the rows not rendered uninitialised (cheap for a band of rows)."""
        W, H, B = cam.width, cam.height, self.nbands
        shapes = {"normal_global": (3, H, W), "velocity_global": (3, H, W), "velocity_camera": (3, H, W),
                  "depth": (H, W), "alpha": (H, W), "triangle_id": (H, W), "triangle_size": (H, W)}
        planes = {}
        for k in (outputs or self.PLANES):
            if k == "received_power":
                continue
            dt = np.uint32 if k == "triangle_id" else np.float32
            shape = shapes.get(k, (B, H, W))
            planes[k] = (np.full(shape, 0xFFFFFFFF if k == "triangle_id" else np.nan, dt) if fill
                         else np.empty(shape, dt))
        f = capi.Film()
        for k, v in planes.items():
            setattr(f, k, v.ctypes.data)
        if omega is not None and (outputs is None or "received_power" in outputs):
            planes["received_power"] = (np.full((B, H, W), np.nan, np.float32) if fill
                                        else np.empty((B, H, W), np.float32))
            om = np.ascontiguousarray(omega, np.float32)
            f.received_power = planes["received_power"].ctypes.data
            f.pixel_solid_angle = om.ctypes.data
        f.on_device = 0
        r0, r1, step = (tuple(rows) + (1,))[:3] if rows is not None else (0, H, 1)
        counts = (C.c_uint64 * 2)()
        rc = load().oracle_render(self.h, C.byref(cam), C.cast(lights, C.c_void_p) if nlights else None, nlights,
                                  C.byref(opts), C.byref(f), r0, r1, step, threads or nthreads(), counts)
        if rc != 0:
            raise ValueError("oracle_render rejected its arguments")
        return planes, (int(counts[0]), int(counts[1]))
