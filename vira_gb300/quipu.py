"""DEM Quipu files (.qld): Vira's on-disk DEM pyramid, read into device meshes.

``DEMQuipu(path, options)`` mirrors vira::quipu::DEMQuipu (include/vira/quipu/dem_quipu.hpp,
include/implementation/quipu/dem_quipu.ipp): the header on construction, ``read_pyramid()``,
``read_buffers(required_gsd)`` (the LoD choice of readBuffers) and the static ``write``.  Reading
goes through libvgb's C ABI: the file is indexed and LZ4-decoded on the host, and the stored
codes are decoded, posed, triangulated and given vertex normals on the GPU
(vgb_quipu_read_mesh).  ``DEM`` holds one LoD's heights, albedo and projection.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .scene import Mesh, _mesh_context

CONSTANT_ALBEDO, FLOAT_IMAGE_ALBEDO, COLOR_IMAGE_ALBEDO = 0, 1, 2
PRECISION = {3: "uint8", 4: "uint16", 1: "float32"}


@dataclass
class DEMProjection:
    """vira::dems::DEMProjection (non-OGR fields; map projections need GDAL)."""

    width: int
    height: int
    pixel_scale: tuple = (1.0, 1.0)
    tile_definitions: tuple = (0, 0)
    tile_row: int = 0
    tile_col: int = 0
    xoff: float = 0.0
    yoff: float = 0.0
    dx: float = 1.0
    dy: float = 1.0
    is_ogr: bool = False
    row_col_rotation: tuple = (0.0, 0.0)
    model_tie_point: tuple = (0.0, 0.0)

    def to_c(self) -> capi.QuipuProjection:
        p = capi.QuipuProjection()
        p.width, p.height = self.width, self.height
        p.pixel_scale[:] = list(self.pixel_scale)
        p.tile_definitions[:] = list(self.tile_definitions)
        p.tile_row, p.tile_col = self.tile_row, self.tile_col
        p.xoff, p.yoff, p.dx, p.dy = self.xoff, self.yoff, self.dx, self.dy
        p.is_ogr = 1 if self.is_ogr else 0
        p.row_col_rotation[:] = list(self.row_col_rotation)
        p.model_tie_point[:] = list(self.model_tie_point)
        return p

    @staticmethod
    def from_c(p: capi.QuipuProjection) -> "DEMProjection":
        return DEMProjection(p.width, p.height, tuple(p.pixel_scale), tuple(p.tile_definitions), p.tile_row,
                             p.tile_col, p.xoff, p.yoff, p.dx, p.dy, bool(p.is_ogr), tuple(p.row_col_rotation),
                             tuple(p.model_tie_point))


@dataclass
class DEM:
    """vira::dems::DEM: heights [H][W] (+inf = no data), albedo (constant [B], grey [H][W] or per
    band [H][W][B], or None) and the projection."""

    heights: np.ndarray
    projection: DEMProjection
    albedo: np.ndarray | None = None
    albedo_type: int = CONSTANT_ALBEDO

    def get_gsd(self):
        """DEM::getGSD (dem.ipp:615-621)."""
        p = self.projection
        return (p.dx * p.pixel_scale[0], p.dy * p.pixel_scale[1])

    def downsample(self, factor: int) -> "DEM":
        """Every `factor`-th post, the projection's dx/dy scaled to match: a coarser LoD."""
        h = np.ascontiguousarray(self.heights[::factor, ::factor])
        p = self.projection
        proj = DEMProjection(h.shape[1], h.shape[0], p.pixel_scale, p.tile_definitions, p.tile_row, p.tile_col,
                             p.xoff, p.yoff, p.dx * factor, p.dy * factor)
        a = self.albedo
        if a is not None and self.albedo_type != CONSTANT_ALBEDO:
            a = np.ascontiguousarray(a[::factor, ::factor])
        return DEM(h, proj, a, self.albedo_type)


@dataclass
class DEMQuipuReaderOptions:
    read_albedos: bool = True
    default_gsd: float = math.inf
    default_albedo: float = 0.06
    albedo_profile: np.ndarray | None = None   # per band, multiplies a grey albedo


@dataclass
class DEMQuipuWriterOptions:
    compress: bool = False
    write_albedos: bool = True


def _err() -> str:
    m = capi.load().vgb_quipu_last_error()
    return m.decode() if m else ""


class DEMQuipu:
    """An open .qld file (vira::quipu::DEMQuipu)."""

    def __init__(self, path, options: DEMQuipuReaderOptions | None = None, nbands: int = 1):
        self.filepath = str(path)
        self.options = options or DEMQuipuReaderOptions()
        self.nbands = nbands
        lib = capi.load()
        h = C.c_void_p()
        st = lib.vgb_quipu_open(self.filepath.encode(), C.byref(h))
        if st != 0:
            raise capi.VgbError(st, _err())
        self._h = h
        hd = capi.QuipuHeader()
        capi.check(lib.vgb_quipu_get_header(h, C.byref(hd)), what="quipu_get_header")
        self.class_id = hd.class_id
        self.number_of_lods = hd.num_lods
        self._has_albedos = bool(hd.has_albedos)
        self.position = np.array(hd.position[:], np.float64)
        self.rotation = np.array(hd.rotation[:], np.float64).reshape(3, 3).T    # stored column-major
        self.scale = np.array(hd.scale[:], np.float64)
        self.normal = np.array(hd.normal[:], np.float32)
        self.cone_angle = float(hd.cone_angle)
        self.lods = []
        for i in range(hd.num_lods):
            info = capi.QuipuLodInfo()
            capi.check(lib.vgb_quipu_get_lod(h, i, C.byref(info)), what="quipu_get_lod")
            self.lods.append(info)
        self.gsds = [L.gsd for L in self.lods]
        self.default_gsd = self.options.default_gsd
        self.current_gsd = math.inf
        self._compressed = False

    def close(self):
        if getattr(self, "_h", None):
            capi.load().vgb_quipu_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- header queries (dem_quipu.hpp:66-78)
    def get_transformation(self) -> np.ndarray:
        """ReferenceFrame::makeTransformationMatrix(position, rotation, scale) (reference_frame.ipp:488-500)."""
        T = np.eye(4)
        T[:3, :3] = self.rotation * self.scale[None, :]
        T[:3, 3] = self.position
        return T

    def has_albedos(self) -> bool:
        return self._has_albedos

    def is_compressed(self) -> bool:
        return self._compressed

    def select_lod(self, required_gsd: float) -> int:
        return int(capi.load().vgb_quipu_select_lod(self._h, float(required_gsd)))

    # --- reading
    def read_heights(self, lod: int) -> np.ndarray:
        L = self.lods[lod]
        out = np.empty((L.height, L.width), np.float32)
        capi.check(capi.load().vgb_quipu_read_heights(self._h, lod, capi.ptr(out)), what="quipu_read_heights: " + _err())
        return out

    def read_albedo(self, lod: int, nbands: int | None = None):
        L = self.lods[lod]
        nb = nbands or self.nbands
        if L.albedo_type == capi.QUIPU_NO_ALBEDO:
            return None
        if L.albedo_type == CONSTANT_ALBEDO:
            out = np.empty(nb, np.float32)
        elif L.albedo_type == FLOAT_IMAGE_ALBEDO:
            out = np.empty((L.height, L.width), np.float32)
        else:
            out = np.empty((L.height, L.width, L.albedo_channels), np.float32)
            nb = L.albedo_channels
        capi.check(capi.load().vgb_quipu_read_albedo(self._h, lod, nb, capi.ptr(out)), what="quipu_read_albedo: " + _err())
        return out

    def read_pyramid(self) -> list:
        """DEMQuipu::readPyramid (dem_quipu.ipp:64-121): every LoD as a DEM."""
        out = []
        for i, L in enumerate(self.lods):
            a = self.read_albedo(i) if (self._has_albedos and self.options.read_albedos) else None
            at = L.albedo_type if a is not None else CONSTANT_ALBEDO
            if a is None:
                a = np.full(self.nbands, np.float32(self.options.default_albedo), np.float32)
            out.append(DEM(self.read_heights(i), DEMProjection.from_c(L.projection), a, at))
        return out

    def _read_options(self, nbands: int) -> capi.QuipuReadOptions:
        o = capi.QuipuReadOptions()
        o.nbands = nbands
        o.read_albedos = 1 if self.options.read_albedos else 0
        o.default_albedo = float(self.options.default_albedo)
        prof = np.ones(capi.MAX_BANDS, np.float32)
        if self.options.albedo_profile is not None:
            p = np.asarray(self.options.albedo_profile, np.float32)
            prof[: p.size] = p
        o.albedo_profile[:] = [float(x) for x in prof]
        return o

    def read_lod_mesh(self, lod: int, gpu: int = 0, nbands: int | None = None, normals: bool = True,
                      device_arrays: bool = False):
        """One LoD as mesh arrays built on GPU `gpu`: (positions, indices, albedo, normals), numpy
        arrays, or torch CUDA tensors with device_arrays."""
        L = self.lods[lod]
        nb = nbands or self.nbands
        nv = L.width * L.height
        nq = (L.width - 1) * (L.height - 1)
        if L.width < 2 or L.height < 2 or nv >= 1 << 31:   # checked again by vgb_quipu_read_mesh
            raise capi.VgbError(1, f"quipu_read_mesh: LoD {lod} has {L.width} x {L.height} posts, "
                                   "outside 2 x 2 .. 2^31 (32-bit triangle ids)")
        ctx = _mesh_context(gpu)
        lib = capi.load()
        nt = C.c_uint32(0)
        opts = self._read_options(nb)
        if device_arrays:
            import torch

            dev = torch.device("cuda", gpu)
            pos = torch.empty((nv, 3), dtype=torch.float32, device=dev)
            alb = torch.empty((nv, nb), dtype=torch.float32, device=dev)
            nrm = torch.empty((nv, 3), dtype=torch.float32, device=dev) if normals else None
            idx = torch.empty((2 * nq, 3), dtype=torch.int32, device=dev)
            torch.cuda.synchronize(dev)
        else:
            pos = np.empty((nv, 3), np.float32)
            alb = np.empty((nv, nb), np.float32)
            nrm = np.empty((nv, 3), np.float32) if normals else None
            idx = np.empty((2 * nq, 3), np.uint32)
        capi.check(lib.vgb_quipu_read_mesh(ctx, self._h, lod, C.byref(opts), capi.ptr(pos), capi.ptr(alb),
                                           capi.ptr(nrm), capi.ptr(idx), C.byref(nt), 1 if device_arrays else 0),
                   ctx, "quipu_read_mesh")
        self._compressed = bool(L.compressed)
        return pos, idx[: nt.value], alb, nrm

    def read_buffers(self, required_gsd: float | None = None, gpu: int = 0, nbands: int | None = None) -> Mesh | None:
        """DEMQuipu::readBuffers (dem_quipu.ipp:124-221): the LoD for the required GSD (the
        default GSD when none is given) as a Mesh; None when that LoD is already loaded."""
        g = self.default_gsd if required_gsd is None else required_gsd
        lod = self.select_lod(g)
        gsd = float(np.float32(self.gsds[lod]))
        if gsd == self.current_gsd and not math.isinf(self.current_gsd):
            return None
        self.current_gsd = gsd
        if math.isinf(self.default_gsd):
            self.default_gsd = gsd
        pos, idx, alb, nrm = self.read_lod_mesh(lod, gpu, nbands)
        return Mesh(pos, np.ascontiguousarray(idx), albedo=alb, normals=nrm)

    # --- writing
    @staticmethod
    def write(path, pyramid: list, transformation=None, options: DEMQuipuWriterOptions | None = None,
              position=None, rotation=None, scale=None):
        """DEMQuipu::write (dem_quipu.ipp:224-332): `pyramid` finest first.  The transformation is
        given as position / rotation (3x3) / scale, or as a 4x4 without shear (split into those)."""
        opts = options or DEMQuipuWriterOptions()
        if transformation is not None:
            T = np.asarray(transformation, np.float64)
            position = T[:3, 3]
            scale = np.linalg.norm(T[:3, :3], axis=0)
            rotation = T[:3, :3] / scale[None, :]
        position = np.zeros(3) if position is None else np.asarray(position, np.float64)
        rotation = np.eye(3) if rotation is None else np.asarray(rotation, np.float64)
        scale = np.ones(3) if scale is None else np.asarray(scale, np.float64)
        n = len(pyramid)
        arr = (capi.QuipuLodData * n)()
        keep = []
        for k, dem in enumerate(pyramid):
            h = np.ascontiguousarray(dem.heights, np.float32)
            keep.append(h)
            arr[k].projection = dem.projection.to_c()
            arr[k].heights = h.ctypes.data
            arr[k].albedo_type = dem.albedo_type
            a = np.ascontiguousarray(dem.albedo if dem.albedo is not None else np.ones(1), np.float32)
            keep.append(a)
            arr[k].albedo = a.ctypes.data
            arr[k].nbands = a.shape[-1] if dem.albedo_type == COLOR_IMAGE_ALBEDO else (a.size if dem.albedo_type == CONSTANT_ALBEDO else 1)
        pos_c = (C.c_double * 3)(*position.tolist())
        rot_c = (C.c_double * 9)(*rotation.T.ravel().tolist())   # column-major
        sc_c = (C.c_double * 3)(*scale.tolist())
        write_alb = opts.write_albedos and all(d.albedo is not None for d in pyramid)
        st = capi.load().vgb_quipu_write(str(path).encode(), C.cast(arr, C.c_void_p), n, pos_c, rot_c, sc_c,
                                         1 if write_alb else 0, 1 if opts.compress else 0)
        if st != 0:
            raise capi.VgbError(st, _err())
