"""TEST INFRASTRUCTURE ONLY: a restatement of Vira's DEM Quipu file format (.qld), the checker of
vira_gb300's Quipu reader and writer.  Only tests/ and bench.py's CPU baseline use it.

Follows, field by field:
  quipu::open / readClassID / readVec / readMat / readTransformation / readDEMProjection /
  readDEMHeights / readAlbedos_f / readAlbedos / readImage / decompressData
      include/implementation/quipu/quipu_io.ipp:24-54, 95-102, 151-161, 216-231, 338-377,
      411-440, 480-489, 573-626, 643-702, 717-752
  DEMQuipu::DEMQuipu / readBuffers / write
      include/implementation/quipu/dem_quipu.ipp:29-60, 124-221, 224-332
  floatToFixed / fixedToFloat            include/implementation/images/image_utils.ipp:485-527
  Image::min / max (finite values only)  include/implementation/images/image.ipp:693-737
  DEM::makeVertexBuffer, DEMProjection (non-OGR), imageToIndexBuffer
      include/implementation/dems/dem.ipp:165-211, dem_projection.ipp:66-71, 131-141,
      image_utils.ipp:364-409

LZ4 (the third-party codec the reference links, lz4 1.9.4 pinned in dependencies/vcpkg.json) is
decoded by oracle_lz4_decompress (vgb_oracle.cpp, restated from the published block format).
``liblz4()`` opens the system's liblz4 when one is installed; the fixture script compresses
with its LZ4_compress_default, exactly what quipu::compressData calls, and the CPU tests pin
both the oracle's and the product's decoders against its LZ4_decompress_safe.

PARITY PINNING: the reference ships no Quipu files or known-answer vectors for this format (its
only Quipu test, tests/quipu/test_quipu_io.cpp, round-trips vectors and matrices and is not
built), and it cannot be built here (GDAL, Embree and the rest are absent).  This restatement
is pinned by liblz4 1.9.4 for the compressed payloads and by the byte layout written out above.
"""
from __future__ import annotations

import ctypes as C
import ctypes.util
import struct
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import oracle

IDENT = b"QUIPU"
CLS_FLOAT, CLS_DOUBLE, CLS_U8, CLS_U16, CLS_DEM_PYRAMID = 1, 2, 3, 4, 2002
ELEM = {CLS_U8: np.uint8, CLS_U16: np.uint16, CLS_FLOAT: np.float32}
CONSTANT_ALBEDO, FLOAT_IMAGE_ALBEDO, COLOR_IMAGE_ALBEDO = 0, 1, 2

_lz4 = None


def liblz4():
    """The system's liblz4 (LZ4_compress_default / LZ4_decompress_safe), or None."""
    global _lz4
    if _lz4 is None:
        for name in ("liblz4.so.1", ctypes.util.find_library("lz4")):
            if not name:
                continue
            try:
                lib = C.CDLL(name)
            except OSError:
                continue
            lib.LZ4_compress_default.restype = C.c_int
            lib.LZ4_compress_default.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
            lib.LZ4_decompress_safe.restype = C.c_int
            lib.LZ4_decompress_safe.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int]
            lib.LZ4_compressBound.restype = C.c_int
            lib.LZ4_compressBound.argtypes = [C.c_int]
            lib.LZ4_versionNumber.restype = C.c_int
            _lz4 = lib
            break
        else:
            _lz4 = False
    return _lz4 or None


def lz4_compress_reference(data: bytes) -> bytes:
    lib = liblz4()
    if lib is None:
        raise RuntimeError("liblz4 is not installed: compressed Quipu fixtures cannot be written")
    n = len(data)
    cap = lib.LZ4_compressBound(n)
    out = C.create_string_buffer(cap)
    src = C.create_string_buffer(bytes(data), n)
    got = lib.LZ4_compress_default(src, out, n, cap)
    if got <= 0:
        raise RuntimeError("LZ4_compress_default failed")
    return out.raw[:got]


def lz4_decompress(block: bytes, raw_size: int) -> bytes:
    src = np.frombuffer(block, np.uint8)
    out = np.empty(max(raw_size, 1), np.uint8)
    got = oracle.load().oracle_lz4_decompress(src.ctypes.data, len(block), out.ctypes.data, raw_size)
    if got != raw_size:
        raise ValueError("The provided data failed to be decompressed")
    return out[:raw_size].tobytes()


# ------------------------------------------------------------------ fixed point
def valid_minmax(img: np.ndarray):
    """Image<float>::minmax: over the finite, non-NaN values; FLT_MAX / lowest when none."""
    v = np.asarray(img, np.float32).ravel()
    v = v[np.isfinite(v)]
    if v.size == 0:
        return np.float32(np.finfo(np.float32).max), np.float32(-np.finfo(np.float32).max)
    return np.float32(v.min()), np.float32(v.max())


def float_to_fixed(img, mn, mx, dtype):
    """floatToFixed<T> (clamp = false): code = T((m-1) * (v-min)/(max-min) + 1); 0 for inf, and
    for NaN, where the reference's cast is undefined and x86-64 yields 0."""
    x = np.asarray(img, np.float32)
    m = np.float32(np.iinfo(dtype).max)
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        v = (x - np.float32(mn)) / (np.float32(mx) - np.float32(mn))
        code = (np.float32(m - np.float32(1.0)) * v) + np.float32(1.0)
    bad = np.isinf(x) | np.isnan(code)
    out = np.where(bad, np.float32(0.0), code)
    return np.trunc(out).astype(dtype)


def fixed_to_float(codes, mn, mx):
    c = np.asarray(codes)
    m = np.float32(np.iinfo(c.dtype).max)
    f = c.astype(np.float32) / np.float32(m - np.float32(1.0))
    v = ((np.float32(mx) - np.float32(mn)) * f) + np.float32(mn)
    return np.where(c == 0, np.float32(np.inf), v).astype(np.float32)


# ------------------------------------------------------------------ reading
class _Buf:
    def __init__(self, data: bytes, pos: int = 0):
        self.d, self.p = data, pos

    def take(self, n):
        if self.p + n > len(self.d):
            raise ValueError("truncated Quipu")
        b = self.d[self.p:self.p + n]
        self.p += n
        return b

    def get(self, fmt):
        return struct.unpack("<" + fmt, self.take(struct.calcsize("<" + fmt)))[0]


@dataclass
class Image:
    cls: int
    w: int
    h: int
    compressed: bool
    pixels: np.ndarray      # [h][w] row-major, the stored dtype


@dataclass
class Lod:
    gsd: float
    offset: int
    projection: dict
    hmin: np.float32
    hmax: np.float32
    precision: int
    heights: Image
    albedo_type: int | None = None
    constant_bytes: bytes = b""           # a constant albedo's raw float32 values
    planes: list = field(default_factory=list)   # (min, max, Image)


@dataclass
class QuipuDEM:
    class_id: int
    position: tuple
    rotation: tuple
    scale: tuple
    num_lods: int
    has_albedos: bool
    normal: tuple
    cone_angle: float
    lods: list


def _read_image(b: _Buf) -> Image:
    cls = b.get("H")
    w, h = b.get("I"), b.get("I")
    compressed = b.get("B") != 0
    dt = np.dtype(ELEM[cls])
    n = w * h
    if compressed:
        raw = b.get("Q")
        stored = b.get("Q")
        if raw != n * dt.itemsize:
            raise ValueError("image size mismatch")
        pix = np.frombuffer(lz4_decompress(b.take(stored), raw), dt).reshape(h, w)
    else:
        col = np.frombuffer(b.take(n * dt.itemsize), dt).reshape(w, h)   # x outer, y inner
        pix = np.ascontiguousarray(col.T)
    return Image(cls, w, h, compressed, pix.copy())


def _read_vec(b: _Buf, n):
    cls, k = b.get("H"), b.get("B")
    if k != n:
        raise ValueError("vector length")
    f = "d" if cls == CLS_DOUBLE else "f"
    return tuple(b.get(f) for _ in range(n))


def read(path) -> QuipuDEM:
    data = Path(path).read_bytes()
    b = _Buf(data)
    if b.take(5) != IDENT:
        raise ValueError(f"{path} exists, but is not a valid Quipu!")
    cls = b.get("H")
    position = _read_vec(b, 3)
    mc, n, m = b.get("H"), b.get("B"), b.get("B")
    if (n, m) != (3, 3):
        raise ValueError("rotation size")
    rotation = tuple(b.get("d" if mc == CLS_DOUBLE else "f") for _ in range(9))
    scale = _read_vec(b, 3)
    nl = b.get("H")
    has_alb = b.get("B") != 0
    normal = _read_vec(b, 3)
    cone = b.get("f")
    toc = [(b.get("d"), b.get("Q")) for _ in range(nl)]
    lods = []
    for gsd, off in toc:
        b.p = off
        pr = dict(width=b.get("I"), height=b.get("I"), pixel_scale=(b.get("d"), b.get("d")),
                  tile_definitions=(b.get("I"), b.get("I")), tile_row=b.get("I"), tile_col=b.get("I"),
                  xoff=b.get("d"), yoff=b.get("d"), dx=b.get("d"), dy=b.get("d"), is_ogr=b.get("B") != 0)
        if pr["is_ogr"]:
            ln = b.get("I")
            pr["proj_ref"] = b.take(ln).decode()
            pr["row_col_rotation"] = (b.get("d"), b.get("d"))
            pr["model_tie_point"] = (b.get("d"), b.get("d"))
        hmin, hmax = np.float32(b.get("f")), np.float32(b.get("f"))
        prec = b.get("H")
        img = _read_image(b)
        if img.cls != prec:
            raise ValueError("height image class")
        L = Lod(gsd, off, pr, hmin, hmax, prec, img)
        if has_alb:
            L.albedo_type = b.get("B")
            if L.albedo_type == CONSTANT_ALBEDO:
                L.constant_bytes = data[b.p:b.p + 4 * 8]   # sizeof(TSpectral) bytes are read by the caller
            elif L.albedo_type == FLOAT_IMAGE_ALBEDO:
                mn, mx = np.float32(b.get("f")), np.float32(b.get("f"))
                L.planes.append((mn, mx, _read_image(b)))
            elif L.albedo_type == COLOR_IMAGE_ALBEDO:
                nch = b.get("I")
                b.get("B")
                for _ in range(nch):
                    mn, mx = np.float32(b.get("f")), np.float32(b.get("f"))
                    L.planes.append((mn, mx, _read_image(b)))
            else:
                raise ValueError("albedo type")
        lods.append(L)
    return QuipuDEM(cls, position, rotation, scale, nl, has_alb, normal, cone, lods)


def select_lod(q: QuipuDEM, required_gsd: float) -> int:
    sel = 0
    for i in range(1, len(q.lods)):
        if q.lods[i].gsd <= required_gsd:
            sel = i
        else:
            break
    return sel


def heights(L: Lod) -> np.ndarray:
    if L.precision == CLS_FLOAT:
        return L.heights.pixels.astype(np.float32)
    return fixed_to_float(L.heights.pixels, L.hmin, L.hmax)


def vertex_positions(h: np.ndarray, pr: dict) -> np.ndarray:
    """DEM::makeVertexBuffer positions through DEMProjection::transformToWorld (non-OGR), FP64
    then FP32; +inf where the height is not finite."""
    H, W = h.shape
    pw, ph = pr["width"], pr["height"]
    tsx, tsy = (float(pw) - 1.0) / 2.0, (float(ph) - 1.0) / 2.0
    start_x, start_y = -tsx, -tsy
    scale_x, scale_y = (tsx + 0.5) / float(pw), (tsy + 0.5) / float(ph)
    dx, dy = pr["dx"], pr["dy"]
    ix = np.arange(W, dtype=np.float32).astype(np.float64) + (pr["xoff"] / dx)
    iy = np.arange(H, dtype=np.float32).astype(np.float64) + (pr["yoff"] / dy)
    x_step = ix * scale_x
    y_step = -iy * scale_y
    x = (dx * pr["pixel_scale"][0]) * (start_x + (2.0 * x_step))
    y = (dy * pr["pixel_scale"][1]) * (-start_y + (2.0 * y_step))
    pos = np.empty((H, W, 3), np.float32)
    pos[:, :, 0] = x[None, :].astype(np.float32)
    pos[:, :, 1] = y[:, None].astype(np.float32)
    pos[:, :, 2] = h
    bad = ~np.isfinite(h)
    pos[bad] = np.float32(np.inf)
    return pos.reshape(-1, 3)


def index_buffer(h: np.ndarray) -> np.ndarray:
    """imageToIndexBuffer through the C oracle's DEM triangulation (its faces do not depend on
    the projection)."""
    _, idx = oracle.dem_triangulate(h, 1.0)
    return idx


def vertex_albedo(L: Lod | None, h: np.ndarray, nbands: int, read_albedos=True, default_albedo=0.06,
                  profile=None) -> np.ndarray:
    """Per-vertex albedo of DEMQuipu::readBuffers -> DEM::makeVertexBuffer: the DEM's albedo
    where the height is finite, Vertex's default 1 elsewhere."""
    n = h.size
    prof = np.ones(nbands, np.float32) if profile is None else np.asarray(profile, np.float32)[:nbands]
    out = np.empty((n, nbands), np.float32)
    valid = np.isfinite(h.ravel())
    if L is None or not read_albedos or L.albedo_type is None:
        val = np.full((n, nbands), np.float32(default_albedo), np.float32)
    elif L.albedo_type == CONSTANT_ALBEDO:
        c = np.frombuffer(L.constant_bytes[:4 * nbands], np.float32)
        val = np.broadcast_to(c, (n, nbands))
    elif L.albedo_type == FLOAT_IMAGE_ALBEDO:
        mn, mx, img = L.planes[0]
        g = fixed_to_float(img.pixels, mn, mx).ravel()
        val = prof[None, :] * g[:, None]
    else:
        if len(L.planes) != nbands:
            raise ValueError("channel count differs from the bands")
        val = np.stack([fixed_to_float(img.pixels, mn, mx).ravel() for mn, mx, img in L.planes], axis=1)
    out[:] = np.float32(1.0)
    out[valid] = val[valid]
    return out


# ------------------------------------------------------------------ writing
def _vec(fmt_cls, vals):
    f = "d" if fmt_cls == CLS_DOUBLE else "f"
    return struct.pack("<HB", fmt_cls, len(vals)) + struct.pack("<" + f * len(vals), *vals)


def _image(pix: np.ndarray, cls: int, compress: bool, compressor) -> bytes:
    h, w = pix.shape
    out = struct.pack("<HIIB", cls, w, h, 1 if compress else 0)
    if compress:
        raw = np.ascontiguousarray(pix).tobytes()
        blk = compressor(raw)
        out += struct.pack("<QQ", len(raw), len(blk)) + blk
    else:
        out += np.ascontiguousarray(pix.T).tobytes()     # column by column
    return out


def write(path, lods: list, position=(0.0, 0.0, 0.0), rotation=(1.0, 0, 0, 0, 1.0, 0, 0, 0, 1.0),
          scale=(1.0, 1.0, 1.0), write_albedos=True, compress=False, compressor=None, normal_cone=None):
    """DEMQuipu::write.  Each LoD: dict(heights=[H][W] float32, projection=dict as read() gives,
    albedo_type, albedo=constant [B] | grey [H][W] | per band [H][W][B]).  normal_cone overrides
    the computed (normal, angle), for map-projected LoDs whose vertices need GDAL."""
    compressor = compressor or lz4_compress_reference
    path = Path(path).with_suffix(".qld")
    head = IDENT + struct.pack("<H", CLS_DEM_PYRAMID)
    head += _vec(CLS_DOUBLE, position)
    head += struct.pack("<HBB", CLS_DOUBLE, 3, 3) + struct.pack("<9d", *rotation)
    head += _vec(CLS_DOUBLE, scale)
    head += struct.pack("<HB", len(lods), 1 if write_albedos else 0)
    if normal_cone is None:
        S = lods[-1]
        h = np.asarray(S["heights"], np.float32)
        pos = vertex_positions(h, S["projection"])
        nrm = oracle.compute_normals(pos, index_buffer(h))
        cone = np.zeros(4, np.float32)
        oracle.load().oracle_normal_cone(np.ascontiguousarray(nrm).ctypes.data, nrm.shape[0], cone.ctypes.data)
        normal_cone = (tuple(float(x) for x in cone[:3]), float(cone[3]))
    head += _vec(CLS_FLOAT, normal_cone[0]) + struct.pack("<f", normal_cone[1])
    hmn, hmx = valid_minmax(lods[0]["heights"])
    blocks = []
    atype = lods[0].get("albedo_type", CONSTANT_ALBEDO)
    for L in lods:
        pr = L["projection"]
        h = np.asarray(L["heights"], np.float32)
        blk = struct.pack("<II2d2III4dB", pr["width"], pr["height"], *pr["pixel_scale"], *pr["tile_definitions"],
                          pr["tile_row"], pr["tile_col"], pr["xoff"], pr["yoff"], pr["dx"], pr["dy"],
                          1 if pr.get("is_ogr") else 0)
        if pr.get("is_ogr"):
            s = pr["proj_ref"].encode()
            blk += struct.pack("<I", len(s)) + s + struct.pack("<4d", *pr["row_col_rotation"], *pr["model_tie_point"])
        gsd = np.float32(min(pr["dx"] * pr["pixel_scale"][0], pr["dy"] * pr["pixel_scale"][1]))
        gsd_scale = np.float32(gsd / np.float32(50.0))
        delta = np.float32(hmx - hmn)
        blk += struct.pack("<2f", hmn, hmx)
        if np.float32(delta / np.float32(255.0)) < gsd_scale:
            blk += struct.pack("<H", CLS_U8) + _image(float_to_fixed(h, hmn, hmx, np.uint8), CLS_U8, compress, compressor)
        elif np.float32(delta / np.float32(65535.0)) < gsd_scale:
            blk += struct.pack("<H", CLS_U16) + _image(float_to_fixed(h, hmn, hmx, np.uint16), CLS_U16, compress,
                                                       compressor)
        else:
            blk += struct.pack("<H", CLS_FLOAT) + _image(h, CLS_FLOAT, compress, compressor)
        if write_albedos:
            blk += struct.pack("<B", atype)
            a = np.asarray(L["albedo"], np.float32)
            if atype == CONSTANT_ALBEDO:
                blk += a.tobytes()
            elif atype == FLOAT_IMAGE_ALBEDO:
                mn, mx = valid_minmax(a)
                blk += struct.pack("<2f", mn, mx) + _image(float_to_fixed(a, mn, mx, np.uint8), CLS_U8, compress,
                                                           compressor)
            else:
                nb = a.shape[2]
                blk += struct.pack("<IB", nb, 1 if compress else 0)
                for k in range(nb):
                    mn, mx = valid_minmax(a[:, :, k])
                    blk += struct.pack("<2f", mn, mx) + _image(float_to_fixed(a[:, :, k], mn, mx, np.uint8), CLS_U8,
                                                               compress, compressor)
        blocks.append(blk)
    off = len(head) + 16 * len(lods)
    toc = b""
    for L, blk in zip(lods, blocks):
        toc += struct.pack("<dQ", L["projection"]["dx"] * L["projection"]["pixel_scale"][0], off)
        off += len(blk)
    path.parent.mkdir(parents=True, exist_ok=True)
    path.write_bytes(head + toc + b"".join(blocks))
    return path


def projection(width, height, pixel_scale=(1.0, 1.0), dx=1.0, dy=1.0, xoff=0.0, yoff=0.0, tile=(0, 0, 0, 0)):
    return dict(width=width, height=height, pixel_scale=tuple(pixel_scale), tile_definitions=(tile[0], tile[1]),
                tile_row=tile[2], tile_col=tile[3], xoff=xoff, yoff=yoff, dx=dx, dy=dy, is_ogr=False)

