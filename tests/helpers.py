"""Shared test utilities: primary rays in numpy FP32 (same operation order as the kernels and
the oracle), GPU renders into host arrays, and comparisons."""
from __future__ import annotations

import ctypes as C

import numpy as np

from vira_gb300 import capi

F = np.float32


def primary_rays(cam: capi.Camera):
    """Camera::pixelToRay for sample 0 (pixel corner), FP32, glm operation order."""
    W, H = cam.width, cam.height
    j, i = np.meshgrid(np.arange(H, dtype=F), np.arange(W, dtype=F), indexing="ij")
    K = np.array(cam.kinv[:], F)
    R = np.array(cam.rotation[:], F)
    hx = (K[0] * i + K[2] * j) + K[4] * F(1)
    hy = (K[1] * i + K[3] * j) + K[5] * F(1)
    zd = F(cam.z_dir)
    dc = [hx, zd * hy, np.full_like(hx, zd)]
    dw = [(R[r] * dc[0] + R[3 + r] * dc[1]) + R[6 + r] * dc[2] for r in range(3)]
    n2 = (dw[0] * dw[0] + dw[1] * dw[1]) + dw[2] * dw[2]
    s = F(1) / np.sqrt(n2)
    d = np.stack([dw[0] * s, dw[1] * s, dw[2] * s], -1).reshape(-1, 3).astype(F)
    o = np.broadcast_to(np.array(cam.origin[:], F), d.shape).copy()
    return o, d


def gpu_render_host(scene, cam_id):
    """Renders through the Python API and returns host numpy planes."""
    import torch

    rp = scene.pathtracer.render(scene[cam_id], scene)
    torch.cuda.synchronize()
    out = {}
    for k in ("total_radiance", "direct_radiance", "indirect_radiance", "received_power", "albedo",
              "normal_global", "depth", "alpha"):
        v = getattr(rp, k)
        if v is not None:
            out[k] = v.cpu().numpy()
    out["triangle_id"] = rp.triangle_id.cpu().numpy().view(np.uint32)
    return out


def oracle_render(scene, cam_id, omega=None, rows=None):
    from oracle import oracle

    cam = scene[cam_id].to_c(scene.origin, scene.bands.size)
    if scene.flat is None:
        scene.flatten()
    osc = oracle.OracleScene.from_flat(scene.flat, scene.bands.size)
    lights, nl = scene.c_lights()
    planes, counts = osc.render(cam, lights, nl, scene.pathtracer.c_options(scene), omega=omega, rows=rows)
    osc.close()
    return planes, counts


def rel_err(a, b, floor=1e-30):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    both_inf = np.isinf(a) & np.isinf(b) & (np.sign(a) == np.sign(b))
    with np.errstate(invalid="ignore"):
        e = np.abs(a - b) / np.maximum(np.abs(b), floor)
    e[both_nan | both_inf] = 0.0
    return e


def same_bits(a, b) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


def same_bits_or_nan(a, b) -> bool:
    """Bit-identical wherever either value is a number; NaN wherever either is NaN (CUDA and the
    host libm produce NaNs of different sign and payload, e.g. normalize(0) on sky pixels)."""
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    if a.shape != b.shape:
        return False
    na, nb = np.isnan(a), np.isnan(b)
    return np.array_equal(na, nb) and np.array_equal(a[~na].view(np.uint32), b[~nb].view(np.uint32))


def lz4_zero_run(n: int) -> bytes:
    """A valid LZ4 block of n >= 25 zero bytes at the format's largest expansion: one literal,
    one match at offset 1 whose length runs on in 255-bytes, then the five closing literals."""
    v = n - 25
    ext = b"\xff" * (v // 255) + bytes([v % 255])
    return bytes([0x1F, 0]) + b"\x01\x00" + ext + bytes([0x50]) + bytes(5)


def quipu_with_claimed_lod(path, width: int, height: int, block: bytes | None = None):
    """A one-LoD Quipu (no albedo) whose LZ4-compressed uint8 heights claim width x height posts,
    with `block` (default: lz4_zero_run of that size) as the stored block.  Built from a 3x3
    pyramid written by the oracle's writer, with its height image replaced."""
    import struct

    from oracle import quipu as Q

    def enc(raw: bytes) -> bytes:
        lib = capi.load()
        cap = lib.vgb_lz4_bound(len(raw))
        dst = np.empty(cap, np.uint8)
        src = np.frombuffer(raw, np.uint8)
        return dst[:lib.vgb_lz4_compress(src.ctypes.data, len(raw), dst.ctypes.data, cap)].tobytes()

    h = np.array([[0.0, 0.5, 1.0], [0.2, 0.7, 0.1], [0.9, 0.3, 0.6]], np.float32)
    small = Q.write(path, [dict(heights=h, projection=Q.projection(3, 3))], write_albedos=False,
                    compress=True, compressor=enc)
    data = small.read_bytes()
    head = struct.pack("<HIIB", Q.CLS_U8, 3, 3, 1)
    at = data.index(head)
    assert data.count(head) == 1
    blk = lz4_zero_run(width * height) if block is None else block
    small.write_bytes(data[:at] + struct.pack("<HIIBQQ", Q.CLS_U8, width, height, 1, width * height, len(blk)) + blk)
    return small
