"""Committed golden fixtures (tests/golden/, made by make_golden.py): the oracle must keep
reproducing them, and the GPU path must match them through the C ABI."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from vira_gb300 import capi
from helpers import rel_err

GOLDEN = Path(__file__).resolve().parent / "golden"
FIXTURES = sorted(GOLDEN.glob("golden_*.npz"))


def _load(path):
    z = np.load(path)
    d = {k: z[k] for k in z.files}
    # fixtures written before the lens fields were appended to vgb_camera hold the shorter
    # struct: no distortion, no depth of field (the reference's defaults)
    raw = d["camera"].tobytes()
    cam = capi.Camera.from_buffer_copy(raw.ljust(C.sizeof(capi.Camera), b"\0"))
    if len(raw) < C.sizeof(capi.Camera):
        cam.interpolate_directions = 1
        cam.focus_distance = float("inf")
    nl = int(d["nlights"])
    lights = (capi.Light * max(1, nl)).from_buffer_copy(d["lights"].tobytes().ljust(C.sizeof(capi.Light) * max(1, nl), b"\0"))
    # fixtures written before the adaptive-sampling fields were appended hold the shorter struct;
    # the appended fields are zero (adaptive sampling off, as in the reference's defaults)
    opts = capi.PtOptions.from_buffer_copy(d["options"].tobytes().ljust(C.sizeof(capi.PtOptions), b"\0"))
    tex = d["texture"] if d["texture"].size else None
    return d, cam, lights, nl, opts, tex


def _compare(out, d, deterministic):
    assert np.array_equal(out["triangle_id"], d["out_triangle_id"])
    for k in ("total_radiance", "direct_radiance", "indirect_radiance", "received_power", "albedo", "normal_global",
              "depth", "alpha"):
        e = rel_err(out[k], d["out_" + k])
        if deterministic:
            assert float(e.max()) <= 1e-6, (k, float(e.max()))
        else:
            # path-traced fixtures go through acos/sin/cos, which may differ by an ulp between libms
            assert np.mean(e <= 1e-4) >= 0.98, k
            assert abs(np.nanmean(out[k]) - np.nanmean(d["out_" + k])) <= 1e-3 * abs(np.nanmean(d["out_" + k])) + 1e-9


@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_oracle_reproduces_golden(path):
    d, cam, lights, nl, opts, tex = _load(path)
    B = int(d["nbands"])
    osc = oracle.OracleScene(d["positions"], d["indices"], B, d["albedo"], d["normals"], d["uv"], tex)
    planes, counts = osc.render(cam, lights, nl, opts, omega=d["omega"], threads=2)
    osc.close()
    assert np.array_equal(oracle.pixel_solid_angle(cam), d["omega"])
    _compare(planes, d, deterministic=bool(opts.deterministic_light) and opts.bounces == 0)
    if opts.deterministic_light and opts.bounces == 0:
        assert counts == tuple(int(x) for x in d["ray_counts"])


@pytest.mark.gpu
@pytest.mark.parametrize("path", FIXTURES, ids=[p.stem for p in FIXTURES])
def test_gpu_matches_golden(gpu, path):
    import torch

    d, cam, lights, nl, opts, tex = _load(path)
    B = int(d["nbands"])
    lib = capi.load()
    ctx = C.c_void_p()
    capi.check(lib.vgb_context_create(C.byref(ctx), 0))
    try:
        arrs = [np.ascontiguousarray(d[k], np.float32) for k in ("positions", "albedo", "normals", "uv")]
        idx = np.ascontiguousarray(d["indices"], np.uint32)
        t = None if tex is None else np.ascontiguousarray(tex, np.float32)
        th, tw = (t.shape[0], t.shape[1]) if t is not None else (0, 0)
        capi.check(lib.vgb_scene_upload(ctx, capi.ptr(arrs[0]), arrs[0].shape[0], capi.ptr(idx), idx.shape[0], B,
                                        capi.ptr(arrs[1]), capi.ptr(arrs[2]), capi.ptr(arrs[3]), capi.ptr(t), tw, th), ctx)
        capi.check(lib.vgb_bvh_build(ctx, C.byref(capi.BvhOptions(0, 0, 0, 0))), ctx)
        H, W = cam.height, cam.width
        om = np.empty((H, W), np.float32)
        capi.check(lib.vgb_pixel_solid_angle(ctx, C.byref(cam), capi.ptr(om), 0), ctx)
        assert float(rel_err(om, d["omega"]).max()) <= 1e-6
        out = {
            "total_radiance": np.empty((B, H, W), np.float32), "direct_radiance": np.empty((B, H, W), np.float32),
            "indirect_radiance": np.empty((B, H, W), np.float32), "received_power": np.empty((B, H, W), np.float32),
            "albedo": np.empty((B, H, W), np.float32), "normal_global": np.empty((3, H, W), np.float32),
            "depth": np.empty((H, W), np.float32), "alpha": np.empty((H, W), np.float32),
            "triangle_id": np.empty((H, W), np.uint32),
        }
        f = capi.Film()
        for k, v in out.items():
            setattr(f, k, v.ctypes.data)
        omega = np.ascontiguousarray(d["omega"])
        f.pixel_solid_angle = omega.ctypes.data
        f.on_device = 0
        capi.check(lib.vgb_render(ctx, C.byref(cam), lights, nl, C.byref(opts), C.byref(f)), ctx)
        _compare(out, d, deterministic=bool(opts.deterministic_light) and opts.bounces == 0)
    finally:
        lib.vgb_context_destroy(ctx)
