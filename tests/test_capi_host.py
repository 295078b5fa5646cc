"""C ABI and host-side logic on the CPU: the library loads and exports every symbol
include/vgb.h declares, its host functions validate arguments, and the reference-shaped host
API does its FP64 pose, ephemeris and rebasing work correctly.  No kernel runs here."""
from __future__ import annotations

import ctypes as C
import math
import re
from pathlib import Path

import numpy as np
import pytest

from vira_gb300 import Camera, Mesh, Scene, FOUR_BAND, EIGHT_BAND, capi

ROOT = Path(__file__).resolve().parent.parent


def _declared_symbols():
    text = (ROOT / "include" / "vgb.h").read_text()
    return sorted(set(re.findall(r"VGB_API\s+[\w\s\*]+?\b(vgb_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    names = _declared_symbols()
    assert len(names) >= 18
    for n in names:
        assert hasattr(lib, n), n
        assert n in capi.SIGNATURES, f"{n} has no ctypes signature"
    assert set(capi.SIGNATURES) == set(names)
    assert b"sm_103a" in lib.vgb_version()


def test_struct_layouts_match_the_header(tmp_path):
    """Every ctypes struct has the size and field offsets a C compiler gives the header's struct."""
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    pairs = {"vgb_camera": capi.Camera, "vgb_light": capi.Light, "vgb_pt_options": capi.PtOptions,
             "vgb_film": capi.Film, "vgb_frame": capi.Frame, "vgb_view": capi.View,
             "vgb_batch_options": capi.BatchOptions, "vgb_bvh_options": capi.BvhOptions, "vgb_stats": capi.Stats, "vgb_sensor": capi.Sensor,
             "vgb_denoise_options": capi.DenoiseOptions, "vgb_quipu_header": capi.QuipuHeader,
             "vgb_quipu_projection": capi.QuipuProjection, "vgb_quipu_lod_info": capi.QuipuLodInfo,
             "vgb_quipu_read_options": capi.QuipuReadOptions, "vgb_quipu_lod_data": capi.QuipuLodData,
             "vgb_raster_options": capi.RasterOptions, "vgb_instance_motion": capi.InstanceMotion,
             "vgb_rgb_conversion": capi.RgbConversion}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "vgb.h"', "int main(void) {"]
    for cname, py in pairs.items():
        lines.append(f'    printf("{cname} %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'    printf("{cname}.{f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    inc = Path(__file__).resolve().parents[1] / "include"
    subprocess.run([cc, "-std=c99", "-I", str(inc), str(src), "-o", str(exe)], check=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines())
    for cname, py in pairs.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for f in py._fields_:
            assert int(got[f"{cname}.{f[0]}"]) == getattr(py, f[0]).offset, f"{cname}.{f[0]}"


def test_context_without_gpu_fails_cleanly():
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except Exception:
        pass
    lib = capi.load()
    h = C.c_void_p()
    assert lib.vgb_context_create(C.byref(h), 0) != 0
    assert not h.value
    assert lib.vgb_context_destroy(None) == 1
    assert lib.vgb_render(None, None, None, 0, None, None) == 1
    assert lib.vgb_last_error(None) == b"null context"


def test_host_functions_validate_arguments():
    lib = capi.load()
    p = np.zeros((3, 3), np.float32)
    i = np.array([[0, 1, 5]], np.uint32)  # index out of range
    n = np.zeros_like(p)
    assert lib.vgb_compute_vertex_normals(capi.ptr(p), 3, capi.ptr(i), 1, capi.ptr(n)) == 1
    assert lib.vgb_compute_vertex_normals(None, 3, capi.ptr(i), 1, capi.ptr(n)) == 1
    nt = C.c_uint32(0)
    h = np.zeros((1, 5), np.float32)
    assert lib.vgb_dem_triangulate(capi.ptr(h), 5, 1, 1.0, 1.0, capi.ptr(p), capi.ptr(i), C.byref(nt)) == 1
    out = (C.c_float * 6)()
    assert lib.vgb_camera_intrinsics(0.0, 0.036, 0.036, 64, 64, math.inf, math.inf, 0, 0, 1.0, out) == 1
    assert lib.vgb_camera_intrinsics(0.05, 0.036, 0.036, 0, 64, math.inf, math.inf, 0, 0, 1.0, out) == 1


def test_degenerate_and_infinite_triangles_in_normals():
    p = np.array([[0, 0, 0], [1, 0, 0], [2, 0, 0], [0, 1, 0], [np.inf, 0, 0]], np.float32)
    i = np.array([[0, 1, 2], [0, 1, 3], [0, 3, 4]], np.uint32)  # degenerate, good, infinite
    m = Mesh(p, i)
    n = m.compute_normals()
    assert np.allclose(n[0], [0, 0, 1]) and np.allclose(n[3], [0, 0, 1])
    assert np.allclose(n[2], 0) and np.allclose(n[4], 0)


def test_look_in_direction_is_a_rotation_with_the_boresight_as_z():
    c = Camera()
    d = np.array([math.sin(math.radians(20)), 0.0, -math.cos(math.radians(20))])
    c.look_in_direction(d)
    R = c.rotation
    assert np.allclose(R.T @ R, np.eye(3), atol=1e-12)
    assert abs(np.linalg.det(R) - 1) < 1e-12
    assert np.allclose(R[:, 2], d / np.linalg.norm(d))
    # degenerate up vector (parallel to the direction) picks another candidate
    c.look_in_direction((0, 0, -1), up=(0, 0, 1))
    assert np.allclose(c.rotation[:, 2], [0, 0, -1])
    assert abs(np.linalg.det(c.rotation) - 1) < 1e-12
    c.enable_blender_frame()
    c.look_in_direction((1, 0, 0))
    assert np.allclose(c.rotation[:, 2], [-1, 0, 0])


def test_fp64_rebasing_keeps_km_offsets_exact_at_au_scale():
    """An asteroid 1 AU from the global origin: FP64 poses, rebased before the FP32 cast."""
    au = 149597870700.0
    s = Scene(FOUR_BAND)
    p = np.array([[0, 0, 0], [1.5, 0, 0], [0, 2.25, 0]], np.float32)
    mid = s.add_mesh(Mesh(p, np.array([[0, 1, 2]], np.uint32)))
    inst = s.new_instance(mid)
    s[inst].set_local_position(au, 1000.0, -3.0)
    s.origin = np.array([au, 1000.0, 0.0])
    f = s.flatten()
    assert np.array_equal(f["positions"], p + np.array([0, 0, -3.0], np.float32))
    cid = s.new_camera()
    s[cid].set_local_position(au + 12.5, 1000.0, 500.25)
    c = s[cid].to_c(s.origin, 4)
    assert list(c.origin) == [12.5, 0.0, 500.25]
    # without rebasing, FP32 loses the metre offsets entirely
    assert np.float32(au + 12.5) == np.float32(au)
    sun = s.new_sun()
    s.set_sun_direction(sun, 0.0, 90.0)
    lights, nl = s.c_lights()
    assert nl == 1 and abs(lights[0].position[2] - np.float32(au)) < 1e5
    assert abs(lights[0].radius - 6.96e8) < 1


def test_instance_rotation_and_normals_follow_the_pose():
    s = Scene(FOUR_BAND)
    p = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    mid = s.add_mesh(Mesh(p, np.array([[0, 1, 2]], np.uint32)))
    inst = s.new_instance(mid)
    Rx = np.array([[1, 0, 0], [0, 0, -1], [0, 1, 0]], np.float64)  # +90 deg about x
    s[inst].set_local_rotation(Rx)
    f = s.flatten()
    assert np.allclose(f["positions"][2], [0, 0, 1])
    assert np.allclose(f["normals"][0], [0, -1, 0])


def test_camera_defaults_and_setters_follow_the_reference():
    c = Camera()
    assert c.resolution == (1920, 1080) and float(c.focal_length) == np.float32(0.05)
    c.set_resolution(100, 50)
    assert abs(float(c.sensor_size[1]) - 0.018) < 1e-9  # square pixels keep the aspect
    c.set_field_of_view(30.0)
    assert abs(2 * math.degrees(math.atan(float(c.sensor_size[0]) / 2 / float(c.focal_length))) - 30.0) < 1e-4
    area = c.aperture_area()
    d = float(c.focal_length) / float(c.f_stop)
    assert abs(float(area) - math.pi * d * d / 4) < 1e-9


def test_sphere_light_power_mode():
    s = Scene(FOUR_BAND)
    lid = s.new_sphere_light(1000.0, 2.0, is_power=True)
    r = s[lid].radiance
    assert np.allclose(r, 1000.0 / (4 * math.pi * 4 * math.pi), rtol=1e-6)


def test_options_validation():
    s = Scene(EIGHT_BAND)
    s.pathtracer.options.samples = 0
    with pytest.raises(ValueError):
        s.pathtracer.c_options(s)


def test_failed_host_allocation_returns_a_status():
    """No exception crosses the C boundary: in a child whose address space is capped at 6 GB, a
    host entry whose buffers would need 51 GB returns VGB_ERR_OUT_OF_MEMORY instead of ending
    the process (the caller's one-element arrays are never touched)."""
    import subprocess
    import sys
    import textwrap

    code = textwrap.dedent("""
        import ctypes as C, resource, sys
        import numpy as np
        from vira_gb300 import capi
        lib = capi.load()
        resource.setrlimit(resource.RLIMIT_AS, (6 << 30, resource.RLIM_INFINITY))
        p = np.zeros(3, np.float32); i = np.zeros(3, np.uint32); o = np.full(3, 7.0, np.float32)
        st = lib.vgb_compute_vertex_normals(p.ctypes.data, 0xFFFFFFFF, i.ctypes.data, 0, o.ctypes.data)
        print(st, float(o.sum()))
    """)
    root = Path(__file__).resolve().parents[1]
    r = subprocess.run([sys.executable, "-c", code], cwd=root, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.split() == ["3", "21.0"]


def test_parallel_for_each_joins_and_rethrows(tmp_path):
    """The host thread helper behind the Quipu decode and the SAH builder: every body runs once,
    an exception thrown on a worker (or on the calling thread) reaches the caller only after every
    other body has finished, and an entry's function-try-block turns it into a status."""
    import subprocess

    root = Path(__file__).resolve().parents[1]
    exe = tmp_path / "pfe"
    subprocess.run(["g++", "-O2", "-std=c++17", "-pthread", "-I", str(root / "include"),
                    str(root / "tests/cpp/parallel_for_each.cpp"), "-o", str(exe)], check=True, capture_output=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "worker exception -> status 3 after 7 bodies" in r.stdout
