"""The C++ host API (include/vgb.hpp) as a Vira program would use it: compiled with g++ against
libvgb.so, run, and compared with the Python host's render of the same scene."""
from __future__ import annotations

import subprocess
from pathlib import Path

import numpy as np
import pytest

from vira_gb300 import capi, synthetic, workloads

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parent.parent


def test_cpp_drop_in_matches_python_host(gpu, tmp_path):
    import torch

    lib = capi.library_path()
    exe = tmp_path / "drop_in_render"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", str(ROOT / "include"), str(ROOT / "tests/cpp/drop_in_render.cpp"),
                    "-o", str(exe), "-L", str(lib.parent), "-lvgb", f"-Wl,-rpath,{lib.parent}"], check=True)
    posts, res = 129, 96
    h = synthetic.fbm_heights(posts, 0.8, seed=1, lo=-200.0, hi=200.0)
    hf = tmp_path / "h.bin"
    h.tofile(hf)
    out = tmp_path / "out.bin"
    r = subprocess.run([str(exe), str(hf), str(posts), str(res), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    raw = np.fromfile(out, np.float32)
    P = res * res
    rad_c = raw[: 4 * P].reshape(4, res, res)
    tri_c = raw[4 * P: 5 * P].view(np.uint32).reshape(res, res)
    velc_c = raw[5 * P: 8 * P].reshape(3, res, res)
    tsz_c = raw[8 * P: 9 * P].reshape(res, res)
    scene, cam_id = workloads.plain_direct(posts=posts, resolution=res)
    cam = scene[cam_id]
    cam.velocity = np.array([30.0, -4.0, 2.0])
    cam.angular_rate = np.array([0.0, 0.01, 0.0])
    scene.pathtracer.render_passes.save_velocity = True
    scene.pathtracer.render_passes.save_triangle_size = True
    rp = scene.pathtracer.render(cam, scene)
    torch.cuda.synchronize()
    rad_p = rp.total_radiance.cpu().numpy()
    tri_p = rp.triangle_id.cpu().numpy().view(np.uint32)
    velc_p = rp.velocity_camera.cpu().numpy()
    tsz_p = rp.triangle_size.cpu().numpy()
    scene.close()
    hit = (tri_c == tri_p) & (tri_p != capi.NO_HIT)
    assert hit.mean() > 0.5
    # the C++ layer passes the camera's motion, sensor size and rotation-origin term as the Python host
    assert float(np.abs(velc_c[:, hit] - velc_p[:, hit]).max()) <= 1e-3 * float(np.abs(velc_p[:, hit]).max())
    assert float((np.abs(tsz_c[hit] - tsz_p[hit]) / tsz_p[hit]).max()) <= 1e-4
    assert np.mean(tri_c == tri_p) >= 0.999
    same = tri_c == tri_p
    rel = np.abs(rad_c - rad_p)[:, same] / np.maximum(np.abs(rad_p[:, same]), 1e-30)
    assert float(rel.max()) <= 1e-4
    print(f"C++ vs Python host: identical triangle ids {same.mean():.6f}, "
          f"bit-identical radiance {np.mean(rad_c.view(np.uint32) == rad_p.view(np.uint32)):.6f}")
