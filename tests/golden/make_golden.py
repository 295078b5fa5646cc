"""Generates the golden fixtures of this directory with the oracle (run from the repo root:
``python tests/golden/make_golden.py``).

Each fixture holds a small flattened scene (positions, indices, per-vertex albedo, normals,
uv, optional albedo texture), the FP32 camera / light / option structs as raw bytes, and the
oracle's film planes.  tests/test_golden.py re-runs the oracle (and, on a GPU, libvgb.so) on
the stored inputs and compares with the stored outputs.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import oracle  # noqa: E402
from vira_gb300 import workloads  # noqa: E402

HERE = Path(__file__).resolve().parent


def _pack(scene, cam_id, name):
    f = scene.flatten()
    B = scene.bands.size
    cam = scene[cam_id].to_c(scene.origin, B)
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    omega = oracle.pixel_solid_angle(cam)
    osc = oracle.OracleScene.from_flat(f, B)
    planes, counts = osc.render(cam, lights, nl, opts, omega=omega, threads=1)
    osc.close()
    arrays = dict(
        positions=f["positions"], indices=f["indices"], albedo=f["albedo"], normals=f["normals"], uv=f["uv"],
        texture=f["texture"] if f["texture"] is not None else np.zeros((0, 0, B), np.float32),
        camera=np.frombuffer(bytes(cam), np.uint8), lights=np.frombuffer(bytes(lights)[: nl * C.sizeof(lights[0])], np.uint8),
        nlights=np.array(nl), options=np.frombuffer(bytes(opts), np.uint8), nbands=np.array(B),
        omega=omega, ray_counts=np.array(counts, np.uint64),
    )
    for k, v in planes.items():
        arrays["out_" + k] = v
    np.savez_compressed(HERE / f"{name}.npz", **arrays)
    print(name, {k: v.shape for k, v in arrays.items()})


def main():
    s, c = workloads.plain_direct(posts=33, resolution=32, seed=1)
    _pack(s, c, "golden_direct_dem33_32px")
    s, c = workloads.path_traced(posts=65, tex=32, resolution=24, spp=4, bounces=2, rr_depth=1, seed=3)
    s.meshes[0].set_smooth_shading(True)
    _pack(s, c, "golden_path_dem65_24px")


if __name__ == "__main__":
    main()
