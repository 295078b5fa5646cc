"""Generates the DEM Quipu fixtures of this directory (run from the repo root:
``python tests/golden/make_quipu.py``; needs the system's liblz4).

The files are written by the oracle's restatement of DEMQuipu::write (oracle/quipu.py) with
payloads compressed by liblz4's LZ4_compress_default -- the call and library version (1.9.4)
the reference's quipu::compressData uses -- so they hold the bytes the reference writer would
produce for the same DEMs.  The source DEMs are kept in quipu_sources.npz.

  quipu_u16_lz4_color.qld     3 LoDs (65x49, 33x25, 17x13; dx = 1, 2, 4; tile offsets), uint16
                              heights with no-data holes, 4-band albedo, LZ4
  quipu_u8_raw_grey.qld       2 LoDs (33x33, 17x17), uint8 heights (coarse GSD), grey albedo,
                              raw (column-ordered) payloads
  quipu_f32_lz4_constant.qld  1 LoD (40x24), FP32 heights (fine GSD, large relief) with NaN and
                              inf posts, constant 4-band albedo, LZ4
  quipu_noalbedo.qld          1 LoD (20x30), uint16 heights, no albedo, LZ4
  quipu_ogr.qld               1 map-projected LoD (projection string, tie point), raw; read for
                              its header and heights only (its vertices need GDAL)
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import quipu as Q  # noqa: E402
from vira_gb300 import synthetic  # noqa: E402

HERE = Path(__file__).resolve().parent


def _heights(w, h, seed, lo, hi):
    n = max(w, h)
    z = synthetic.fbm_heights(n, 0.8, seed=seed, lo=lo, hi=hi)[:h, :w]
    return np.ascontiguousarray(z, np.float32)


def main():
    if Q.liblz4() is None:
        raise SystemExit("liblz4 is required to write the compressed fixtures")
    src = {}

    # 1: uint16, LZ4, per-band albedo, three LoDs with tile offsets
    z = _heights(65, 49, 11, -60.0, 60.0)
    z[5:8, 10:14] = np.inf
    z[40, 60] = -np.inf
    alb = np.stack([synthetic.lognormal_albedo(65, 0.12 + 0.02 * k, 0.3, seed=20 + k)[:49, :65] for k in range(4)], 2)
    alb = np.ascontiguousarray(alb, np.float32)
    lods = []
    for f in (1, 2, 4):
        lods.append(dict(heights=np.ascontiguousarray(z[::f, ::f]),
                         projection=Q.projection(z[::f, ::f].shape[1], z[::f, ::f].shape[0], (10.0, 10.0), dx=f, dy=f,
                                                 xoff=3.0, yoff=-2.0, tile=(4, 4, 1, 2)),
                         albedo_type=Q.COLOR_IMAGE_ALBEDO, albedo=np.ascontiguousarray(alb[::f, ::f])))
    Q.write(HERE / "quipu_u16_lz4_color", lods, position=(1.0e3, -2.0e3, 3.5e2), scale=(1.0, 1.0, 1.0),
            rotation=(0.0, 1.0, 0.0, -1.0, 0.0, 0.0, 0.0, 0.0, 1.0), write_albedos=True, compress=True)
    src["u16_heights"], src["u16_albedo"] = z, alb

    # 2: uint8, raw, grey albedo
    z = _heights(33, 33, 12, 0.0, 300.0)
    g = np.ascontiguousarray(synthetic.lognormal_albedo(33, 0.1, 0.4, seed=30), np.float32)
    lods = [dict(heights=z, projection=Q.projection(33, 33, (100.0, 100.0)), albedo_type=Q.FLOAT_IMAGE_ALBEDO, albedo=g),
            dict(heights=np.ascontiguousarray(z[::2, ::2]), projection=Q.projection(17, 17, (100.0, 100.0), dx=2, dy=2),
                 albedo_type=Q.FLOAT_IMAGE_ALBEDO, albedo=np.ascontiguousarray(g[::2, ::2]))]
    Q.write(HERE / "quipu_u8_raw_grey", lods, write_albedos=True, compress=False)
    src["u8_heights"], src["u8_albedo"] = z, g

    # 3: FP32, LZ4, constant albedo, NaN and inf posts
    z = _heights(40, 24, 13, -1000.0, 1000.0)
    z[3, 4] = np.nan
    z[10:12, 30] = np.inf
    c = np.array([0.05, 0.07, 0.09, 0.11], np.float32)
    lods = [dict(heights=z, projection=Q.projection(40, 24, (0.5, 0.5)), albedo_type=Q.CONSTANT_ALBEDO, albedo=c)]
    Q.write(HERE / "quipu_f32_lz4_constant", lods, write_albedos=True, compress=True)
    src["f32_heights"], src["f32_albedo"] = z, c

    # 4: no albedo
    z = _heights(20, 30, 14, -20.0, 20.0)
    lods = [dict(heights=z, projection=Q.projection(20, 30, (5.0, 5.0)))]
    Q.write(HERE / "quipu_noalbedo", lods, write_albedos=False, compress=True)
    src["noalb_heights"] = z

    # 5: map-projected (parse only)
    z = _heights(16, 12, 15, -5.0, 5.0)
    pr = Q.projection(16, 12, (20.0, -20.0))
    pr.update(is_ogr=True, proj_ref='GEOGCS["Moon 2000",DATUM["D_Moon_2000",SPHEROID["Moon_2000_IAU_IAG",1737400.0,0.0]]]',
              row_col_rotation=(0.0, 0.0), model_tie_point=(-180.0, 90.0))
    Q.write(HERE / "quipu_ogr", [dict(heights=z, projection=pr)], write_albedos=False, compress=False,
            normal_cone=((0.0, 0.0, 1.0), 0.25))
    src["ogr_heights"] = z

    np.savez_compressed(HERE / "quipu_sources.npz", **src)
    for p in sorted(HERE.glob("quipu_*")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
