"""Small cases of each kernel family for profiler captures (a few GB on the device at most).

    python -m vira_gb300.profile_cases path [scale]   # k_trace / k_shade / k_shadow / k_end_sample
    python -m vira_gb300.profile_cases batch          # k_batch: 24 trajectory frames, 256^2-1024^2
    python -m vira_gb300.profile_cases adjoint        # k_adjoint: 2 views of a 513^2 crater DEM
    python -m vira_gb300.profile_cases after_film     # k_dn_*, k_psf, k_sensor on a 1024^2 frame
    python -m vira_gb300.profile_cases quipu          # k_quipu_decode, k_dem_*, normals: a 2049^2 LoD, twice
    python -m vira_gb300.profile_cases raster         # k_raster_*: 8.4M triangles at 1024^2, 8 bands, twice
    python -m vira_gb300.profile_cases lbvh           # GPU BVH build of 8.4M triangles twice, then one refit

``path`` renders the path-traced workload shrunk by ``scale`` (posts, texture and pixels; 4 spp)
twice; the captures skip the launches of the first render.
"""
from __future__ import annotations

import sys


def main(argv=None):
    import torch

    from . import workloads

    argv = sys.argv[1:] if argv is None else argv
    kind = argv[0] if argv else "path"
    scale = float(argv[1]) if len(argv) > 1 else 0.25
    if kind == "path":
        posts = int(4096 * scale) + 1
        scene, cam = workloads.path_traced(posts=posts, tex=int(4096 * scale), resolution=int(2048 * scale), spp=4)
        for _ in range(2):
            scene.pathtracer.render(scene[cam], scene)
        torch.cuda.synchronize()
        print("path", scene.pathtracer.last_stats.ms_last, "ms")
    elif kind == "batch":
        scene, frames = workloads.trajectory(nframes=24, resolutions=(256, 512, 1024), spps=(1, 4, 16))
        for _ in range(2):
            scene.render_batch(frames, autotune=False, use_graph=False)
        torch.cuda.synchronize()
        print("batch", scene.pathtracer.last_stats.ms_last, "ms")
    elif kind == "adjoint":
        from .autograd import adjoint_views, forward_views

        scene, views = workloads.inversion(posts=513, tex=512, resolution=256, nviews=2, spp=4)
        dev = torch.device("cuda", 0)
        imgs = forward_views(scene, views, dev)
        gt, gz = adjoint_views(scene, views, [torch.ones_like(i) for i in imgs], dev)
        torch.cuda.synchronize()
        print("adjoint", float(gt.abs().sum()))
    elif kind == "after_film":
        from . import sensor

        scene, cam = workloads.path_traced(posts=1025, tex=1024, resolution=1024, spp=2)
        scene.pathtracer.options.denoise = True
        rp = scene.pathtracer.render(scene[cam], scene)
        sensor.psf_convolve(scene, rp.received_power, sensor.GaussianPSF(1.5).make_kernel(scene.bands, 81, 20))
        sm = sensor.SensorModel(simulate_photon_noise=True, noise_model=sensor.NoiseModelConfig(dark_current=20.0))
        img = sensor.simulate_sensor(scene, rp.received_power, sm)
        torch.cuda.synchronize()
        print("after_film", float(img.mean()))
    elif kind == "quipu":
        import tempfile
        from pathlib import Path

        import numpy as np

        from . import quipu, synthetic

        n = 2049
        z = np.ascontiguousarray(synthetic.fbm_heights(n, 0.8, seed=21, lo=-200.0, hi=200.0), np.float32)
        dem = quipu.DEM(z, quipu.DEMProjection(n, n, (1.0, 1.0)), synthetic.lognormal_albedo(n, 0.12, 0.3, seed=23),
                        quipu.FLOAT_IMAGE_ALBEDO)
        with tempfile.TemporaryDirectory() as tmp:
            quipu.DEMQuipu.write(Path(tmp) / "dem", [dem], options=quipu.DEMQuipuWriterOptions(compress=True))
            q = quipu.DEMQuipu(Path(tmp) / "dem.qld", nbands=8)
            for _ in range(2):
                out = q.read_lod_mesh(0, nbands=8, device_arrays=True)
            torch.cuda.synchronize()
            print("quipu", int(out[1].shape[0]), "triangles")
            q.close()
    elif kind in ("raster", "lbvh"):
        import ctypes as C

        from . import capi

        scene, cam = workloads.path_traced(posts=2049, tex=2048, resolution=1024, spp=1)
        scene.build_tlas()
        if kind == "raster":
            scene.rasterizer.render_passes.simulate_lighting = True
            for _ in range(2):
                scene.rasterizer.render(scene[cam], scene)
            torch.cuda.synchronize()
            print("raster", scene.rasterizer.last_stats.ms_last, "ms")
        else:
            lib = capi.load()
            ctx = scene.context()
            for _ in range(2):
                capi.check(lib.vgb_bvh_build(ctx, C.byref(capi.BvhOptions(0, 1, 0, 2))), ctx, "bvh_build")
            p = scene.meshes[0].positions.copy()
            p[:, 2] += 1.0
            scene.update_positions(0, p)
            torch.cuda.synchronize()
            print("lbvh + refit done")
    else:
        raise SystemExit(f"unknown case {kind!r}: path | batch | adjoint | after_film | quipu | raster | lbvh")


if __name__ == "__main__":
    main()
