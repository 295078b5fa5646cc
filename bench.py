#!/usr/bin/env python
"""Benchmark of the spectral ray-tracing hot path on one GB300 (or N replicas).

Workload (default): the plain path-tracing configuration -- 4097^2 fBm DEM plus a Poisson
crater field (33.5M triangles), 4096^2 lognormal albedo texture, 8 bands 400-1000 nm, 2048^2
image, 64 spp, 3 bounces with sun NEE, Russian roulette after bounce 2.  A step is one full
render of that frame.  Metric: Mrays/s (closest-hit + shadow queries, each one traversal).

  value    device time of K renders, CUDA events on the render stream, inputs resident in HBM
  e2e      the same renders through vgb_render() with host (pinned) film planes: host<->device
           copies inside the timed region
  roofline the dominant kernel family's algorithmic bytes per launch (node and triangle visits
           from a counting pass of the same BVH and rays, ray I/O, shading gathers) over its
           average launch time, against MEASURED_PEAKS.json's HBM copy bandwidth
  cpu_baseline  the oracle (CPU restatement) on the host cores over a bounded band of rows

`--impl reference` times the reference's CPU path tracer as restated by the oracle (the
reference itself cannot be compiled: Embree, TBB and glm are absent) on all host threads.
Multi-GPU: replicas only (the path does not need a collective); each rank renders its own frame.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent

# ncu capture of the full path-traced frame: dram__bytes_read.sum + dram__bytes_write.sum of the
# k_trace launches of one sample, averaged over its four bounces (one pass per launch).
MEASURED_TRAFFIC = {
    ("path_traced_dem4097_tex4096_2048px_64spp_3b_rr2_8band", 2): {"k_trace": 103060416.0},
}
# ncu counters of k_trace on the path-traced workload at scale 0.25 (1025^2 DEM, 512^2, 4 spp):
# bounce 0 (camera rays) and bounce 1 (diffuse continuation rays).
MEASURED_TRACE_COUNTERS = {
    "case": "path_traced scale 0.25 (1025^2 DEM + craters, 512^2, 4 spp, 3 bounces)",
    "issue_active_pct": {"bounce0": 56.4, "bounce1": 48.61},
    "l1_throughput_pct": {"bounce0": 47.76, "bounce1": 31.07},
    "threads_per_warp_inst": {"bounce0": 26.05, "bounce1": 16.06},
    "long_scoreboard_stalls_per_issue": {"bounce0": 5.63, "bounce1": 5.59},
}
L2_PROBE_BYTES = 64 << 20
sys.path.insert(0, str(ROOT))

TRI_BYTES = 48
RAY_IO_CLOSEST = 32 + 16
RAY_IO_SHADOW = 32 + 4


def shade_bytes(B: int) -> int:
    """Per shaded hit: 3 indices, 3 x (position 16 + normal 16 + uv 8 + B albedo), 4 texels x B,
    and the path-state / film read-modify-writes (3 x B floats)."""
    return 12 + 3 * (40 + 4 * B) + 16 * B + 12 * B


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["path_traced", "plain_direct"], default="path_traced")
    ap.add_argument("--scale", type=float, default=1.0, help="shrinks posts and pixels (tests only)")
    ap.add_argument("--spp", type=int, default=None)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU sample time")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-direct", action="store_true", help="skip the extra plain-direct line item")
    ap.add_argument("--layout", type=int, choices=[2, 8], default=2, help="device BVH node layout")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-trajectory line item")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint line item")
    ap.add_argument("--no-asteroid", action="store_true", help="skip the fused batched-adjoint asteroid line item")
    ap.add_argument("--no-after-film", action="store_true", help="skip the denoiser / PSF / sensor line item")
    ap.add_argument("--no-quipu", action="store_true", help="skip the DEM Quipu ingestion line item")
    ap.add_argument("--no-raster", action="store_true", help="skip the rasterizer line item")
    ap.add_argument("--no-bvh", action="store_true", help="skip the BVH build line item")
    ap.add_argument("--profile-case", default=None,
                    help="run one small case for a profiler capture instead of the benchmark "
                         "(path | batch | adjoint | after_film | quipu | raster | lbvh)")
    return ap.parse_args()


def workload_params(args):
    if args.workload == "path_traced":
        posts = int(round((4096 * args.scale))) + 1
        tex = max(2, int(round(4096 * args.scale)))
        res = max(8, int(round(2048 * args.scale)))
        spp = args.spp or 64
        return dict(kind="path_traced", posts=posts, tex=tex, resolution=res, spp=spp, bounces=3, rr_depth=2)
    posts = int(round(512 * args.scale)) + 1
    res = max(8, int(round(1024 * args.scale)))
    return dict(kind="plain_direct", posts=posts, resolution=res, spp=args.spp or 1, bounces=0)


def build_scene(p, device, mesher=None):
    """The workload's scene; `mesher` triangulates the DEM (default: the product's host code; the
    reference arm passes the oracle's restatement so that it never loads libvgb.so)."""
    from vira_gb300 import workloads

    if p["kind"] == "path_traced":
        scene, cam = workloads.path_traced(posts=p["posts"], tex=p["tex"], resolution=p["resolution"], spp=p["spp"],
                                           bounces=p["bounces"], rr_depth=p["rr_depth"], device=device, mesher=mesher)
    else:
        scene, cam = workloads.plain_direct(posts=p["posts"], resolution=p["resolution"], device=device, mesher=mesher)
        scene.pathtracer.options.samples = p["spp"]
    return scene, cam


def bench_config(p, world):
    """The workload as both arms report it (`config` of the JSON line)."""
    res = p["resolution"]
    out = {"workload": config_name(p), "triangles": 2 * (p["posts"] - 1) ** 2, "image": [res, res],
           "spp": p["spp"], "bounces": p["bounces"], "bands": 8 if p["kind"] == "path_traced" else 4}
    if p["kind"] == "path_traced":
        out["rr_after_bounce"] = p["rr_depth"]
    out["l2"] = "flushed between timed GPU renders (256 MB write); the scene working set also exceeds L2"
    out["parallelism"] = "replicas" if world > 1 else "none (one device or one host process)"
    return out


def config_name(p):
    if p["kind"] == "path_traced":
        return f"path_traced_dem{p['posts']}_tex{p['tex']}_{p['resolution']}px_{p['spp']}spp_{p['bounces']}b_rr{p['rr_depth']}_8band"
    return f"plain_direct_dem{p['posts']}_{p['resolution']}px_{p['spp']}spp_4band"


# ------------------------------------------------------------------------ clocks
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, r in rows for k in range(4) if r[k].lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------------ CPU legs
def oracle_scene(scene):
    from oracle import oracle

    if scene.flat is None:
        scene.flatten()
    return oracle.OracleScene.from_flat(scene.flat, scene.bands.size)


# The CPU sample of the frame both CPU legs time: every 64th row (rows 31, 95, 159, ...; a
# stratified sample of 1/64 of the frame's pixels at the frame's full samples per pixel).
ROW_STRIDE, ROW_OFFSET = 64, 31


def sample_rows(H: int):
    stride = max(1, min(ROW_STRIDE, H // 4))
    return list(range(ROW_OFFSET % stride, H, stride))


# the film planes both arms write per step
STEP_PLANES = ("total_radiance", "received_power", "triangle_id", "depth")


def cpu_step(cam, lights, nl, opts, osc, threads: int, omega):
    """One pass of the oracle over the sampled rows (one call, the threads sharing all of them),
    writing the planes the GPU arm writes; returns (rays, pixel samples, seconds)."""
    rows = sample_rows(cam.height)
    step = rows[1] - rows[0] if len(rows) > 1 else 1
    t = time.perf_counter()
    _, counts = osc.render(cam, lights, nl, opts, omega=omega, rows=(rows[0], rows[-1] + 1, step), threads=threads,
                           outputs=STEP_PLANES, fill=False)
    dt = time.perf_counter() - t
    return counts[0] + counts[1], len(rows) * cam.width * opts.samples, dt


def cpu_sample(cam, lights, nl, opts, osc, seconds: float, threads: int, omega):
    """Repeats cpu_step until about `seconds` of CPU work (at least one pass)."""
    rays, px, total = 0, 0, 0.0
    passes = 0
    while passes == 0 or total < seconds:
        r, n, dt = cpu_step(cam, lights, nl, opts, osc, threads, omega)
        rays, px, total, passes = rays + r, px + n, total + dt, passes + 1
    return {"mrays_s": rays / total / 1e6, "spp_s": px / total, "passes": passes, "seconds": total, "rays": rays}


def sample_text(cam, opts):
    rows = sample_rows(cam.height)
    stride = rows[1] - rows[0] if len(rows) > 1 else 1
    return (f"rows {rows[0]}, {rows[0] + stride}, ... ({len(rows)} rows, 1 in {stride}) x {cam.width} px of the "
            f"frame at {opts.samples} spp (CPU restatement of cpu_path_tracer.ipp, BVH2 of vira_blas.ipp, not Embree)")


def run_reference(args, p, rank, world):
    """The reference arm: the oracle's CPU path tracer on all host threads over the fixed row
    sample of the frame.  The scene is built from numpy and the oracle's own triangulation,
    normals and intrinsics; libvgb.so is never loaded."""
    if rank != 0:
        return
    from oracle import oracle

    scene, cam_id = build_scene(p, device=0, mesher=oracle.dem_mesh)
    threads = oracle.nthreads()
    osc = oracle_scene(scene)  # the oracle's own BVH, built once outside the timed steps
    camera = scene[cam_id]
    cam = camera.to_c(scene.origin, scene.bands.size, kinv=oracle.camera_kinv(camera))
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    omega = oracle.pixel_solid_angle(cam)   # Camera::initialize, outside the timed steps
    for _ in range(args.warmup):
        cpu_step(cam, lights, nl, opts, osc, threads, omega)
    rays, px, secs = 0, 0, 0.0
    for _ in range(args.steps):
        r, n, dt = cpu_step(cam, lights, nl, opts, osc, threads, omega)
        rays, px, secs = rays + r, px + n, secs + dt
    osc.close()
    v = rays / secs / 1e6
    line = {
        "metric": "Mrays/s", "value": v, "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 * secs / max(1, args.steps), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded fBm DEM + Poisson craters, lognormal albedo); random-free poses",
        "impl": "reference",
        "config": bench_config(p, 1),
        "spectral_path_samples_per_s": px / secs,
        "cpu_baseline": {"value": v, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": "each step: " + sample_text(cam, opts)},
        "e2e": {"value": v, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ------------------------------------------------------------------------ GPU leg
class Renderer:
    """Lean render loop over the C ABI with preallocated device planes."""

    def __init__(self, scene, cam_id, torch, stream):
        from vira_gb300 import capi

        self.capi = capi
        self.lib = capi.load()
        self.scene = scene
        self.torch = torch
        self.ctx = scene.context()
        camera = scene[cam_id]
        self.cam = camera.to_c(scene.origin, scene.bands.size)
        self.lights, self.nl = scene.c_lights()
        self.opts = scene.pathtracer.c_options(scene)
        self.omega = scene.pixel_solid_angle(camera, self.cam)
        capi.check(self.lib.vgb_set_stream(self.ctx, C.c_void_p(stream.cuda_stream)), self.ctx, "set_stream")
        W, H, B = self.cam.width, self.cam.height, scene.bands.size
        dev = self.omega.device
        self.planes = {
            "total_radiance": torch.empty((B, H, W), device=dev), "received_power": torch.empty((B, H, W), device=dev),
            "triangle_id": torch.empty((H, W), dtype=torch.int32, device=dev), "depth": torch.empty((H, W), device=dev),
        }
        self.film = capi.Film()
        for k, v in self.planes.items():
            setattr(self.film, k, v.data_ptr())
        self.film.pixel_solid_angle = self.omega.data_ptr()
        self.film.on_device = 1
        # host (pinned) planes for the end-to-end leg
        self.host = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in self.planes.items()}
        self.omega_host = self.omega.cpu().pin_memory()
        self.hfilm = capi.Film()
        for k, v in self.host.items():
            setattr(self.hfilm, k, v.data_ptr())
        self.hfilm.pixel_solid_angle = self.omega_host.data_ptr()
        self.hfilm.on_device = 0
        self.d2h_bytes = sum(v.numel() * v.element_size() for v in self.host.values())
        self.h2d_bytes = (self.omega_host.numel() * 4 + C.sizeof(self.cam) + C.sizeof(self.opts)
                          + C.sizeof(capi.Light) * max(1, self.nl))

    def render(self, host=False):
        f = self.hfilm if host else self.film
        self.capi.check(self.lib.vgb_render(self.ctx, C.byref(self.cam), self.lights, self.nl, C.byref(self.opts),
                                            C.byref(f)), self.ctx, "render")

    def stats(self):
        st = self.capi.Stats()
        self.lib.vgb_get_stats(self.ctx, C.byref(st))
        return st


def reduce_replicas(total_ms: float, rays: float, paths: float, world: int, device):
    """Whole-job figures of N replicas: the slowest rank's time, the sum of all ranks' work."""
    if world <= 1:
        return total_ms, rays, paths
    import torch
    import torch.distributed as dist

    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    w = torch.tensor([rays, paths], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t[0]), float(w[0]), float(w[1])


def l2_peak(lib, ctx):
    """GB/s of streaming reads of an L2-resident 64 MiB buffer (vgb_measure_l2_read: 20 passes
    per launch, best of 5 launches, CUDA events)."""
    from vira_gb300 import capi

    g = C.c_double(0.0)
    capi.check(lib.vgb_measure_l2_read(ctx, L2_PROBE_BYTES, 20, 5, C.byref(g)), ctx, "measure_l2_read")
    return float(g.value)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def run_ours(args, p, rank, world, local_rank):
    import torch

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    t0 = time.perf_counter()
    scene, cam_id = build_scene(p, device=local_rank)
    scene.pathtracer.options.frame = rank  # replicas render distinct sample streams
    scene.bvh_options.layout = args.layout
    t1 = time.perf_counter()
    scene.build_tlas()
    t2 = time.perf_counter()
    stream = torch.cuda.Stream(device=dev)
    r = Renderer(scene, cam_id, torch, stream)
    lib = r.lib
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)  # > 129 MB L2
    for _ in range(args.warmup):
        r.render()
    lib.vgb_set_profiling(r.ctx, 1)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    clocks = ClockSampler(local_rank)
    clocks.start()
    ms, rays, paths, st_list = [], 0, 0, []
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)  # L2 flush between timed renders, outside the event pair
            ev0.record(stream)
        r.render()
        with torch.cuda.stream(stream):
            ev1.record(stream)
        ev1.synchronize()
        ms.append(ev0.elapsed_time(ev1))
        st = r.stats()
        st_list.append(st)
        rays += st.rays_closest + st.rays_shadow
        paths += r.cam.width * r.cam.height * r.opts.samples
    torch.cuda.synchronize(dev)
    clk = clocks.stop()
    lib.vgb_set_profiling(r.ctx, 0)
    total_ms, rays, paths = reduce_replicas(float(sum(ms)), float(rays), float(paths), world, dev)
    value = rays / (total_ms / 1000.0) / 1e6

    # e2e through the C ABI with host buffers (wall clock around the blocking call)
    e2e_ms = []
    e2e_rays = 0
    for _ in range(max(1, min(args.steps, 3))):
        t = time.perf_counter()
        r.render(host=True)
        e2e_ms.append((time.perf_counter() - t) * 1000.0)
        st = r.stats()
        e2e_rays += st.rays_closest + st.rays_shadow
    e2e_value = e2e_rays / (sum(e2e_ms) / 1000.0) / 1e6 * (world if world > 1 else 1)

    # roofline: counting pass for algorithmic bytes, live per-family times from the timed region
    lib.vgb_set_count_pass(r.ctx, 1)
    r.render()
    lib.vgb_set_count_pass(r.ctx, 0)
    cst = r.stats()
    s0 = st_list[-1]
    fam = {"k_trace": (sum(s.ms_trace for s in st_list), sum(s.launches_trace for s in st_list)),
           "k_shade": (sum(s.ms_shade for s in st_list), sum(s.launches_shade for s in st_list)),
           "k_shadow": (sum(s.ms_shadow for s in st_list), sum(s.launches_shadow for s in st_list)),
           "k_end_sample": (sum(s.ms_film for s in st_list), sum(s.launches_film for s in st_list))}
    B = scene.bands.size
    node_bytes = cst.bvh_node_bytes
    nodes_sh = cst.nodes_visited - cst.nodes_closest
    tris_sh = cst.tris_tested - cst.tris_closest
    # algorithmic bytes of one render, per kernel family
    alg = {
        "k_trace": cst.nodes_closest * node_bytes + cst.tris_closest * TRI_BYTES + cst.rays_closest * RAY_IO_CLOSEST,
        "k_shade": cst.hits_closest * shade_bytes(B) + cst.rays_closest * 16,
        "k_shadow": nodes_sh * node_bytes + tris_sh * TRI_BYTES + cst.rays_shadow * (RAY_IO_SHADOW + 4 * B + 8),
        "k_end_sample": r.cam.width * r.cam.height * r.opts.samples * 4 * (4 * B + 2),
    }
    launches_one = {"k_trace": s0.launches_trace, "k_shade": s0.launches_shade, "k_shadow": s0.launches_shadow,
                    "k_end_sample": s0.launches_film}
    dominant = max(fam, key=lambda k: fam[k][0])
    dms, dl = fam[dominant]
    per_launch_bytes = alg[dominant] / max(1, launches_one[dominant])
    per_launch_ms = dms / max(1, dl)
    achieved = per_launch_bytes / (per_launch_ms / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    l2 = l2_peak(lib, r.ctx)
    # DRAM bytes (read + write) per launch of the dominant kernel from one ncu capture of this
    # workload, or None for other workloads.
    traffic = MEASURED_TRAFFIC.get((config_name(p), args.layout), {}).get(dominant)
    # the traversal kernels read their nodes and triangles through L1/L2: their bound is the L2
    # read bandwidth; the shading and film kernels stream HBM
    traversal = dominant in ("k_trace", "k_shadow")
    bound_peak = l2 if traversal else peak

    after_film = None
    if not args.no_after_film and p["kind"] == "path_traced" and rank == 0:
        after_film = after_film_item(torch, dev, scene, cam_id, peak)
    raster = None
    if not args.no_raster and p["kind"] == "path_traced" and rank == 0:
        raster = raster_item(torch, dev, scene, cam_id, peak, cpu=not args.no_cpu_baseline)
    bvh = None
    if not args.no_bvh and p["kind"] == "path_traced" and rank == 0 and args.layout == 2:
        bvh = bvh_item(torch, dev, scene, cam_id)
    quipu = None
    if not args.no_quipu and p["kind"] == "path_traced" and rank == 0:
        quipu = quipu_item(torch, dev, peak, cpu=not args.no_cpu_baseline)
    direct = None
    if not args.no_direct and p["kind"] == "path_traced" and rank == 0:
        direct = plain_direct_item(torch, dev, args.layout, 0.0 if args.no_cpu_baseline else 5.0)
    batched = None
    if not args.no_batched and p["kind"] == "path_traced" and rank == 0:
        scene.close()
        batched = batched_item(torch, dev, args.layout)
    adjoint = None
    if not args.no_adjoint and p["kind"] == "path_traced" and rank == 0:
        scene.close()
        adjoint = adjoint_item(torch, dev, args.layout)
    asteroid = None
    if not args.no_asteroid and p["kind"] == "path_traced" and rank == 0:
        scene.close()
        asteroid = asteroid_item(torch, dev, args.layout)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import oracle

        threads = oracle.nthreads()
        osc = oracle_scene(scene)
        c = cpu_sample(r.cam, r.lights, r.nl, r.opts, osc, args.cpu_seconds, threads, r.omega.cpu().numpy())
        osc.close()
        cpu = {"value": c["mrays_s"], "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": f"{c['passes']} passes over " + sample_text(r.cam, r.opts) +
                         f"; {c['rays']} rays in {c['seconds']:.1f} s"}
    if rank == 0:
        launches = int(sum(s.kernel_launches for s in st_list))
        line = {
            "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded fBm DEM + Poisson craters, lognormal albedo); random-free poses",
            "config": bench_config(p, world),
            "bvh": {"layout": f"{args.layout}-wide" if args.layout == 8 else "binary",
                    "nodes": int(cst.bvh_nodes), "node_bytes": int(cst.bvh_node_bytes)},
            "traversal_counts_per_frame": {"nodes_closest": int(cst.nodes_closest),
                                           "tris_closest": int(cst.tris_closest),
                                           "nodes_shadow": int(cst.nodes_visited - cst.nodes_closest),
                                           "tris_shadow": int(cst.tris_tested - cst.tris_closest)},
            "spectral_path_samples_per_s": paths / (total_ms / 1000.0),
            "rays_per_step": rays / args.steps / max(1, world),
            "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": int(r.h2d_bytes),
                    "d2h_bytes_per_step": int(r.d2h_bytes)},
            "roofline": {"bound": "l2" if traversal else "hbm", "kernel": dominant, "achieved": achieved,
                         "peak": bound_peak, "unit": "GB/s", "frac": achieved / bound_peak,
                         "peak_source": ("measured L2 read bandwidth (vgb_measure_l2_read, 64 MiB L2-resident buffer, "
                                         "same run)") if traversal else f"{peak_kind} HBM copy bandwidth (MEASURED_PEAKS.json)",
                         "traffic": traffic,
                         "algorithmic_bytes_per_launch": per_launch_bytes, "ms_per_launch": per_launch_ms,
                         "hbm": {"achieved": (traffic / (per_launch_ms / 1000.0) / 1e9) if traffic else None,
                                 "peak": peak, "frac": (traffic / (per_launch_ms / 1000.0) / 1e9 / peak) if traffic else None,
                                 "peak_source": f"{peak_kind} (MEASURED_PEAKS.json)",
                                 "note": "DRAM bytes per launch (ncu) over the live launch time"},
                         "l2_peak_gb_s": l2,
                         "ncu": MEASURED_TRACE_COUNTERS if traversal else None,
                         "kernel_share": {k: v[0] / max(1e-9, sum(x[0] for x in fam.values())) for k, v in fam.items()}},
            "gpu_launches": launches,
            "setup_s": {"scene": t1 - t0, "upload_and_bvh": t2 - t1},
            "clocks": clk,
        }
        if direct is not None:
            line["plain_direct"] = direct
        if batched is not None:
            line["batched"] = batched
        if adjoint is not None:
            line["adjoint"] = adjoint
        if asteroid is not None:
            line["batched_adjoint"] = asteroid
        if after_film is not None:
            line["after_film"] = after_film
        if quipu is not None:
            line["quipu_ingest"] = quipu
        if raster is not None:
            line["raster"] = raster
        if bvh is not None:
            line["bvh_build"] = bvh
        if cpu is not None:
            line["cpu_baseline"] = cpu
        print(json.dumps(line))
    scene.close()


def batched_item(torch, dev, layout=2, nframes=256, reps=2):
    """The trajectory workload: 256 frames of uneven size and spp in one persistent launch
    (autotuned, CUDA-graph replay) against per-frame vgb_render calls of the same frames."""
    from vira_gb300 import capi, workloads

    scene, frames = workloads.trajectory(nframes=nframes, device=dev.index)
    scene.bvh_options.layout = layout
    scene.build_tlas()
    lib = capi.load()
    ctx = scene.context()
    B = scene.bands.size
    arr = (capi.Frame * len(frames))()
    films = []
    for i, fr in enumerate(frames):
        cam = fr.camera.to_c(scene.origin, B)
        W, H = fr.camera.resolution
        om = scene._batch_omega(fr.camera, cam)
        planes = {"total_radiance": torch.empty((B, H, W), device=dev), "received_power": torch.empty((B, H, W), device=dev),
                  "triangle_id": torch.empty((H, W), dtype=torch.int32, device=dev)}
        f = arr[i]
        f.camera = cam
        L = scene.lights[0]
        p = (np.asarray(fr.light_positions[0]) - scene.origin).astype(np.float32)
        for a in range(3):
            f.lights[0].position[a] = float(p[a])
        f.lights[0].radius = float(L.radius)
        for b in range(B):
            f.lights[0].radiance[b] = float(L.radiance[b])
        f.nlights = 1
        f.samples = fr.samples
        f.frame = fr.frame
        for k, t in planes.items():
            setattr(f.film, k, t.data_ptr())
        f.film.pixel_solid_angle = om.data_ptr()
        f.film.on_device = 1
        films.append(planes)
    opts = scene.pathtracer.c_options(scene)

    def checksum():
        torch.cuda.synchronize(dev)
        return [float(p["total_radiance"].double().sum()) + float(p["triangle_id"].double().sum()) for p in films]

    torch.cuda.synchronize(dev)
    tune = capi.BatchOptions(1, 1, 0, 0, 0)
    capi.check(lib.vgb_render_batch(ctx, arr, len(frames), C.byref(opts), C.byref(tune)), ctx, "render_batch")
    bo = capi.BatchOptions(0, 1, 0, 0, 0)
    bt, rays = [], 0
    for _ in range(reps):
        t = time.perf_counter()
        capi.check(lib.vgb_render_batch(ctx, arr, len(frames), C.byref(opts), C.byref(bo)), ctx, "render_batch")
        bt.append(time.perf_counter() - t)
        st = capi.Stats()
        lib.vgb_get_stats(ctx, C.byref(st))
        rays = st.rays_closest + st.rays_shadow
    sums_batch = checksum()
    # per-frame launches of the plain renderer, same frames
    pt, pr = [], 0
    for _ in range(reps):
        t = time.perf_counter()
        pr = 0
        for i in range(len(frames)):
            f = arr[i]
            o = capi.PtOptions.from_buffer_copy(bytes(opts))
            o.samples, o.frame = f.samples, f.frame
            lights = (capi.Light * 1)(f.lights[0])
            film = capi.Film.from_buffer_copy(bytes(f.film))
            capi.check(lib.vgb_render(ctx, C.byref(f.camera), lights, 1, C.byref(o), C.byref(film)), ctx, "render")
            st = capi.Stats()
            lib.vgb_get_stats(ctx, C.byref(st))
            pr += st.rays_closest + st.rays_shadow
        pt.append(time.perf_counter() - t)
    sums_plain = checksum()
    th, bps, grab = C.c_uint32(), C.c_uint32(), C.c_uint32()
    lib.vgb_batch_tuning(ctx, C.byref(th), C.byref(bps), C.byref(grab))
    samples = sum(int(f.samples) * f.camera.width * f.camera.height for f in arr)
    scene.close()
    tb, tp = min(bt), min(pt)
    return {"workload": f"trajectory_{len(frames)}frames_dem513_8band_direct", "path_samples": samples,
            "rays": int(rays), "batched_s": tb, "per_frame_s": tp, "speedup": tp / tb,
            "batched_mrays_s": rays / tb / 1e6, "per_frame_mrays_s": pr / tp / 1e6,
            "batched_path_samples_per_s": samples / tb,
            "identical_per_pixel": sums_batch == sums_plain and rays == pr,
            "tuned": {"block_threads": th.value, "blocks_per_sm": bps.value, "tiles_per_grab": grab.value},
            "timing": "wall clock around the blocking C-ABI calls, best of %d" % reps}


def adjoint_item(torch, dev, layout=2, reps=2):
    """The inversion workload: 16 views of a 1025^2 crater DEM, albedo texels and vertex heights as
    parameters; one forward (all views) and one backward (path-replay adjoint, all views)."""
    from vira_gb300 import workloads
    from vira_gb300.autograd import _apply_parameters, adjoint_views, forward_views

    scene, views = workloads.inversion(device=dev.index)
    scene.bvh_options.layout = layout
    mesh = scene.meshes[0]
    base_tex = mesh.albedo_map.copy()
    base_z = mesh.positions[:, 2].copy()
    rng = np.random.default_rng(4)
    tgt_tex = (base_tex * (1.0 + 0.05 * rng.standard_normal(base_tex.shape[:2]))[:, :, None]).astype(np.float32)
    tgt_z = (base_z + rng.normal(0.0, 0.5, base_z.shape)).astype(np.float32)
    _apply_parameters(scene, torch.tensor(tgt_tex), torch.tensor(tgt_z))
    targets = forward_views(scene, views, dev)
    _apply_parameters(scene, torch.tensor(base_tex), torch.tensor(base_z))
    imgs = forward_views(scene, views, dev)  # warm-up
    grads = [2.0 * (i - t) for i, t in zip(imgs, targets)]
    adjoint_views(scene, views, grads, dev)  # warm-up
    fw, bw = [], []
    for _ in range(reps):
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        imgs = forward_views(scene, views, dev)
        torch.cuda.synchronize(dev)
        fw.append(time.perf_counter() - t)
        grads = [2.0 * (i - t_) for i, t_ in zip(imgs, targets)]
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        gt, gz = adjoint_views(scene, views, grads, dev)
        torch.cuda.synchronize(dev)
        bw.append(time.perf_counter() - t)
    loss = float(sum(((i - t_) ** 2).double().sum() for i, t_ in zip(imgs, targets)))
    ntexel = base_tex.shape[0] * base_tex.shape[1]
    nz = base_z.shape[0]
    res = views[0].camera.resolution
    out = {"workload": f"inversion_dem{int(round(nz ** 0.5))}_tex{base_tex.shape[0]}_{len(views)}views_{res[0]}px_"
                       f"{scene.pathtracer.options.samples}spp_{scene.pathtracer.options.bounces}b_4band",
           "parameters": ntexel + nz, "texels": ntexel, "heights": nz,
           "forward_s": min(fw), "backward_s": min(bw), "backward_over_forward": min(bw) / min(fw),
           "backward_passes_per_s": 1.0 / min(bw), "loss": loss,
           "grad_norm": {"texture": float(gt.double().norm()), "heights": float(gz.double().norm())},
           "timing": "wall clock over all views (blocking C-ABI calls), best of %d" % reps}
    scene.close()
    return out


def bvh_item(torch, dev, scene, cam_id):
    """BVH build of the path-traced frame's 33.5M triangles: the host binned-SAH builder (all host
    threads) against the GPU linear BVH (builder 1), and one render of the frame with each tree
    (the closest hits are the same; the traversal work differs)."""
    from vira_gb300 import capi

    lib = capi.load()
    ctx = scene.context()
    out = {}
    for name, builder in (("host_sah", 0), ("gpu_lbvh", 1)):
        o = capi.BvhOptions(0, builder, 0, 2)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        capi.check(lib.vgb_bvh_build(ctx, C.byref(o)), ctx, "bvh_build")
        torch.cuda.synchronize(dev)
        build_s = time.perf_counter() - t0
        scene.pathtracer.render(scene[cam_id], scene)
        st = scene.pathtracer.last_stats
        out[name] = {"build_s": build_s, "nodes": int(st.bvh_nodes), "render_ms": float(st.ms_last),
                     "mrays_s": (st.rays_closest + st.rays_shadow) / (st.ms_last / 1e3) / 1e6}
    out["build_speedup"] = out["host_sah"]["build_s"] / out["gpu_lbvh"]["build_s"]
    out["timing"] = "wall clock around the blocking build call; render: CUDA events of one render"
    capi.check(lib.vgb_bvh_build(ctx, C.byref(capi.BvhOptions(0, 0, 0, 2))), ctx, "bvh_build")
    return out


def raster_item(torch, dev, scene, cam_id, hbm_peak, reps=5, cpu=True):
    """The rasterizer (vgb_rasterize, CPURasterizer::render) with lighting on the path-traced
    frame's scene (33.5M triangles, 2048^2, 8 bands) and on the direct-lighting scene (0.52M
    triangles, 1024^2, 4 bands); the oracle's sequential restatement times the latter on one
    host core.  Unique bytes: per triangle its 3 indices and 3 vertex records (60 B), per pixel
    the 8-byte fragment key, the solid angle and the written planes (depth, alpha, triangle id,
    normal: 24 B; albedo, total, direct, indirect radiance and power: 20 B per band)."""

    def unique(ntri, npix, nb):
        return 60.0 * ntri + (8 + 4 + 24 + 20 * nb) * float(npix)
    from vira_gb300 import workloads

    def timed(sc, cid):
        rz = sc.rasterizer
        rz.render_passes.simulate_lighting = True
        rz.render(sc[cid], sc)        # warm-up (scratch, solid angles)
        ms = []
        for _ in range(reps):
            rz.render(sc[cid], sc)
            ms.append(rz.last_stats.ms_last)
        return min(ms), rz.render_passes

    out = {}
    ms, rp = timed(scene, cam_id)
    W, H = scene[cam_id].resolution
    ntri = int(scene.flat["indices"].shape[0])
    gbs = unique(ntri, W * H, scene.bands.size) / (ms / 1e3) / 1e9
    out["path_traced_scene"] = {"triangles": ntri, "image": [W, H], "bands": scene.bands.size, "ms": ms,
                                "mtris_per_s": ntri / ms / 1e3,
                                "covered_pixels": int(torch.isfinite(rp.depth).sum().item()),
                                "unique_gb_s": gbs, "frac_of_hbm": gbs / hbm_peak}
    small, cid = workloads.plain_direct(device=dev.index)
    ms2, rp2 = timed(small, cid)
    ntri2 = int(small.flat["indices"].shape[0])
    W2, H2 = small[cid].resolution
    item = {"triangles": ntri2, "image": [W2, H2], "bands": small.bands.size, "ms": ms2,
            "mtris_per_s": ntri2 / ms2 / 1e3}
    if cpu:
        from oracle import oracle

        B = small.bands.size
        c = small[cid].to_c(small.origin, B)
        lights, nl = small.c_lights()
        omega = small.pixel_solid_angle(small[cid], c).cpu().numpy()
        osc = oracle.OracleScene.from_flat(small.flat, B)
        t0 = time.perf_counter()
        osc.rasterize(c, small[cid].intrinsic_matrix(), lights, nl, True, small.smooth_shading(), omega)
        cs = time.perf_counter() - t0
        osc.close()
        item["cpu_baseline"] = {"value": ntri2 / cs / 1e6, "unit": "Mtris/s", "cores": 1, "kind": "port",
                                "sample": f"the whole frame ({cs:.2f} s): the oracle's sequential CPURasterizer"}
        item["speedup_over_cpu"] = cs * 1e3 / ms2
    out["plain_direct_scene"] = item
    out["timing"] = "CUDA events around the three raster kernels on the context stream, best of %d" % reps
    small.close()
    return out


def quipu_item(torch, dev, hbm_peak, reps=3, cpu=True):
    """DEM ingestion from a Quipu file: a 4097^2 crater DEM at 1 m posts (uint16 heights, grey
    uint8 albedo, LZ4 blocks) with a 1025^2 LoD, read into a device mesh (positions, indices,
    8-band vertex albedo, vertex normals) by vgb_quipu_read_mesh -- DEMQuipu::readBuffers and
    Mesh::init -- against the oracle's CPU restatement of the same steps on the same file."""
    import shutil
    import tempfile

    from vira_gb300 import capi, synthetic
    from vira_gb300 import quipu as VQ
    from vira_gb300.scene import _mesh_context

    n, nb = 4097, 8
    z = synthetic.fbm_heights(n, 0.8, seed=21, lo=-200.0, hi=200.0)
    z = np.ascontiguousarray(synthetic.add_crater_field(z, 1.0, seed=22, dmin=20, dmax=2000), np.float32)
    alb = synthetic.lognormal_albedo(n, 0.12, 0.3, seed=23)
    dem = VQ.DEM(z, VQ.DEMProjection(n, n, (1.0, 1.0)), alb, VQ.FLOAT_IMAGE_ALBEDO)
    tmp = Path(tempfile.mkdtemp())
    try:
        t0 = time.perf_counter()
        VQ.DEMQuipu.write(tmp / "dem", [dem, dem.downsample(4)], options=VQ.DEMQuipuWriterOptions(compress=True))
        write_s = time.perf_counter() - t0
        path = tmp / "dem.qld"
        fbytes = path.stat().st_size
        q = VQ.DEMQuipu(path, nbands=nb)
        q.read_lod_mesh(0, gpu=dev.index, nbands=nb, device_arrays=True)      # warm-up, pinned staging
        lib = capi.load()
        ctx = _mesh_context(dev.index)
        e2e, dev_ms = [], []
        for _ in range(reps):
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            out = q.read_lod_mesh(0, gpu=dev.index, nbands=nb, device_arrays=True)
            torch.cuda.synchronize(dev)
            e2e.append(time.perf_counter() - t0)
            st = capi.Stats()
            capi.check(lib.vgb_get_stats(ctx, C.byref(st)), ctx, "stats")
            dev_ms.append(st.ms_last)
            del out
        t0 = time.perf_counter()
        q.read_heights(0)
        host_decode_s = time.perf_counter() - t0
        info = q.lods[0]
        posts, quads = n * n, (n - 1) * (n - 1)
        # unique bytes of the device phase: codes 2 + albedo code 1 in; heights 4 (written, read
        # back), positions 12, albedo 4 nb, normals 12 per post and 2 x 12 index bytes per quad out
        uniq = posts * (2 + 1 + 4 + 12 + 4 * nb + 12) + quads * 24
        best_dev = min(dev_ms)
        line = {"workload": f"quipu_dem{n}_u16_lz4_grey_albedo_{nb}band_2lods",
                "file_mb": fbytes / 1e6, "precision": VQ.PRECISION[info.precision], "write_s": write_s,
                "e2e_ms": 1e3 * min(e2e), "device_ms": best_dev, "host_read_decode_ms": 1e3 * host_decode_s,
                "mposts_per_s_e2e": posts / min(e2e) / 1e6,
                "device_unique_gb_s": uniq / (best_dev / 1e3) / 1e9,
                "device_frac_of_hbm": uniq / (best_dev / 1e3) / 1e9 / hbm_peak,
                "timing": "wall clock around the blocking call (file in page cache) / CUDA events around the "
                          "device phase, best of %d" % reps}
        if cpu:
            from oracle import oracle
            from oracle import quipu as Q

            t0 = time.perf_counter()
            o = Q.read(path)
            L = o.lods[0]
            h = Q.heights(L)
            pos = Q.vertex_positions(h, L.projection)
            Q.vertex_albedo(L, h, nb)
            idx = Q.index_buffer(h)
            oracle.compute_normals(pos, idx)
            cs = time.perf_counter() - t0
            line["cpu_baseline"] = {"value": posts / cs / 1e6, "unit": "Mposts/s", "cores": 1, "kind": "port",
                                    "sample": f"the whole file ({cs:.1f} s): oracle LZ4 decode, fixed point, "
                                              "makeVertexBuffer, imageToIndexBuffer, calculateNormals"}
        q.close()
        return line
    finally:
        shutil.rmtree(tmp, ignore_errors=True)


def after_film_item(torch, dev, scene, cam_id, hbm_peak, reps=5):
    """The steps after the film on the path-traced frame (2048^2, 8 bands): the EATWT denoiser
    (vgb_denoise, 5 levels on direct and indirect), the 81x81 Gaussian PSF convolution of the
    received power and the sensor chain with photon, dark and readout noise.  CUDA events on the
    context's stream, best of `reps`."""
    from vira_gb300 import capi, sensor

    rp = scene.pathtracer.render(scene[cam_id], scene)
    lib = capi.load()
    ctx = scene.context()
    B, H, W = rp.direct_radiance.shape
    P = H * W
    stream = torch.cuda.Stream(device=dev)
    capi.check(lib.vgb_set_stream(ctx, C.c_void_p(stream.cuda_stream)), ctx, "set_stream")
    d0, i0 = rp.direct_radiance.clone(), rp.indirect_radiance.clone()
    d, i = torch.empty_like(d0), torch.empty_like(i0)

    def timed(fn):
        best = float("inf")
        for _ in range(reps + 1):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                e0.record(stream)
            fn()
            with torch.cuda.stream(stream):
                e1.record(stream)
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        return best

    def den():
        with torch.cuda.stream(stream):
            d.copy_(d0)
            i.copy_(i0)
        capi.check(lib.vgb_denoise(ctx, d.data_ptr(), i.data_ptr(), rp.albedo.data_ptr(), rp.depth.data_ptr(),
                                   rp.normal_global.data_ptr(), W, H, B, None, 1), ctx, "denoise")

    t_den = timed(den)
    kern = sensor.GaussianPSF(1.5).make_kernel(scene.bands, 81, 20)
    kt = torch.tensor(kern, device=dev)
    pw = rp.received_power.clone()

    def psf():
        capi.check(lib.vgb_psf_convolve(ctx, pw.data_ptr(), W, H, B, kt.data_ptr(), 81, 81, 1), ctx, "psf")

    t_psf = timed(psf)
    sm = sensor.SensorModel(simulate_photon_noise=True,
                            noise_model=sensor.NoiseModelConfig(dark_current=20.0, readout_noise_mean=1.0,
                                                                readout_noise_std=3.0))
    sc = sm.to_c(scene.bands)
    img = torch.empty((H, W), device=dev)

    def sen():
        capi.check(lib.vgb_sensor_simulate(ctx, rp.received_power.data_ptr(), W, H, B, C.byref(sc), img.data_ptr(), 1),
                   ctx, "sensor")

    t_sen = timed(sen)
    capi.check(lib.vgb_set_stream(ctx, None), ctx, "set_stream")
    # unique bytes: split reads 3 and writes 2 planes of B; each of 20 passes (5 levels x 2
    # directions x direct+indirect share one launch, so 10 launches) reads 2B + 4 and writes 2B
    # floats per pixel; merge reads 3B, writes 2B
    den_bytes = 4 * P * ((3 * B + 2 * B) + 10 * (2 * B + 4 + 2 * B) + (3 * B + 2 * B))
    psf_flops = 2.0 * 81 * 81 * B * P
    sen_bytes = 4 * P * (B + 1)
    return {"image": [W, H], "bands": B,
            "denoise": {"ms": t_den, "levels": 5, "unique_gb_s": den_bytes / (t_den / 1e3) / 1e9,
                        "frac_of_hbm": den_bytes / (t_den / 1e3) / 1e9 / hbm_peak},
            "psf_81x81": {"ms": t_psf, "tflop_s": psf_flops / (t_psf / 1e3) / 1e12,
                          "note": "FP32 multiply + add per tap (no FMA contraction, reference rounding); CUDA cores"},
            "sensor_with_noise": {"ms": t_sen, "unique_gb_s": sen_bytes / (t_sen / 1e3) / 1e9,
                                  "frac_of_hbm": sen_bytes / (t_sen / 1e3) / 1e9 / hbm_peak},
            "timing": "CUDA events on the context stream, best of %d" % reps}


def asteroid_item(torch, dev, layout=2, reps=2):
    """The batched-adjoint asteroid workload: 64 views of uneven size, per-vertex radial offsets as
    parameters (smooth shading), the fused forward + L2 loss + adjoint of all views in one
    persistent launch, against per-view forward renders followed by per-view adjoint launches."""
    from vira_gb300 import workloads
    from vira_gb300.autograd import _apply_positions, adjoint_views, forward_views, render_adjoint_batch

    t0 = time.perf_counter()
    scene, views, dirs = workloads.asteroid(device=dev.index)
    scene.bvh_options.layout = layout
    mesh = scene.meshes[0]
    base = torch.tensor(mesh.positions.copy())
    dr = torch.tensor(dirs)
    rng = np.random.default_rng(9)
    off = torch.tensor(rng.normal(0.0, 0.5, dirs.shape[0]), dtype=torch.float32)
    _apply_positions(scene, None, base + off[:, None] * dr)
    targets = forward_views(scene, views, dev)
    _apply_positions(scene, None, base)
    setup = time.perf_counter() - t0
    render_adjoint_batch(scene, views, targets, dev, want_texture=False)  # warm-up
    fused, sep = [], []
    loss = 0.0
    gp = None
    for _ in range(reps):
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        loss, _, _, gp = render_adjoint_batch(scene, views, targets, dev, want_texture=False, keep_radiance=False)
        torch.cuda.synchronize(dev)
        fused.append(time.perf_counter() - t)
    for _ in range(reps):
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        imgs = forward_views(scene, views, dev)
        grads = [2.0 * (i - t_) for i, t_ in zip(imgs, targets)]
        adjoint_views(scene, views, grads, dev, want_texture=False, want_heights=True, positions=True)
        torch.cuda.synchronize(dev)
        sep.append(time.perf_counter() - t)
    # applying one optimizer step's offsets: device vertices + normals + BVH refit, against the
    # re-upload and host SAH rebuild the scene does when it is flattened again
    from vira_gb300 import capi

    lib = capi.load()
    ctx = scene.context()
    moved = (base + off[:, None] * dr).to(dev).contiguous()
    refit = []
    for k in range(reps + 1):
        src = moved if k % 2 == 0 else base.to(dev).contiguous()
        torch.cuda.synchronize(dev)
        t = time.perf_counter()
        capi.check(lib.vgb_scene_update_positions(ctx, capi.ptr(src), None, 1), ctx, "scene_update_positions")
        refit.append(time.perf_counter() - t)
    t = time.perf_counter()
    scene.mark_dirty()
    scene.build_tlas()
    rebuild = time.perf_counter() - t
    g_off = (gp.cpu() * dr).sum(dim=1)
    pix = sum(v.camera.resolution[0] * v.camera.resolution[1] for v in views)
    out = {"workload": f"asteroid_ico9_{mesh.indices.shape[0]}tris_{len(views)}views_256-1024px_"
                       f"{scene.pathtracer.options.samples}spp_4band_smooth",
           "parameters": int(dirs.shape[0]), "pixels": int(pix), "loss": loss,
           "fused_s": min(fused), "per_view_forward_plus_adjoint_s": min(sep),
           "speedup_over_per_view": min(sep) / min(fused), "gradient_evaluations_per_s": 1.0 / min(fused),
           "grad_norm_radial": float(g_off.double().norm()), "setup_s": setup,
           "parameter_update": {"device_refit_ms": 1e3 * min(refit[1:]), "host_rebuild_s": rebuild,
                                "note": "vertices + normals + BVH refit on the device vs flatten, upload and SAH build"},
           "timing": "wall clock around the blocking C-ABI calls, best of %d" % reps}
    scene.close()
    return out


def plain_direct_item(torch, dev, layout=2, cpu_seconds=0.0):
    """The 513^2 / 1024^2 direct-lighting frame: Mrays/s (primary + shadow) on the same GPU."""
    from vira_gb300 import capi, workloads

    scene, cam_id = workloads.plain_direct(device=dev.index)
    scene.bvh_options.layout = layout
    scene.build_tlas()
    stream = torch.cuda.Stream(device=dev)
    r = Renderer(scene, cam_id, torch, stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(5):
        r.render()
    ms, rays, trav_ms = [], 0, 0.0
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for it in range(40):
        # even renders: the frame time; odd renders: per-launch events for the traversal kernels
        prof = it % 2 == 1
        r.lib.vgb_set_profiling(r.ctx, 1 if prof else 0)
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
            ev0.record(stream)
        r.render()
        with torch.cuda.stream(stream):
            ev1.record(stream)
        ev1.synchronize()
        st = r.stats()
        if prof:
            trav_ms += st.ms_trace + st.ms_shadow
        else:
            ms.append(ev0.elapsed_time(ev1))
            rays += st.rays_closest + st.rays_shadow
    r.lib.vgb_set_profiling(r.ctx, 0)
    # algorithmic bytes of the same frame (counting pass: nodes x 64 B + triangles x 48 B)
    lib = r.lib
    capi.check(lib.vgb_set_count_pass(r.ctx, 1), r.ctx, "count_pass")
    r.render()
    cst = r.stats()
    capi.check(lib.vgb_set_count_pass(r.ctx, 0), r.ctx, "count_pass")
    alg = int(cst.nodes_visited) * int(cst.bvh_node_bytes) + int(cst.tris_tested) * int(cst.tri_record_bytes)
    tot = sum(ms)
    l2 = l2_peak(lib, r.ctx)
    trav_gbs = alg / (trav_ms / len(ms) / 1000.0) / 1e9
    out = {"workload": "plain_direct_dem513_1024px_1spp_4band", "mrays_s": rays / (tot / 1000.0) / 1e6,
           "ms_per_frame": tot / len(ms), "rays_per_frame": rays / len(ms),
           "roofline": {"bound": "l2", "kernels": "k_trace + k_shadow", "achieved": trav_gbs, "peak": l2, "unit": "GB/s",
                        "frac": trav_gbs / l2, "traversal_ms_per_frame": trav_ms / len(ms),
                        "algorithmic_bytes_per_frame": alg,
                        "peak_source": "measured L2 read bandwidth (vgb_measure_l2_read, 64 MiB, same run)",
                        "note": "node + triangle bytes of the counting pass over the traversal kernels' time "
                                "(CUDA events per launch); the 0.52M-triangle BVH (17 MB nodes, 25 MB triangles) "
                                "is L2-resident"}}
    if cpu_seconds > 0:
        from oracle import oracle

        threads = oracle.nthreads()
        osc = oracle_scene(scene)
        c = cpu_sample(r.cam, r.lights, r.nl, r.opts, osc, cpu_seconds, threads, r.omega.cpu().numpy())
        osc.close()
        out["cpu_baseline"] = {"value": c["mrays_s"], "unit": "Mrays/s", "cores": threads, "kind": "port",
                               "sample": f"{c['passes']} passes over " + sample_text(r.cam, r.opts) +
                                         f"; {c['rays']} rays in {c['seconds']:.1f} s"}
    scene.close()
    return out


def profile_case(kind: str, scale: float, layout: int = 2):
    """Small cases of each kernel family for profiler captures (a few GB on the device at most):

      path [--scale S]  k_trace / k_shade / k_shadow / k_end_sample: the path-traced workload shrunk
                        by S (posts, texture, pixels; 4 spp), rendered twice
      batch             k_batch / k_batch_direct: 24 trajectory frames of 256^2-1024^2 at 1-16 spp
      adjoint [--scale] k_adjoint: 2 views of the inversion scene at 512^2 x S (crater DEM 1025^2 x S)
      after_film        k_dn_*, k_psf, k_sensor on a 1024^2 frame
      quipu             Quipu decode and DEM mesh kernels: a 2049^2 LoD read twice
      raster            k_raster_*: 8.4M triangles at 1024^2, 8 bands, twice
      lbvh              GPU BVH build of 8.4M triangles twice, then one refit
      l2                k_l2_read: the L2 read-bandwidth probe (64 MiB, 20 passes per launch)
    `layout` selects the BVH node layout of the path case (2 binary, 8 compressed 8-wide).
    """
    import torch

    from vira_gb300 import workloads

    if kind == "path":
        posts = int(4096 * scale) + 1
        scene, cam = workloads.path_traced(posts=posts, tex=int(4096 * scale), resolution=int(2048 * scale), spp=4)
        scene.bvh_options.layout = layout
        for _ in range(2):
            scene.pathtracer.render(scene[cam], scene)
        torch.cuda.synchronize()
        print("path", scene.pathtracer.last_stats.ms_last, "ms")
    elif kind == "l2":
        from vira_gb300 import capi

        import ctypes

        lib = capi.load()
        ctx = ctypes.c_void_p()
        capi.check(lib.vgb_context_create(ctypes.byref(ctx), 0), None, "context_create")
        print("l2 GB/s", l2_peak(lib, ctx))
        lib.vgb_context_destroy(ctx)
    elif kind == "batch":
        scene, frames = workloads.trajectory(nframes=24, resolutions=(256, 512, 1024), spps=(1, 4, 16))
        for _ in range(2):
            scene.render_batch(frames, autotune=False, use_graph=False)
        torch.cuda.synchronize()
        print("batch", scene.pathtracer.last_stats.ms_last, "ms")
    elif kind == "adjoint":
        from vira_gb300.autograd import adjoint_views, forward_views

        posts = int(1024 * scale) + 1
        scene, views = workloads.inversion(posts=posts, tex=max(2, posts - 1), resolution=max(8, int(512 * scale)),
                                           nviews=2, spp=4)
        dev = torch.device("cuda", 0)
        imgs = forward_views(scene, views, dev)
        gt, gz = adjoint_views(scene, views, [torch.ones_like(i) for i in imgs], dev)
        torch.cuda.synchronize()
        print("adjoint", float(gt.abs().sum()))
    elif kind == "after_film":
        from vira_gb300 import sensor

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

        from vira_gb300 import quipu, synthetic

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

        from vira_gb300 import capi

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
        raise SystemExit(f"unknown profile case {kind!r}")


def main():
    args = parse()
    if args.profile_case:
        profile_case(args.profile_case, args.scale if args.scale != 1.0 else (1.0 if args.profile_case == "adjoint" else 0.25),
                     args.layout)
        return
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    p = workload_params(args)
    if world > 1:
        import torch
        import torch.distributed as dist

        if args.impl == "reference":
            if rank != 0:
                return
        else:
            torch.cuda.set_device(local_rank)
            dist.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, p, rank, world)
        return
    run_ours(args, p, rank, world, local_rank)
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
