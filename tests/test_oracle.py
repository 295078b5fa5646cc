"""The oracle (CPU restatement of Vira's path tracer) against known answers.

The reference ships no golden vectors for this path and cannot be built here, so the oracle
is pinned by (a) published known-answer vectors of its RNG, (b) closed-form answers derived
from the reference's formulas, (c) brute force, and (d) the committed fixtures of
tests/golden/ (test_golden.py).
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from oracle import oracle
from vira_gb300 import FOUR_BAND, capi, spectral, synthetic, workloads
from helpers import primary_rays

F = np.float32


def test_philox_known_answers():
    # Random123 philox4x32-10 known-answer vectors (Salmon et al., SC 2011)
    assert [hex(x) for x in oracle.philox([0, 0, 0, 0], [0, 0])] == ["0x6627e8d5", "0xe169c58d", "0xbc57ac4c", "0x9b00dbd8"]
    assert [hex(x) for x in oracle.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2)] == [
        "0x408f276d", "0x41c83b0e", "0xa20bc7c6", "0x6d5451fd"]
    assert [hex(x) for x in oracle.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])] == [
        "0xd16cfe09", "0x94fdcceb", "0x5001e420", "0x24126ea1"]


def test_blackbody_band_integral():
    bands = spectral.FOUR_BAND
    for T in (5778.0, 5800.0):
        prod = spectral.black_body_radiance(bands, T, 1000)
        for i in range(bands.size):
            lo, hi = float(bands.min_wavelength[i]), float(bands.max_wavelength[i])
            o = oracle.blackbody_band(T, bands.min_wavelength[i], bands.max_wavelength[i], 1000)
            assert abs(prod[i] - o) <= 1e-6 * o
            lam = np.linspace(lo, hi, 200001)
            fine = np.trapezoid(spectral.planck(T, lam), lam)
            assert abs(o - fine) <= 2e-6 * fine
    # Stefan-Boltzmann check of the Planck implementation over a wide band
    lam = np.linspace(50e-9, 200e-6, 2_000_001)
    tot = np.trapezoid(spectral.planck(5778.0, lam), lam)
    assert abs(tot * math.pi - 5.670374419e-8 * 5778.0 ** 4) / (5.670374419e-8 * 5778.0 ** 4) < 2e-3


def test_band_layouts():
    c = spectral.FOUR_BAND.wavelengths * 1e9
    assert np.allclose(c, [450, 550, 650, 850], atol=1e-3)
    e = spectral.EIGHT_BAND
    assert e.size == 8
    # FP32 edges, as SpectralData stores them: edge_nm * 1e-9f
    assert e.min_wavelength[0] == F(400) * F(1e-9) and e.max_wavelength[-1] == F(1000) * F(1e-9)


def _flat_scene(posts=33, extent=2000.0, res=48, sun_el=35.0, albedo=0.12):
    from vira_gb300 import FOUR_BAND, Mesh, Scene

    h = np.zeros((posts, posts), F)
    scene = Scene(FOUR_BAND)
    mid = scene.add_mesh(Mesh.from_dem(h, extent / (posts - 1), albedo=albedo, nbands=4))
    scene.new_instance(mid)
    sun = scene.new_sun(5778.0)
    scene.set_sun_direction(sun, 0.0, sun_el)
    cam_id = scene.new_camera()
    cam = scene[cam_id]
    cam.set_resolution(res, res)
    cam.set_sensor_size(0.036)
    cam.set_field_of_view(20.0)
    cam.set_local_position(0.0, 0.0, 3000.0)
    cam.look_in_direction((0.0, 0.0, -1.0), up=(0.0, 1.0, 0.0))
    scene.pathtracer.options.deterministic_light = True
    scene.pathtracer.render_passes.simulate_lighting = True
    return scene, cam_id


def test_flat_plane_known_answer():
    """radiance = albedo/pi * cos^2(theta) * L * Omega_fp32 * MIS weight (double-cosine quirk,
    lambertian.ipp:14 and cpu_path_tracer.ipp:416,425), Omega in FP32 (sphere_light.ipp:60)."""
    sun_el = 35.0
    scene, cam_id = _flat_scene(sun_el=sun_el)
    scene.flatten()
    from helpers import oracle_render

    o, _ = oracle_render(scene, cam_id)
    L = scene.lights[0]
    d = F(np.linalg.norm((L.position - scene.origin).astype(F).astype(np.float64)))
    r2 = F(L.radius * L.radius)
    omega = F(F(2) * F(math.pi)) * (F(1) - F(np.sqrt(F(d * d) - r2)) / d)
    lpdf = F(1) / omega
    cos = math.sin(math.radians(sun_el))
    mpdf = cos / math.pi
    w = lpdf ** 2 / (lpdf ** 2 + mpdf ** 2)
    hit = o["triangle_id"] != capi.NO_HIT
    assert hit.all()
    for b in range(4):
        expect = 0.12 / math.pi * cos * cos * float(L.radiance[b]) * w / float(lpdf)
        got = o["total_radiance"][b]
        assert np.all(np.abs(got - expect) <= 2e-5 * expect), (b, got.min(), got.max(), expect)
    # the FP32 solid angle (sphere_light.ipp:60) loses digits to cancellation for the sun's tiny cap
    exact = 2 * math.pi * (1 - math.sqrt(1 - (float(L.radius) / float(d)) ** 2))
    assert abs(float(omega) - exact) / exact < 2e-2
    assert np.allclose(o["depth"][hit], o["depth"][hit], equal_nan=True)
    assert np.all(o["alpha"] == 1.0)


def test_normals_and_dem_restatement_match_product():
    rng = np.random.default_rng(3)
    h = rng.standard_normal((23, 19)).astype(F) * F(5)
    h[4, 7] = np.inf
    h[11, 2] = np.nan
    p_o, i_o = oracle.dem_triangulate(h, 2.5)
    from vira_gb300 import Mesh

    m = Mesh.from_dem(h, 2.5)
    assert np.array_equal(p_o.view(np.uint32), m.positions.view(np.uint32))
    assert np.array_equal(i_o, m.indices)
    # quad (0,0) of a 19-wide grid: {(0,1),(1,0),(0,0)} and {(1,0),(0,1),(1,1)}
    assert list(i_o[0]) == [19, 1, 0] and list(i_o[1]) == [1, 19, 20]
    fin = np.isfinite(p_o).all(axis=1)
    n_o = oracle.compute_normals(p_o, i_o)
    m.normals = None
    n_p = m.compute_normals()
    assert np.array_equal(n_o.view(np.uint32), n_p.view(np.uint32))
    ln = np.linalg.norm(n_o[fin], axis=1)
    assert np.all((np.abs(ln - 1) < 1e-6) | (ln == 0))


def test_intrinsics_restatement_matches_product():
    from vira_gb300 import Camera

    c = Camera()
    c.set_resolution(640, 480)
    c.set_sensor_size(0.0123)
    c.set_focal_length(0.031)
    k_p = c.kinv()
    k_o = oracle.intrinsics(c.focal_length, c.sensor_size[0], c.sensor_size[1], 640, 480)
    assert np.array_equal(k_p, k_o)
    fx = float(c.focal_length) * 640 / float(c.sensor_size[0])
    K = np.array([[fx, 0, 320], [0, fx, 240], [0, 0, 1.0]])
    Kinv = np.array([[k_o[0], k_o[2], k_o[4]], [k_o[1], k_o[3], k_o[5]], [0, 0, 1]], np.float64)
    assert np.allclose(Kinv @ K, np.eye(3), atol=1e-5)


def test_pixel_solid_angle_sums_to_the_frustum():
    scene, cam_id = workloads.plain_direct(posts=17, resolution=64)
    cam = scene[cam_id].to_c(scene.origin, 4)
    om = oracle.pixel_solid_angle(cam)
    a = math.atan(cam.kinv[0] * 32)
    assert abs(om.sum() - 4 * math.asin(math.sin(a) ** 2)) < 1e-5
    assert om.min() > 0 and om[32, 32] > om[0, 0]


def _brute_closest(o, d, pos, idx):
    v0, v1, v2 = pos[idx[:, 0]].astype(np.float64), pos[idx[:, 1]].astype(np.float64), pos[idx[:, 2]].astype(np.float64)
    e1, e2 = v1 - v0, v2 - v0
    best_t = np.full(o.shape[0], np.inf)
    best = np.full(o.shape[0], capi.NO_HIT, np.uint64)
    for r in range(o.shape[0]):
        p = np.cross(d[r], e2)
        det = np.einsum("ij,ij->i", e1, p)
        inv = 1.0 / np.where(det == 0, np.nan, det)
        tv = o[r] - v0
        u = np.einsum("ij,ij->i", tv, p) * inv
        q = np.cross(tv, e1)
        v = (q @ d[r]) * inv
        t = np.einsum("ij,ij->i", e2, q) * inv
        ok = (u >= 0) & (v >= 0) & (u + v <= 1) & (t > 0)
        if ok.any():
            k = np.nonzero(ok)[0][np.argmin(t[ok])]
            best_t[r], best[r] = t[k], k
    return best, best_t


def test_oracle_trace_matches_brute_force_and_interpolates():
    scene, cam_id = workloads.plain_direct(posts=33, resolution=40)
    f = scene.flatten()
    cam = scene[cam_id].to_c(scene.origin, 4)
    o, d = primary_rays(cam)
    osc = oracle.OracleScene.from_flat(f, 4)
    tri, t, w = osc.trace(o, d)
    bt, btt = _brute_closest(o.astype(np.float64), d.astype(np.float64), f["positions"], f["indices"])
    hit = tri != capi.NO_HIT
    agree = (tri.astype(np.uint64) == bt)
    assert agree.mean() > 0.99
    assert np.all(np.abs(t[hit & agree] - btt[hit & agree]) <= 1e-4 * btt[hit & agree])
    # Interaction::w interpolates {v1, v2, v0} to the hit point o + t d
    idx = f["indices"][tri[hit]]
    pos = f["positions"].astype(np.float64)
    P = w[hit, 0:1] * pos[idx[:, 1]] + w[hit, 1:2] * pos[idx[:, 2]] + w[hit, 2:3] * pos[idx[:, 0]]
    Q = o[hit] + t[hit, None] * d[hit]
    assert np.abs(P - Q).max() < 1e-2
    # occlusion agrees with the closest hit
    occ, _, _ = osc.trace(o, d, any_hit=True, tmax=np.where(hit, t * 1.0001, 1e9).astype(F))
    assert np.array_equal(occ != capi.NO_HIT, hit)
    osc.close()


def test_edge_grazing_rays_are_cracks_or_shared_edge_ties():
    scene, cam_id = workloads.plain_direct(posts=65, resolution=64)
    f = scene.flatten()
    cam = scene[cam_id].to_c(scene.origin, 4)
    o, d = primary_rays(cam)
    osc = oracle.OracleScene.from_flat(f, 4)
    tri, t, _ = osc.trace(o, d)
    tri_r, t_r, _ = osc.trace(o, d, mode=1)
    osc.close()
    idx = f["indices"]
    for b in np.nonzero(tri != tri_r)[0]:
        if tri_r[b] == capi.NO_HIT:
            continue
        assert len(set(idx[tri[b]]) & set(idx[tri_r[b]])) >= 2
        assert abs(t[b] - t_r[b]) <= 1e-5 * t[b]


def test_render_is_deterministic_and_thread_count_invariant():
    scene, cam_id = workloads.path_traced(posts=129, tex=128, resolution=24, spp=3, bounces=2, rr_depth=1)
    f = scene.flatten()
    cam = scene[cam_id].to_c(scene.origin, 8)
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    osc = oracle.OracleScene.from_flat(f, 8)
    a, ca = osc.render(cam, lights, nl, opts, threads=1)
    b, cb = osc.render(cam, lights, nl, opts, threads=5)
    # a row sample (every 5th row from 3, as the CPU baseline takes them) renders those rows
    # exactly as the whole frame does and leaves the others untouched
    c, cc = osc.render(cam, lights, nl, opts, rows=(3, 24, 5), threads=3)
    osc.close()
    assert ca == cb
    for k in a:
        assert np.array_equal(a[k].view(np.uint32), b[k].view(np.uint32)), k
        sel = [3, 8, 13, 18, 23]
        other = [j for j in range(24) if j not in sel]
        assert np.array_equal(a[k][..., sel, :].view(np.uint32), c[k][..., sel, :].view(np.uint32)), k
        assert np.all(c[k][..., other, :].view(np.uint32) == (0xFFFFFFFF if k == "triangle_id" else 0x7FC00000)), k
    assert 0 < cc[0] < ca[0]
    assert np.all(a["indirect_radiance"] >= -1e-6)
    assert a["indirect_radiance"].mean() > 0


def test_synthetic_generators():
    h1 = synthetic.fbm_heights(65, 0.8, seed=1)
    h2 = synthetic.fbm_heights(65, 0.8, seed=1)
    assert np.array_equal(h1, h2) and h1.dtype == np.float32
    assert abs(h1.min() + 200) < 1e-3 and abs(h1.max() - 200) < 1e-3
    hc = synthetic.add_crater_field(h1, 10.0, seed=2, dmin=20, dmax=200)
    assert not np.array_equal(hc, h1)
    d = synthetic.crater_diameters(100000, 20, 2000, -2.5, np.random.default_rng(0))
    assert d.min() >= 20 and d.max() <= 2000 and np.median(d) < 40
    a = synthetic.lognormal_albedo(256, 0.12, 0.3, seed=3)
    assert abs(np.median(a) - 0.12) < 0.005
    v, fcs = synthetic.icosphere(3)
    assert v.shape[0] == 10 * 4 ** 3 + 2 and fcs.shape[0] == 20 * 4 ** 3
    assert np.allclose(np.linalg.norm(v, axis=1), 1.0)
    n = synthetic.real_sh_noise(v, 8, seed=5)
    assert n.shape == (v.shape[0],) and np.isfinite(n).all() and n.std() > 0


def test_oracle_adjoint_albedo_euler_identity():
    """Direct lighting is linear (degree 1) in the albedo texels, so sum_t alb_t dI/dalb_t = I
    (Euler's theorem); with g = dL/dI the FP64 adjoint must satisfy sum alb * grad = sum g * I."""
    from helpers import oracle_render

    scene, cam_id = workloads.path_traced(posts=65, tex=32, resolution=24, spp=2, bounces=0, rr_depth=0, seed=5)
    f = scene.flatten()
    cam = scene[cam_id].to_c(scene.origin, 8)
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    osc = oracle.OracleScene.from_flat(f, 8)
    planes, _ = osc.render(cam, lights, nl, opts)
    I = planes["total_radiance"].astype(np.float64)
    g = np.random.default_rng(2).standard_normal(I.shape).astype(np.float32)
    gt, _ = osc.adjoint(cam, lights, nl, opts, g, tex_shape=f["texture"].shape)
    osc.close()
    lhs = float(np.sum(f["texture"].astype(np.float64) * gt))
    rhs = float(np.sum(g.astype(np.float64) * I))
    assert abs(lhs - rhs) <= 1e-5 * abs(rhs)


def test_oracle_adjoint_heights_translation_invariance():
    """Moving every vertex up by the same amount does not change face normals, and hit points
    slide along with the surface: the sum of the normal terms of each triangle vanishes."""
    scene, cam_id = workloads.path_traced(posts=33, tex=32, resolution=16, spp=1, bounces=0, rr_depth=0, seed=6)
    scene.meshes[0].albedo_map = None  # uniform albedo: only the normal terms remain
    f = scene.flatten()
    cam = scene[cam_id].to_c(scene.origin, 8)
    lights, nl = scene.c_lights()
    opts = scene.pathtracer.c_options(scene)
    osc = oracle.OracleScene.from_flat(f, 8)
    g = np.ones((8, 16, 16), np.float32)
    _, gz = osc.adjoint(cam, lights, nl, opts, g, nverts=f["positions"].shape[0])
    osc.close()
    assert np.abs(gz).max() > 0
    assert abs(gz.sum()) <= 1e-9 * np.abs(gz).sum() + 1e-12


def test_oracle_position_adjoint_translation_invariance():
    """With uniform albedo and flat shading, translating every vertex by one vector changes no
    face normal, and a hit point sliding within its triangle keeps its normal: the position
    gradients of every triangle, and so their sum, vanish in each axis.  (With smooth shading the
    sliding hit point changes its interpolated normal, so there is no such invariance.)"""
    for smooth in (False,):
        scene, cam_id = workloads.path_traced(posts=33, tex=32, resolution=16, spp=1, bounces=0, rr_depth=0, seed=6)
        scene.meshes[0].albedo_map = None
        scene.meshes[0].set_smooth_shading(smooth)
        f = scene.flatten()
        cam = scene[cam_id].to_c(scene.origin, 8)
        lights, nl = scene.c_lights()
        opts = scene.pathtracer.c_options(scene)
        osc = oracle.OracleScene.from_flat(f, 8)
        g = np.ones((8, 16, 16), np.float32)
        _, gp = osc.adjoint_positions(cam, lights, nl, opts, g, nverts=f["positions"].shape[0])
        _, gz = osc.adjoint(cam, lights, nl, opts, g, nverts=f["positions"].shape[0])
        osc.close()
        assert np.abs(gp).max() > 0
        assert np.all(np.abs(gp.sum(axis=0)) <= 1e-9 * np.abs(gp).sum(axis=0) + 1e-12)
        assert np.allclose(gz, gp[:, 2], rtol=0, atol=1e-12 * np.abs(gz).max())


def test_oracle_position_adjoint_matches_finite_differences():
    """The FP64 position adjoint of sum(g * I) against central differences of the oracle's FP32
    renders (step 2e-2 m) for flat and smooth shading; vertices whose step flips a shadow ray
    (visibility, excluded by design) are the rare outliers."""
    rng = np.random.default_rng(8)
    for smooth in (False, True):
        scene, cam_id = workloads.path_traced(posts=33, tex=32, resolution=24, spp=1, bounces=0, rr_depth=0, seed=7)
        scene.meshes[0].albedo_map = None
        scene.meshes[0].set_smooth_shading(smooth)
        f = scene.flatten()
        cam = scene[cam_id].to_c(scene.origin, 8)
        lights, nl = scene.c_lights()
        opts = scene.pathtracer.c_options(scene)
        g = rng.uniform(0.5, 1.5, (8, 24, 24)).astype(np.float32)
        osc = oracle.OracleScene.from_flat(f, 8)
        _, gp = osc.adjoint_positions(cam, lights, nl, opts, g, nverts=f["positions"].shape[0])
        osc.close()

        def loss(pos):
            ff = dict(f)
            ff["positions"] = pos
            ff["normals"] = oracle.compute_normals(pos, f["indices"])
            o = oracle.OracleScene.from_flat(ff, 8)
            planes, _ = o.render(cam, lights, nl, opts, threads=1)
            o.close()
            return float(np.sum(g.astype(np.float64) * planes["total_radiance"]))

        flat_g = np.abs(gp).ravel()
        cand = np.nonzero(flat_g > np.percentile(flat_g, 97))[0]
        pick = rng.choice(cand, size=min(8, len(cand)), replace=False)
        errs = []
        h = 2e-2
        for q in pick:
            v, a = divmod(int(q), 3)
            pp = f["positions"].copy()
            pp[v, a] += h
            lp = loss(pp)
            pp[v, a] -= 2 * h
            lm = loss(pp)
            fd = (lp - lm) / (2 * h)
            errs.append(abs(fd - gp[v, a]) / max(abs(fd), 1e-12))
        errs = np.array(errs)
        print("smooth" if smooth else "flat", "FD relative errors", np.round(errs, 5))
        assert np.median(errs) <= 2e-2 and np.mean(errs <= 5e-2) >= 0.6, (smooth, np.round(errs, 4))


def test_oracle_adaptive_sampling_rule():
    """cpu_path_tracer.ipp:198-226 restated: with a tolerance no interval can miss, every lit pixel
    stops at the first batch check (sample index = samples_per_batch) and is divided by that index,
    so its radiance is the sum of samples_per_batch + 1 samples over samples_per_batch; sky pixels
    stop at the first miss check."""
    from helpers import oracle_render

    scene, cam_id = workloads.plain_direct(posts=65, resolution=16)
    scene[cam_id].look_in_direction((0.454, 0.0, -0.891))
    opt = scene.pathtracer.options
    opt.samples = 7
    ref, _ = oracle_render(scene, cam_id)                 # fixed 7 samples
    opt.samples = 50
    opt.adaptive_sampling = True
    opt.samples_per_batch = 6
    opt.samples_to_detect_miss = 4
    opt.sampling_tolerance = 1e30
    ada, _ = oracle_render(scene, cam_id)
    lit = ref["alpha"] > 0
    sky = ref["alpha"] == 0
    assert lit.any() and sky.any()
    # lit: 7 samples summed, divided by 6 instead of 7
    assert np.allclose(ada["total_radiance"][:, lit], ref["total_radiance"][:, lit] * 7.0 / 6.0, rtol=2e-6, atol=0)
    assert np.allclose(ada["alpha"][lit], ref["alpha"][lit] * 7.0 / 6.0, rtol=1e-6)
    assert np.all(ada["alpha"][sky] == 0) and np.all(np.isinf(ada["depth"][sky]))
    # tolerance 0 with random light sampling: no early batch stop while the variance is positive
    opt.sampling_tolerance = 0.0
    opt.deterministic_light = False
    opt.samples = 13
    ada0, _ = oracle_render(scene, cam_id)
    opt.adaptive_sampling = False
    full, _ = oracle_render(scene, cam_id)
    assert np.array_equal(ada0["total_radiance"][:, lit], full["total_radiance"][:, lit])


def test_oracle_denoiser_properties():
    """EATWT restated: a constant illumination (direct = albedo * c) passes through unchanged,
    and per-pixel noise on a smooth surface loses most of its variance."""
    rng = np.random.default_rng(2)
    B, N = 4, 32
    alb = rng.uniform(0.05, 0.3, (B, N, N)).astype(np.float32)
    depth = np.full((N, N), 1000.0, np.float32) + rng.uniform(0, 1, (N, N)).astype(np.float32)
    normal = np.zeros((3, N, N), np.float32)
    normal[2] = 1.0
    d0 = (alb * 0.7).astype(np.float32)
    i0 = (alb * 0.1).astype(np.float32)
    d, i = oracle.denoise(d0, i0, alb, depth, normal)
    assert np.allclose(d, d0, rtol=1e-5) and np.allclose(i, i0, rtol=1e-5)
    noisy = (alb * (0.7 + 0.2 * rng.standard_normal((B, N, N)))).astype(np.float32)
    d, _ = oracle.denoise(noisy, i0, alb, depth, normal)
    assert np.std(d / alb) < 0.3 * np.std(noisy / alb)
    with pytest.raises(ValueError):
        oracle.denoise(noisy[:, :, :16], i0[:, :, :16], alb[:, :, :16], depth[:, :16], normal[:, :, :16])


def test_oracle_sensor_chain_and_psf():
    """Noise-free sensor chain: electrons are linear in the received power until the ADU clamp;
    the spatial PSF with a delta kernel is the identity and a box kernel sums neighbours."""
    from vira_gb300 import sensor

    e = sensor.photon_energies(FOUR_BAND)
    qe = sensor.default_qe(FOUR_BAND)
    p = np.zeros((4, 2, 3), np.float32)
    p[:, 0, 0] = 1e-16
    p[:, 0, 1] = 2e-16
    p[:, 1, 2] = 1.0  # saturates
    out = oracle.sensor(p, 0.01, e, qe, 0.333333, 255.0)
    assert out[0, 1] == pytest.approx(2 * out[0, 0], rel=1e-6) and 0 < out[0, 0] < 1
    assert out[1, 2] == 1.0 and out[1, 0] == 0.0
    img = np.random.default_rng(0).uniform(0, 1, (2, 7, 9)).astype(np.float32)
    delta = np.zeros((2, 3, 3), np.float32)
    delta[:, 1, 1] = 1.0
    assert np.array_equal(oracle.psf(img, delta), img)
    box = np.ones((2, 3, 3), np.float32)
    s = oracle.psf(img, box)
    assert s[0, 3, 4] == pytest.approx(img[0, 2:5, 3:6].sum(), rel=1e-6)
    assert s[1, 0, 0] == pytest.approx(img[1, 0:2, 0:2].sum(), rel=1e-6)


# ---------------------------------------------------------------- lens distortion
def _np_brown_delta(k, x, y):
    """BrownDistortion::computeDelta (brown_distortion.ipp:24-44) in numpy FP32, written from the
    .ipp's expressions left to right."""
    f = np.float32
    k = [f(v) for v in k]
    r = np.sqrt(x * x + y * y)
    r2 = r * r
    r4 = r2 * r2
    r6 = r2 * r2 * r2
    s = k[0] * r2 + k[1] * r4 + k[2] * r6
    tx = (f(2) * k[3] * x * y) + (k[4] * (r2 + f(2) * x * x))
    ty = (k[3] * (r2 + f(2) * y * y)) + (f(2) * k[4] * x * y)
    return s * x + tx, s * y + ty


def _distortion_camera(model, coeffs):
    from vira_gb300 import capi

    c = capi.Camera()
    c.distortion = model
    for i, v in enumerate(coeffs):
        c.distortion_coeffs[i] = v
    return c


def _points(n=4000, extent=0.4, seed=3):
    rng = np.random.default_rng(seed)
    return rng.uniform(-extent, extent, (n, 2)).astype(np.float32)


def test_distortion_models_round_trip_and_zero_is_identity():
    from oracle import oracle
    from vira_gb300 import capi

    p = _points()
    cases = {
        "brown": (capi.DISTORTION_BROWN, [-0.12, 0.03, -0.004, 2e-3, -1e-3]),
        "opencv": (capi.DISTORTION_OPENCV, [-0.1, 0.02, 0.0, 0.01, -0.002, 0.0, 1e-3, -2e-3, 1e-3, 0.0, -1e-3, 0.0]),
        "owen": (capi.DISTORTION_OWEN, [1e-3, -0.08, 2e-3, 0.01, 1e-3, -1e-3]),
    }
    for name, (model, coeffs) in cases.items():
        cam = _distortion_camera(model, coeffs)
        u = oracle.distortion(cam, p, inverse=True)
        back = oracle.distortion(cam, u, inverse=False)
        if model == capi.DISTORTION_OPENCV:
            # OpenCVDistortion::computeDelta is h - distort(h), the opposite sign of the other
            # models' delta, and undistort still steps u = h - delta(u): its fixed point is
            # u - h = distort(u) - u, not distort(u) = h.  Kept as the reference has it.
            assert float(np.abs((u - p) - (back - u)).max()) < 2e-6, name
        else:
            assert float(np.abs(back - p).max()) < 2e-6, name
        assert float(np.abs(u - p).max()) > 1e-4, name   # the model does move the points
        zero = _distortion_camera(model, [0.0] * len(coeffs))
        assert np.array_equal(oracle.distortion(zero, p, inverse=True), p), name
        assert np.array_equal(oracle.distortion(zero, p, inverse=False), p), name


def test_brown_restatement_matches_its_formula_bit_for_bit():
    """The oracle's Brown model against a numpy FP32 transcription of the reference's
    expression order: distort = h + delta(h); undistort = 20 steps of u = h - delta(u)."""
    from oracle import oracle
    from vira_gb300 import capi

    k = [-0.12, 0.03, -0.004, 2e-3, -1e-3]
    cam = _distortion_camera(capi.DISTORTION_BROWN, k)
    p = _points(500)
    x, y = p[:, 0], p[:, 1]
    dx, dy = _np_brown_delta(k, x, y)
    d = np.stack([x + dx, y + dy], 1)
    assert np.array_equal(oracle.distortion(cam, p, inverse=False), d)
    ux, uy = x.copy(), y.copy()
    for _ in range(20):
        dx, dy = _np_brown_delta(k, ux, uy)
        ux, uy = x - dx, y - dy
    assert np.array_equal(oracle.distortion(cam, p, inverse=True), np.stack([ux, uy], 1))


def test_distortion_changes_the_pixel_solid_angle_consistently():
    """Barrel distortion (k1 < 0 in undistort's direction) spreads the outer pixels' rays: the
    frame's total solid angle grows, the centre pixel's barely moves."""
    from oracle import oracle
    from vira_gb300 import Camera, capi

    cam = Camera()
    cam.set_resolution(64, 48)
    cam.set_sensor_size(0.036)
    cam.set_field_of_view(40.0)
    c0 = cam.to_c(np.zeros(3), 4, kinv=oracle.camera_kinv(cam))
    cam.set_brown_distortion_coefficients(k1=-0.15)
    c1 = cam.to_c(np.zeros(3), 4, kinv=oracle.camera_kinv(cam))
    assert c1.distortion == capi.DISTORTION_BROWN and c1.interpolate_directions == 1
    o0, o1 = oracle.pixel_solid_angle(c0), oracle.pixel_solid_angle(c1)
    assert o1.sum() > o0.sum() * 1.01
    assert abs(float(o1[24, 32] / o0[24, 32]) - 1.0) < 1e-3


def test_rgb_conversion_restatements_agree():
    """spectralToRGB (integrateOver per ColorRGB band / bandwidth) in numpy FP32 against the
    oracle's C restatement, through a noise-free RGB sensor with unit gain and photon energy."""
    from oracle import oracle
    from vira_gb300 import sensor
    from vira_gb300.spectral import EIGHT_BAND, FOUR_BAND

    rng = np.random.default_rng(2)
    rb = sensor.rgb_bands()
    for bands in (FOUR_BAND, EIGHT_BAND):
        v = rng.uniform(0.0, 3.0, (bands.size, 2, 3)).astype(np.float32)
        ones = np.ones(3, np.float32)
        got = oracle.sensor_rgb(v, bands.min_wavelength, bands.max_wavelength, rb.min_wavelength, rb.max_wavelength,
                                (rb.max_wavelength - rb.min_wavelength).astype(np.float32), ones, ones, 1.0, 1.0, 1.0)
        for y in range(2):
            for x in range(3):
                assert np.array_equal(got[:, y, x], sensor.spectral_to_rgb(bands, v[:, y, x]))
    # a flat spectrum over 400-1000 nm: R and G fully covered (value 1), B covered from 400 nm only
    flat = sensor.spectral_to_rgb(EIGHT_BAND, np.ones(8, np.float32))
    assert abs(flat[0] - 1) < 1e-6 and abs(flat[1] - 1) < 1e-6 and abs(flat[2] - 100.0 / 120.0) < 1e-6
    qe = sensor.spectral_to_rgb(FOUR_BAND, sensor.default_qe(FOUR_BAND))
    assert np.all(qe > 0) and qe[0] < qe[2]   # higher photon energy at the blue end
