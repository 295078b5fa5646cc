"""The sensor chain after the film (vgb_sensor_simulate, vgb_psf_convolve).

* Noise-free: photon counts, quantum efficiency, gain and ADU clamp equal the oracle's
  restatement of getPhotonCounts / exposePixel bit for bit, with and without a filter mosaic.
* PSF: the tiled convolution equals the oracle's restatement of Image::convolveSpatial bit for
  bit (3x3 to 81x81 kernels; the reference's FFT path for large kernels equals that sum up to
  rounding).
* Noise: the reference draws from std::mt19937, so the draws are checked by their statistics:
  Poisson photon counts below and above the sampler's switch (mean 3 and 60), Poisson dark current
  and Gaussian readout, against their means and variances over 2^20 pixels (5 sigma); the fixed
  pattern multiplies the noise as the reference's sinusoids.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from vira_gb300 import FOUR_BAND, capi, sensor, workloads

pytestmark = pytest.mark.gpu


def _ctx():
    import torch

    lib = capi.load()
    ctx = C.c_void_p()
    capi.check(lib.vgb_context_create(C.byref(ctx), 0), None, "context_create")
    torch.cuda.synchronize()
    return lib, ctx


def _simulate(lib, ctx, power, s):
    B, H, W = power.shape
    out = np.empty((H, W), np.float32)
    p = np.ascontiguousarray(power, np.float32)
    capi.check(lib.vgb_sensor_simulate(ctx, capi.ptr(p), W, H, B, C.byref(s), capi.ptr(out), 0), ctx, "sensor")
    return out


def _sensor(exposure=0.01, qe=None, gain=0.333333, max_adu=255.0, B=4):
    s = capi.Sensor()
    s.exposure_time = exposure
    e = sensor.photon_energies(FOUR_BAND)
    q = sensor.default_qe(FOUR_BAND) if qe is None else np.asarray(qe, np.float32)
    for k in range(B):
        s.photon_energy[k] = float(e[k])
        s.quantum_efficiency[k] = float(q[k])
    s.gain, s.max_adu = gain, max_adu
    return s


def test_noise_free_sensor_matches_oracle(gpu):
    from oracle import oracle

    lib, ctx = _ctx()
    rng = np.random.default_rng(0)
    power = (10 ** rng.uniform(-17, -13, (4, 64, 96))).astype(np.float32)
    s = _sensor()
    e = np.array(s.photon_energy[:4], np.float32)
    q = np.array(s.quantum_efficiency[:4], np.float32)
    g = _simulate(lib, ctx, power, s)
    o = oracle.sensor(power, 0.01, e, q, 0.333333, 255.0)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    assert (g == 1.0).any() and (g < 1.0).any()
    mosaic = rng.uniform(0, 1, power.shape).astype(np.float32)
    s.filter_mosaic = mosaic.ctypes.data
    g = _simulate(lib, ctx, power, s)
    o = oracle.sensor(power, 0.01, e, q, 0.333333, 255.0, mosaic=mosaic)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    lib.vgb_context_destroy(ctx)


@pytest.mark.parametrize("k", [3, 9, 27, 81])
def test_psf_convolution_matches_oracle(gpu, k):
    from oracle import oracle

    lib, ctx = _ctx()
    rng = np.random.default_rng(k)
    img = rng.uniform(0, 1, (4, 70, 53)).astype(np.float32)
    kern = sensor.GaussianPSF(np.array([0.8, 1.2, 1.6, 2.4], np.float32)).make_kernel(FOUR_BAND, k, 4)
    g = img.copy()
    capi.check(lib.vgb_psf_convolve(ctx, capi.ptr(g), 53, 70, 4, capi.ptr(kern), k, k, 0), ctx, "psf")
    o = oracle.psf(img, kern)
    assert np.array_equal(g.view(np.uint32), o.view(np.uint32))
    lib.vgb_context_destroy(ctx)


def _counts(lib, ctx, lam, B=1, n=1 << 20, **noise):
    """Sensor with QE 1, gain 1 and a huge ADU range: the output times max_adu is the count."""
    W = 1024
    H = n // W
    e = sensor.photon_energies(FOUR_BAND)
    s = capi.Sensor()
    s.exposure_time = 1.0
    s.photon_energy[0] = float(e[0])
    s.quantum_efficiency[0] = 1.0
    s.gain, s.max_adu = 1.0, 1e9
    s.simulate_photon_noise = 1
    s.seed, s.frame = 12345, 7
    for k, v in noise.items():
        setattr(s, k, v)
    power = np.full((1, H, W), lam * float(e[0]), np.float32)
    return _simulate(lib, ctx, power, s).astype(np.float64) * 1e9, s, power


@pytest.mark.parametrize("lam", [3.0, 60.0])
def test_photon_noise_is_poisson(gpu, lam):
    lib, ctx = _ctx()
    c, s, power = _counts(lib, ctx, lam)
    n = c.size
    assert np.allclose(c, np.rint(c), atol=1e-3 * max(1.0, lam))
    mean, var = c.mean(), c.var()
    assert abs(mean - lam) < 5 * np.sqrt(lam / n), mean
    assert abs(var - lam) < 5 * lam * np.sqrt(2.0 / n) + 5 * np.sqrt(lam / n), var
    # reproducible for a key, different for another frame
    c2 = _simulate(lib, ctx, power, s).astype(np.float64) * 1e9
    assert np.array_equal(c, c2)
    s.frame = 8
    c3 = _simulate(lib, ctx, power, s).astype(np.float64) * 1e9
    assert not np.array_equal(c, c3)
    lib.vgb_context_destroy(ctx)


def test_dark_current_readout_and_fixed_pattern(gpu):
    lib, ctx = _ctx()
    # no light: the counts are the noise model's electrons (dark Poisson(20) * 1 s + N(2, 3^2))
    c, s, power = _counts(lib, ctx, 0.0, noise_model=1, dark_current=20.0, readout_noise_mean=2.0,
                          readout_noise_std=3.0)
    n = c.size
    assert abs(c.mean() - 22.0) < 5 * np.sqrt(29.0 / n)
    assert abs(c.var() - 29.0) < 5 * 29.0 * np.sqrt(2.0 / n) * 1.5
    # fixed pattern: column i scales the noise by (1 - h) + h (1 + sin(2 pi i / (2 period)))
    s.horizontal_scale, s.horizontal_pattern_period = 0.5, 16
    s.readout_noise_std = 0.0
    s.dark_current = 0.0
    c = _simulate(lib, ctx, power, s).astype(np.float64) * 1e9
    i = np.arange(c.shape[1])
    expect = 2.0 * ((1 - 0.5) + 0.5 * (1 + np.sin(2 * np.pi * i / 32.0)))
    assert np.allclose(c[0], expect, rtol=1e-5, atol=1e-4)
    lib.vgb_context_destroy(ctx)


def test_pathtrace_render_returns_the_sensor_image(gpu):
    import torch

    from vira_gb300.sensor import simulate_sensor

    scene, cam_id = workloads.plain_direct(posts=65, resolution=48)
    cam = scene[cam_id]
    cam.sensor.psf = sensor.GaussianPSF(1.5)
    cam.sensor.psf_kernel_size = 9
    img = scene.pathtrace_render(cam_id)
    torch.cuda.synchronize()
    rp = scene.pathtracer.render_passes
    again = simulate_sensor(scene, rp.received_power, cam.sensor)
    assert img.shape == (48, 48) and torch.equal(img, again)
    assert float(img.max()) > 0
    scene.close()


def _rgb_sensor(bands, **kw):
    sm = sensor.SensorModel(**kw)
    return sm, sm.to_c(bands), sensor.rgb_conversion(bands, sm)


@pytest.mark.parametrize("mosaic", [False, True])
def test_rgb_sensor_noise_free_matches_oracle(gpu, mosaic):
    """Camera::simulateSensorRGB without noise: bit-identical to the oracle's restatement."""
    from oracle import oracle
    from vira_gb300.spectral import EIGHT_BAND

    lib, ctx = _ctx()
    rng = np.random.default_rng(5)
    B, H, W = 8, 37, 53
    power = rng.lognormal(-26.0, 1.0, (B, H, W)).astype(np.float32)
    sm, s, rgb = _rgb_sensor(EIGHT_BAND, exposure_time=0.02)
    mos = rng.uniform(0.0, 1.0, (B, H, W)).astype(np.float32) if mosaic else None
    if mos is not None:
        s.filter_mosaic = capi.ptr(mos)
    out = np.empty((3, H, W), np.float32)
    capi.check(lib.vgb_sensor_simulate_rgb(ctx, capi.ptr(power), W, H, B, C.byref(s), C.byref(rgb), capi.ptr(out), 0),
               ctx, "sensor_rgb")
    ref = oracle.sensor_rgb(power, EIGHT_BAND.min_wavelength, EIGHT_BAND.max_wavelength, rgb.rgb_min, rgb.rgb_max,
                            rgb.rgb_bandwidth, rgb.rgb_photon_energy, rgb.rgb_quantum_efficiency, s.exposure_time,
                            s.gain, s.max_adu, mosaic=mos)
    lib.vgb_context_destroy(ctx)
    assert np.array_equal(out.view(np.uint32), ref.view(np.uint32))
    assert out.max() > 0 and (out > 1).any() == (ref > 1).any()   # no clamp in the RGB photosite


def test_rgb_sensor_noise_moments(gpu):
    """Per-channel noise-model draws and Poisson photon counts: means and variances over 2^20
    pixels within 5 sigma of the models (dark current Poisson x exposure + Gaussian readout)."""
    from vira_gb300.spectral import FOUR_BAND

    lib, ctx = _ctx()
    H = W = 1024
    B = 4
    sm, s, rgb = _rgb_sensor(FOUR_BAND, exposure_time=1.0,
                             noise_model=sensor.NoiseModelConfig(dark_current=40.0, readout_noise_mean=2.0,
                                                                 readout_noise_std=3.0))
    s.gain = 1.0
    s.max_adu = 1.0
    for c in range(3):
        rgb.rgb_quantum_efficiency[c] = 1.0
    power = np.zeros((B, H, W), np.float32)
    out = np.empty((3, H, W), np.float32)
    capi.check(lib.vgb_sensor_simulate_rgb(ctx, capi.ptr(power), W, H, B, C.byref(s), C.byref(rgb), capi.ptr(out), 0),
               ctx, "sensor_rgb")
    lib.vgb_context_destroy(ctx)
    n = H * W
    mean, var = 40.0 + 2.0, 40.0 + 9.0
    for c in range(3):
        x = out[c].astype(np.float64)
        assert abs(x.mean() - mean) < 5 * np.sqrt(var / n), c
        assert abs(x.var() - var) < 5 * var * np.sqrt(2.0 / n) * 1.5, c
    # the three channels draw independently
    assert abs(np.corrcoef(out[0].ravel(), out[1].ravel())[0, 1]) < 0.01


def test_pathtrace_render_rgb(gpu):
    from oracle import oracle

    scene, cam_id = workloads.plain_direct(posts=65, resolution=48)
    cam = scene[cam_id]
    cam.sensor.exposure_time = 0.5
    rgb = scene.pathtrace_render_rgb(cam_id).cpu().numpy()
    power = scene.pathtracer.render_passes.received_power.cpu().numpy()
    c = sensor.rgb_conversion(scene.bands, cam.sensor)
    s = cam.sensor.to_c(scene.bands)
    ref = oracle.sensor_rgb(power, scene.bands.min_wavelength, scene.bands.max_wavelength, c.rgb_min, c.rgb_max,
                            c.rgb_bandwidth, c.rgb_photon_energy, c.rgb_quantum_efficiency, s.exposure_time, s.gain,
                            s.max_adu)
    scene.close()
    assert rgb.shape == (3, 48, 48)
    assert np.array_equal(rgb.view(np.uint32), ref.view(np.uint32))
    assert rgb.mean() > 0
