"""The sensor chain after the film, with the reference's names.

``PhotositeConfig`` (cameras/photosites/photosite.hpp:19-45), ``NoiseModelConfig``
(cameras/noise_models/noise_model.hpp:16-25), ``GaussianPSF`` and ``AiryDiskPSF``
(cameras/psfs/{gaussian_psf,airy_disk}.ipp) with ``make_kernel`` restating
PointSpreadFunction::makeKernel (psfs/psf.ipp:15-58), and ``simulate_sensor`` /
``psf_convolve`` over the C ABI (vgb_sensor_simulate, vgb_psf_convolve).  Kernel tables are
built once on the host, like the reference's; the per-pixel work runs on the GPU.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import capi

PLANCK = np.float32(6.62607015e-34)     # math.hpp:35
LIGHT_SPEED = np.float32(299792458.0)   # math.hpp:32


def photon_energies(bands) -> np.ndarray:
    """TSpectral::photonEnergies: PhotonEnergy<float>(centre wavelength) = h c / lambda in FP32
    (spectral_data.ipp:125-128, math.ipp:11-14)."""
    lam = bands.wavelengths
    return ((PLANCK * LIGHT_SPEED) / lam).astype(np.float32)


def default_qe(bands) -> np.ndarray:
    """PhotositeConfig::defaultQE (photosite.ipp:64-79): 0.5 * E_k / mean(E) in FP32."""
    e = photon_energies(bands)
    n = np.float32(e.shape[0])
    total = np.float32(0.0)
    for v in e:
        total = np.float32(total + np.float32(v / n))
    return np.array([np.float32(np.float32(0.5) * v / total) for v in e], np.float32)


# ColorRGB (spectral_data.hpp:205): SpectralData<3, BOUNDS, 600, 750, 500, 600, 380, 500>
RGB_BANDS_NM = ((600.0, 750.0), (500.0, 600.0), (380.0, 500.0))


def rgb_bands():
    from .spectral import SpectralBands

    return SpectralBands.bounds(RGB_BANDS_NM)


def integrate_over(bands, values, min_lam, max_lam) -> np.float32:
    """SpectralData::integrateOver (spectral_data.ipp:306-333) in FP32."""
    f = np.float32
    lo, hi = f(min_lam), f(max_lam)
    if lo > hi:
        lo, hi = hi, lo
    if lo == hi:
        return f(0.0)
    integral = f(0.0)
    for bmin, bmax, v in zip(bands.min_wavelength, bands.max_wavelength, values):
        if bmin > hi or bmax < lo:
            continue
        b1 = max(f(bmin), lo)
        b2 = min(f(bmax), hi)
        integral = f(integral + f(f(b2 - b1) * f(v)))
    return integral


def spectral_to_rgb(bands, values) -> np.ndarray:
    """spectralToRGB_val (spectral_data.ipp:588-605): per ColorRGB band, integrateOver / bandwidth."""
    rb = rgb_bands()
    out = []
    for k in range(3):
        lo, hi = rb.min_wavelength[k], rb.max_wavelength[k]
        out.append(np.float32(integrate_over(bands, values, lo, hi) / np.float32(hi - lo)))
    return np.array(out, np.float32)


@dataclass
class PhotositeConfig:
    bit_depth: int = 8
    well_depth: int = 15000
    gain: float = 0.333333
    unity_gain_db: float = 0.0
    quantum_efficiency: np.ndarray | None = None   # default_qe(bands) when None
    linear_scale_factor: float = 1.0
    # RGB quantum efficiency (PhotositeConfig::quantum_efficiency_rgb); None: the constructor's
    # default, spectralToRGB of the default spectral QE (photosite.ipp:84-94) -- a spectral QE set
    # later does not change it, as in the reference
    quantum_efficiency_rgb: np.ndarray | None = None

    def set_gain_db(self, gain_db: float, new_unity_gain_db: float = 0.0):
        """PhotositeConfig::setGainDB (photosite.ipp:34-38)."""
        self.unity_gain_db = float(np.float32(new_unity_gain_db))
        self.gain = float(np.float32(10.0) ** ((np.float32(gain_db) - np.float32(self.unity_gain_db)) / np.float32(20.0)))

    def max_adu(self) -> float:
        """Photosite::Photosite (photosite.ipp:99-103): linear_scale * (2^bits - 1)."""
        return float(np.float32(self.linear_scale_factor) * (np.float32(2.0) ** np.float32(self.bit_depth) - np.float32(1.0)))


@dataclass
class NoiseModelConfig:
    dark_current: float = 0.0
    readout_noise_mean: float = 0.0
    readout_noise_std: float = 0.0
    horizontal_scale: float = 0.0
    vertical_scale: float = 0.0
    horizontal_pattern_period: int = 0
    vertical_pattern_period: int = 0


class PointSpreadFunction:
    supersample_step = 1

    def evaluate(self, dx: np.ndarray, dy: np.ndarray, bands) -> np.ndarray:
        raise NotImplementedError

    def make_kernel(self, bands, kernel_size: int = 81, supersample_factor: int = 20) -> np.ndarray:
        """PointSpreadFunction::makeKernel (psf.ipp:15-58): the PSF averaged over a
        supersample_factor^2 grid inside each kernel pixel (sub-samples summed in the reference's
        order), centred.  Returns [B][k][k] FP32 indexed [band][y][x].  The render uses the largest
        default kernel (81, psf.hpp:55, taken by getKernel(., 0) at cpu_path_tracer.ipp:154-158),
        built with factor 20 (psf.ipp:96)."""
        if kernel_size % 2 == 0 or kernel_size <= 2:
            raise ValueError("Kernel must have an odd resolution >= 3")
        s = int(supersample_factor) or self.supersample_step
        c = np.float32((kernel_size - 1.0) / 2.0)
        idx = np.arange(kernel_size, dtype=np.float32)
        acc = np.zeros((bands.size, kernel_size, kernel_size), np.float32)
        for si in range(s):
            ox = np.float32((np.float32(si) + np.float32(0.5)) / np.float32(s))
            for sj in range(s):
                oy = np.float32((np.float32(sj) + np.float32(0.5)) / np.float32(s))
                sx = (idx + ox - np.float32(0.5)).astype(np.float32) - c      # per kernel column
                sy = (idx + oy - np.float32(0.5)).astype(np.float32) - c      # per kernel row
                dx = np.broadcast_to(sx[None, :], (kernel_size, kernel_size)).ravel()
                dy = np.broadcast_to(sy[:, None], (kernel_size, kernel_size)).ravel()
                v = self.evaluate(dx.astype(np.float32), dy.astype(np.float32), bands)
                acc = (acc + v.reshape(bands.size, kernel_size, kernel_size)).astype(np.float32)
        return (acc / np.float32(s * s)).astype(np.float32)


class GaussianPSF(PointSpreadFunction):
    """GaussianPSF (gaussian_psf.ipp:13-90): a rotated anisotropic Gaussian, per band sigmas in pixels."""

    def __init__(self, sigma_x, sigma_y=None, angle_deg: float = 0.0):
        self.sigma_x = np.asarray(sigma_x, np.float32)
        self.sigma_y = np.asarray(sigma_x if sigma_y is None else sigma_y, np.float32)
        a = np.float32(math.pi / 180.0) * np.float32(angle_deg)
        ca, sa = np.float32(math.cos(a)), np.float32(math.sin(a))
        self.rot = np.array([[ca, -sa], [sa, ca]], np.float32)   # rotation_ * point

    def evaluate(self, dx, dy, bands):
        x = (self.rot[0, 0] * dx + self.rot[0, 1] * dy).astype(np.float32)
        y = (self.rot[1, 0] * dx + self.rot[1, 1] * dy).astype(np.float32)
        sx = np.broadcast_to(self.sigma_x, (bands.size,)).astype(np.float32)[:, None]
        sy = np.broadcast_to(self.sigma_y, (bands.size,)).astype(np.float32)[:, None]
        xn, yn = (x[None, :] / sx).astype(np.float32), (y[None, :] / sy).astype(np.float32)
        expo = (np.float32(-0.5) * (xn * xn + yn * yn)).astype(np.float32)
        coef = (np.float32(1.0) / (np.float32(2.0 * math.pi) * sx * sy)).astype(np.float32)
        return (coef * np.exp(expo)).astype(np.float32)


class AiryDiskPSF(PointSpreadFunction):
    """AiryDiskPSF (airy_disk.ipp:14-60): (2 J1(x)/x)^2 with x = pi D/f r / lambda, r the physical
    radius on the sensor, FP64 Bessel (scipy.special.j1), unnormalised as in the reference."""

    supersample_step = 10

    def __init__(self, focal_length: float, aperture_diameter: float, pixel_size):
        self.coef = math.pi * float(np.float32(aperture_diameter) / np.float32(focal_length))
        self.pixel_size = np.asarray(pixel_size, np.float32).reshape(2)

    def evaluate(self, dx, dy, bands):
        from scipy.special import j1

        r = np.hypot((dx * self.pixel_size[0]).astype(np.float64), (dy * self.pixel_size[1]).astype(np.float64))
        lam = bands.wavelengths.astype(np.float64)[:, None]
        x = self.coef * r[None, :] / lam
        with np.errstate(invalid="ignore", divide="ignore"):
            v = np.where(r[None, :] < 1e-20, 1.0, 2.0 * j1(x) / x).astype(np.float32)
        return (v * v).astype(np.float32)


@dataclass
class SensorModel:
    """The camera's sensor settings (Camera members, camera.hpp:215-268)."""

    exposure_time: float = 0.01
    photosite: PhotositeConfig = field(default_factory=PhotositeConfig)
    noise_model: NoiseModelConfig | None = None
    simulate_photon_noise: bool = False
    filter_mosaic: object = None      # [B][H][W] (numpy or torch) or None
    psf: PointSpreadFunction | None = None
    psf_kernel_size: int = 81
    seed: int = 0

    def to_c(self, bands, frame: int = 0) -> capi.Sensor:
        s = capi.Sensor()
        s.exposure_time = float(np.float32(self.exposure_time))
        e = photon_energies(bands)
        qe = self.photosite.quantum_efficiency
        qe = default_qe(bands) if qe is None else np.broadcast_to(np.asarray(qe, np.float32), (bands.size,))
        for k in range(bands.size):
            s.photon_energy[k] = float(e[k])
            s.quantum_efficiency[k] = float(qe[k])
        s.gain = float(np.float32(self.photosite.gain))
        s.max_adu = self.photosite.max_adu()
        s.simulate_photon_noise = int(bool(self.simulate_photon_noise))
        nm = self.noise_model
        if nm is not None:
            s.noise_model = 1
            s.dark_current, s.readout_noise_mean, s.readout_noise_std = nm.dark_current, nm.readout_noise_mean, nm.readout_noise_std
            s.horizontal_scale, s.vertical_scale = nm.horizontal_scale, nm.vertical_scale
            s.horizontal_pattern_period, s.vertical_pattern_period = nm.horizontal_pattern_period, nm.vertical_pattern_period
        s.seed, s.frame = int(self.seed), int(frame)
        return s


def simulate_sensor(scene, received_power, sensor: SensorModel, frame: int = 0):
    """Camera::simulateSensor on a torch CUDA [B][H][W] received-power plane: returns [H][W]."""
    import torch

    lib = capi.load()
    ctx = scene.context()
    B, H, W = received_power.shape
    img = torch.empty((H, W), dtype=torch.float32, device=received_power.device)
    s = sensor.to_c(scene.bands, frame)
    mos = None
    if sensor.filter_mosaic is not None:
        mos = torch.as_tensor(sensor.filter_mosaic, dtype=torch.float32, device=received_power.device).contiguous()
        s.filter_mosaic = mos.data_ptr()
    p = received_power.contiguous()
    torch.cuda.current_stream(received_power.device).synchronize()
    capi.check(lib.vgb_sensor_simulate(ctx, p.data_ptr(), W, H, B, C.byref(s), img.data_ptr(), 1), ctx, "sensor_simulate")
    return img


def rgb_conversion(bands, sensor: SensorModel) -> capi.RgbConversion:
    """The constants of vgb_sensor_simulate_rgb for the scene's bands and this sensor."""
    c = capi.RgbConversion()
    for k in range(bands.size):
        c.band_min[k] = float(bands.min_wavelength[k])
        c.band_max[k] = float(bands.max_wavelength[k])
    rb = rgb_bands()
    pe = photon_energies(rb)
    qe = sensor.photosite.quantum_efficiency_rgb
    qe = spectral_to_rgb(bands, default_qe(bands)) if qe is None else np.asarray(qe, np.float32).reshape(3)
    for k in range(3):
        c.rgb_min[k] = float(rb.min_wavelength[k])
        c.rgb_max[k] = float(rb.max_wavelength[k])
        c.rgb_bandwidth[k] = float(np.float32(rb.max_wavelength[k] - rb.min_wavelength[k]))
        c.rgb_photon_energy[k] = float(pe[k])
        c.rgb_quantum_efficiency[k] = float(qe[k])
    return c


def simulate_sensor_rgb(scene, received_power, sensor: SensorModel, frame: int = 0):
    """Camera::simulateSensorRGB on a torch CUDA [B][H][W] received-power plane: returns [3][H][W]
    (R, G, B), not clamped (the reference's RGB photosite does not clamp)."""
    import torch

    lib = capi.load()
    ctx = scene.context()
    B, H, W = received_power.shape
    img = torch.empty((3, H, W), dtype=torch.float32, device=received_power.device)
    s = sensor.to_c(scene.bands, frame)
    rgb = rgb_conversion(scene.bands, sensor)
    mos = None
    if sensor.filter_mosaic is not None:
        mos = torch.as_tensor(sensor.filter_mosaic, dtype=torch.float32, device=received_power.device).contiguous()
        s.filter_mosaic = mos.data_ptr()
    p = received_power.contiguous()
    torch.cuda.current_stream(received_power.device).synchronize()
    capi.check(lib.vgb_sensor_simulate_rgb(ctx, p.data_ptr(), W, H, B, C.byref(s), C.byref(rgb), img.data_ptr(), 1),
               ctx, "sensor_simulate_rgb")
    return img


def psf_convolve(scene, received_power, kernel: np.ndarray):
    """Image::convolve of the received power (in place) with a [B][k][k] kernel."""
    import torch

    lib = capi.load()
    ctx = scene.context()
    B, H, W = received_power.shape
    k = torch.as_tensor(np.ascontiguousarray(kernel, np.float32), device=received_power.device)
    torch.cuda.current_stream(received_power.device).synchronize()
    capi.check(lib.vgb_psf_convolve(ctx, received_power.data_ptr(), W, H, B, k.data_ptr(), k.shape[2], k.shape[1], 1),
               ctx, "psf_convolve")
    return received_power
