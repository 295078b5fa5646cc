"""Spectral band layouts and the band-integrated black-body spectrum.

Mirrors ``SpectralData<N, spec, Lam...>`` band metadata
(include/implementation/spectral_data.ipp:65-132): band edges are given in nm and stored in
FP32 metres (``edge * 1e-9f``), the centre wavelength is the FP32 midpoint, and
``blackBodyRadiance`` (spectral_data.ipp:613-629, math.ipp:34-59) integrates Planck's law
over each band in FP64 with the trapezoid rule, returning FP32 values.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

SPEED_OF_LIGHT = 299792458.0
PLANCK_CONSTANT = 6.62607015e-34
BOLTZMANN_CONSTANT = 1.380649e-23
SOLAR_RADIUS = np.float32(696000000.0)
AU_TO_M = 149597870700.0


@dataclass(frozen=True)
class SpectralBands:
    """Band edges in metres, FP32, as the reference stores them."""

    min_wavelength: np.ndarray
    max_wavelength: np.ndarray

    @property
    def size(self) -> int:
        return int(self.min_wavelength.shape[0])

    @property
    def wavelengths(self) -> np.ndarray:
        return ((self.min_wavelength + self.max_wavelength) / np.float32(2.0)).astype(np.float32)

    @staticmethod
    def bounds(pairs_nm) -> "SpectralBands":
        """``SpectralData<N, BOUNDS, lo0, hi0, lo1, hi1, ...>``."""
        lo, hi = [], []
        for a, b in pairs_nm:
            a, b = np.float32(a), np.float32(b)
            lo.append(min(a, b))
            hi.append(max(a, b))
        f = np.float32(1e-9)
        return SpectralBands(np.array(lo, np.float32) * f, np.array(hi, np.float32) * f)

    @staticmethod
    def uniform(n: int, lo_nm: float, hi_nm: float) -> "SpectralBands":
        """``UniformSpectralData<N, lo, hi>`` (linspaceArray<float, N+1>, math.ipp:22-31)."""
        lo_f, hi_f = np.float32(lo_nm), np.float32(hi_nm)
        step = np.float32((hi_f - lo_f) / np.float32(n))
        edges = np.array([np.float32(lo_f + np.float32(np.float32(i) * step)) for i in range(n + 1)], np.float32)
        f = np.float32(1e-9)
        lo = np.minimum(edges[:-1], edges[1:]) * f
        hi = np.maximum(edges[:-1], edges[1:]) * f
        return SpectralBands(lo.astype(np.float32), hi.astype(np.float32))


def planck(temperature: float, wavelength: np.ndarray) -> np.ndarray:
    c, h, kb = SPEED_OF_LIGHT, PLANCK_CONSTANT, BOLTZMANN_CONSTANT
    lam = np.asarray(wavelength, np.float64)
    coeff = 2 * h * c * c / np.power(lam, 5.0)
    return coeff * 1.0 / (np.exp(h * c / (lam * kb * temperature)) - 1.0)


def black_body_radiance(bands: SpectralBands, temperature: float, steps: int = 1000) -> np.ndarray:
    """Band-integrated spectral radiance (W m^-2 sr^-1) per band, FP32."""
    out = np.zeros(bands.size, np.float32)
    for i in range(bands.size):
        mn = float(bands.min_wavelength[i])
        mx = float(bands.max_wavelength[i])
        step = (mx - mn) / float(steps - 1)
        lam = mn + np.arange(steps, dtype=np.float64) * step
        rad = planck(temperature, lam)
        dx = lam[1:] - lam[:-1]
        area = 0.0
        for a, b, d in zip(rad[:-1], rad[1:], dx):  # sequential sum, as the reference loop
            area += d * (a + b) / 2.0
        out[i] = np.float32(area)
    return out


# the band layouts the benchmark configurations name
FOUR_BAND = SpectralBands.bounds([(400, 500), (500, 600), (600, 700), (800, 900)])   # centres 450/550/650/850
EIGHT_BAND = SpectralBands.uniform(8, 400, 1000)
