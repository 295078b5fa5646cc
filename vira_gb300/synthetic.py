"""Seeded synthetic scenes: fBm heightfields, crater fields, lognormal albedo maps,
icospheres with spherical-harmonic noise, and camera trajectories.

The reference ships no terrain generators (it reads GeoTIFF/SPC/Quipu files); these stand in
for real DEMs with the shapes, sizes and value distributions the benchmark configurations name.
All generators take an explicit seed and use numpy's PCG64 stream, so a scene is a pure
function of its parameters.
"""
from __future__ import annotations

import math

import numpy as np


def fbm_heights(n: int, hurst: float = 0.8, seed: int = 1, lo: float = -200.0, hi: float = 200.0) -> np.ndarray:
    """n x n heights [j][i] by spectral synthesis: PSD ~ k^-(2H+2), then scaled to [lo, hi].

    The field is synthesised on the next power-of-two periodic grid and wrapped, so an
    (2^m + 1)-post DEM costs one power-of-two FFT.
    """
    m = 1 << max(1, (n - 1).bit_length())
    if m < n - 1:
        m <<= 1
    rng = np.random.default_rng(seed)
    kx = np.fft.fftfreq(m)
    k = np.sqrt(kx[None, :] ** 2 + kx[:, None] ** 2)
    k[0, 0] = np.inf
    amp = k ** (-(hurst + 1.0))
    noise = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    field = np.fft.ifft2(noise * amp).real
    idx = np.arange(n) % m
    h = field[np.ix_(idx, idx)]
    h = (h - h.min()) / (h.max() - h.min())
    return (lo + (hi - lo) * h).astype(np.float32)


def crater_diameters(count: int, dmin: float, dmax: float, exponent: float, rng) -> np.ndarray:
    """Inverse-CDF samples of p(D) ~ D^exponent on [dmin, dmax] (exponent != -1)."""
    a = exponent + 1.0
    u = rng.random(count)
    return (dmin ** a + u * (dmax ** a - dmin ** a)) ** (1.0 / a)


def add_crater_field(heights: np.ndarray, posting: float, seed: int, dmin: float = 20.0, dmax: float = 2000.0,
                     exponent: float = -2.5, coverage: float = 0.3) -> np.ndarray:
    """Adds a Poisson field of craters: parabolic bowls of depth 0.2 D below the local
    surface with rims raised 0.04 D that fall off to zero at 1.5 R.  The expected crater
    count covers ``coverage`` of the area with bowls."""
    h = heights.astype(np.float64, copy=True)
    H, W = h.shape
    rng = np.random.default_rng(seed)
    area = (W - 1) * posting * (H - 1) * posting
    a = exponent
    # E[D^2] of the truncated power law
    e_d2 = ((dmax ** (a + 3) - dmin ** (a + 3)) / (a + 3)) / ((dmax ** (a + 1) - dmin ** (a + 1)) / (a + 1))
    count = rng.poisson(coverage * area / (math.pi / 4 * e_d2))
    diam = crater_diameters(count, dmin, dmax, exponent, rng)
    cx = rng.random(count) * (W - 1)
    cy = rng.random(count) * (H - 1)
    order = np.argsort(-diam)  # large first, small craters overprint
    for c in order:
        D = diam[c]
        R = D / 2.0 / posting
        ext = int(math.ceil(1.5 * R)) + 1
        x0, x1 = max(0, int(cx[c]) - ext), min(W, int(cx[c]) + ext + 1)
        y0, y1 = max(0, int(cy[c]) - ext), min(H, int(cy[c]) + ext + 1)
        if x0 >= x1 or y0 >= y1:
            continue
        yy, xx = np.mgrid[y0:y1, x0:x1]
        r = np.sqrt((xx - cx[c]) ** 2 + (yy - cy[c]) ** 2) / R
        depth, rim = 0.2 * D, 0.04 * D
        prof = np.where(r <= 1.0, rim - (rim + depth) * (1.0 - r * r),
                        np.where(r <= 1.5, rim * ((1.5 - r) / 0.5) ** 2, 0.0))
        h[y0:y1, x0:x1] += prof
    return h.astype(np.float32)


def lognormal_albedo(n: int, median: float = 0.12, sigma_log: float = 0.3, seed: int = 2) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return (median * np.exp(sigma_log * rng.standard_normal((n, n)))).astype(np.float32)


def grid_uvs(width: int, height: int, tex: int) -> np.ndarray:
    """Per-vertex UV = (i / tex, j / tex) for a (height x width) post grid, [j][i] order."""
    i = np.arange(width, dtype=np.float32) / np.float32(tex)
    j = np.arange(height, dtype=np.float32) / np.float32(tex)
    uv = np.empty((height, width, 2), np.float32)
    uv[:, :, 0] = i[None, :]
    uv[:, :, 1] = j[:, None]
    return uv.reshape(-1, 2)


def icosphere(subdivisions: int):
    """Unit icosphere: 20 * 4^s triangles, 10 * 4^s + 2 vertices (FP64 positions)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
         (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
         (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = np.array(v, np.float64)
    verts /= np.linalg.norm(verts, axis=1, keepdims=True)
    faces = np.array(f, np.int64)
    for _ in range(subdivisions):
        nv = verts.shape[0]
        e = np.concatenate([faces[:, [0, 1]], faces[:, [1, 2]], faces[:, [2, 0]]])
        e.sort(axis=1)
        key = e[:, 0] * (nv + 1) + e[:, 1]
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // (nv + 1), uniq % (nv + 1)
        mids = verts[a] + verts[b]
        mids /= np.linalg.norm(mids, axis=1, keepdims=True)
        verts = np.concatenate([verts, mids])
        m = inv.reshape(3, -1).T + nv  # mid of (0,1), (1,2), (2,0)
        v0, v1, v2 = faces[:, 0], faces[:, 1], faces[:, 2]
        m01, m12, m20 = m[:, 0], m[:, 1], m[:, 2]
        faces = np.concatenate([np.stack([v0, m01, m20], 1), np.stack([v1, m12, m01], 1),
                                np.stack([v2, m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return verts, faces.astype(np.uint32)


def real_sh_noise(dirs: np.ndarray, lmax: int, seed: int) -> np.ndarray:
    """Sum over 1 <= l <= lmax of random real spherical harmonics with amplitude ~ l^-2, evaluated
    at unit directions; uses the associated Legendre recurrence in FP64.  For each order m the
    l-sums of the cos(m phi) and sin(m phi) terms are formed first, so the azimuthal factors are
    evaluated once per m."""
    rng = np.random.default_rng(seed)
    x, y, z = dirs[:, 0], dirs[:, 1], dirs[:, 2]
    ct = np.clip(z, -1.0, 1.0)
    st = np.sqrt(np.maximum(0.0, 1 - ct * ct))
    phi = np.arctan2(y, x)
    out = np.zeros_like(x)
    cs = np.empty_like(x)
    sn = np.empty_like(x)
    tmp = np.empty_like(x)
    # P_m^m, then upward in l
    pmm = np.ones_like(x)
    for m in range(0, lmax + 1):
        if m > 0:
            pmm *= st
            pmm *= -(2 * m - 1)
        cs.fill(0.0)
        sn.fill(0.0)
        p_prev, p_cur = None, pmm
        for l in range(m, lmax + 1):
            if l == m:
                p = pmm
            elif l == m + 1:
                p = ct * ((2 * m + 1) * pmm)
            else:
                p = (ct * ((2 * l - 1) * p_cur) - (l + m - 1) * p_prev) / (l - m)
            if l > m:
                p_prev, p_cur = p_cur, p
            if l >= 1:
                norm = math.sqrt((2 * l + 1) / (4 * math.pi) * math.exp(math.lgamma(l - m + 1) - math.lgamma(l + m + 1)))
                amp = float(l) ** -2.0
                ca, sa = rng.standard_normal(2)
                np.multiply(p, amp * norm * ca, out=tmp)
                cs += tmp
                if m > 0:
                    np.multiply(p, amp * norm * sa, out=tmp)
                    sn += tmp
        if m == 0:
            out += cs
        else:
            out += math.sqrt(2) * (cs * np.cos(m * phi) + sn * np.sin(m * phi))
    return out
