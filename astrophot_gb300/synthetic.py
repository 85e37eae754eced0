"""Seeded synthetic workloads (no dataset exists for this path).

Parameter draws follow the single-Sersic stamp distributions used by the
benchmarks: centre at the stamp middle + U(-1, 1) px, n ~ U(0.5, 4),
Re ~ U(5, 20) px, q ~ U(0.3, 1) (open at 1: ``q = 1`` is rejected by the
parameter limits), PA ~ U(0, pi), log10 Ie ~ U(0, 2), a flat sky, and a
Moffat PSF (beta 3.5) built like ``moffat_psf`` in
``astrophot/utils/initialize/construct_psf.py:38-65``.

Initial guesses are the truth perturbed by 10 %:
  centre  + U(-1, 1) px per axis (additive: 10 % of a 64 px offset would
          leave the galaxy),
  q, n, Re x (1 + 0.1 U(-1, 1)), clipped inside the parameter limits,
  PA      + 0.1 pi U(-1, 1), wrapped into [0, pi),
  log10 Ie + 0.1 U(-1, 1).
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List

import numpy as np

SERSIC_KEYS = ("cx", "cy", "q", "PA", "n", "Re", "Ie")


def moffat_rd(fwhm: float, beta: float) -> float:
    """Moffat core radius for a given FWHM."""
    return fwhm / (2.0 * math.sqrt(2.0 ** (1.0 / beta) - 1.0))


def moffat_stamp(beta: float, rd: float, width: int, pixelscale: float = 1.0, upsample: int = 4) -> np.ndarray:
    """4x4 super-sampled, normalised Moffat stamp (construct_psf.py:38-65)."""
    if width % 2 != 1:
        raise ValueError("psf images should have an odd shape")
    N = width * upsample
    g = np.linspace(-(N - 1) * pixelscale / (2 * upsample), (N - 1) * pixelscale / (2 * upsample), N)
    XX, YY = np.meshgrid(g, g)
    ZZ = 1.0 / (1.0 + (XX**2 + YY**2) / (rd**2)) ** beta
    ZZ = ZZ.reshape(width, upsample, width, upsample).sum(axis=(1, 3)) / (upsample**2)
    return ZZ / np.sum(ZZ)


def gaussian_stamp(sigma: float, width: int, pixelscale: float = 1.0, upsample: int = 4) -> np.ndarray:
    """4x4 super-sampled, normalised Gaussian stamp (construct_psf.py:8-35)."""
    if width % 2 != 1:
        raise ValueError("psf images should have an odd shape")
    N = width * upsample
    g = np.linspace(-(N - 1) * pixelscale / (2 * upsample), (N - 1) * pixelscale / (2 * upsample), N)
    XX, YY = np.meshgrid(g, g)
    ZZ = np.exp(-0.5 * (XX**2 + YY**2) / sigma**2)
    ZZ = ZZ.reshape(width, upsample, width, upsample).sum(axis=(1, 3)) / (upsample**2)
    return ZZ / np.sum(ZZ)


def draw_sersic(rng: np.random.Generator, nx: int, ny: int) -> np.ndarray:
    """[cx, cy, q, PA, n, Re, Ie] (value space) for one stamp of nx x ny pixels, scale 1."""
    cx = nx / 2 + rng.uniform(-1, 1)
    cy = ny / 2 + rng.uniform(-1, 1)
    n = rng.uniform(0.5, 4.0)
    Re = rng.uniform(5.0, 20.0)
    q = rng.uniform(0.3, 1.0)
    while q >= 0.999:
        q = rng.uniform(0.3, 1.0)
    PA = rng.uniform(0.0, math.pi)
    Ie = rng.uniform(0.0, 2.0)
    return np.array([cx, cy, q, PA, n, Re, Ie])


def perturb_sersic(rng: np.random.Generator, truth: np.ndarray) -> np.ndarray:
    """10 % perturbation of a truth vector, rule stated in the module docstring."""
    cx, cy, q, PA, n, Re, Ie = truth
    u = rng.uniform(-1, 1, size=7)
    return np.array(
        [
            cx + u[0],
            cy + u[1],
            float(np.clip(q * (1 + 0.1 * u[2]), 0.05, 0.95)),
            float(np.mod(PA + 0.1 * math.pi * u[3], math.pi)),
            float(np.clip(n * (1 + 0.1 * u[4]), 0.4, 7.5)),
            Re * (1 + 0.1 * u[5]),
            Ie + 0.1 * u[6],
        ]
    )


@dataclass
class StampSpec:
    nx: int
    ny: int
    truth: np.ndarray  # value space [cx, cy, q, PA, n, Re, Ie]
    init: np.ndarray
    psf: np.ndarray
    sky: float  # flat sky level per pixel (locked)
    seed: int


def c0_stamp(seed: int, size: int = 128, fwhm: float = 3.0, beta: float = 3.5, psf_width: int = 25) -> StampSpec:
    """One 128 x 128 single-Sersic stamp with a 25 x 25 Moffat (FWHM 3, beta 3.5) and sky 1."""
    rng = np.random.default_rng(seed)
    truth = draw_sersic(rng, size, size)
    init = perturb_sersic(rng, truth)
    psf = moffat_stamp(beta, moffat_rd(fwhm, beta), psf_width)
    return StampSpec(size, size, truth, init, psf, 1.0, seed)


def cutout_stamps(count: int, seed: int, lo: int = 32, hi: int = 256, beta: float = 3.5) -> List[StampSpec]:
    """Batched-cutout workload: side ~ round(log-uniform(lo, hi)), one Sersic + a flat sky,
    Moffat FWHM ~ U(2, 5) px with side = 4 FWHM rounded to odd."""
    rng = np.random.default_rng(seed)
    out = []
    for s in range(count):
        side = int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))
        truth = draw_sersic(rng, side, side)
        init = perturb_sersic(rng, truth)
        fwhm = rng.uniform(2.0, 5.0)
        width = int(round(4 * fwhm))
        if width % 2 == 0:
            width += 1
        psf = moffat_stamp(beta, moffat_rd(fwhm, beta), width)
        out.append(StampSpec(side, side, truth, init, psf, 1.0, seed * 1_000_003 + s))
    return out


def add_noise(model: np.ndarray, seed: int, floor: float = 10.0):
    """Gaussian noise sigma = sqrt(model + floor); returns (data, weight = 1/(model + floor))."""
    rng = np.random.default_rng(seed + 7919)
    var = model + floor
    data = model + rng.normal(size=model.shape) * np.sqrt(var)
    return data, 1.0 / var


def crowded_field(seed: int, size: int = 1024, n_sources: int = 200, psf_sigma: float = 2.0, psf_width: int = 51,
                  sky: float = 5.0):
    """Crowded field: ``n_sources`` Sersic galaxies with uniform centres on a ``size``^2 image,
    the other parameters from the C0 distributions (Re truncated to 30 px), a ``psf_width``^2
    Gaussian PSF (sigma ``psf_sigma``), a flat sky; each galaxy gets an explicit square pixel
    window of half-size 4 Re + 3 sigma + 2 (clipped to the image).  Returns (truth [n, 7],
    init [n, 7] = truth perturbed 10 %, windows, psf)."""
    rng = np.random.default_rng(seed)
    truth, init, windows = [], [], []
    for _ in range(n_sources):
        t = draw_sersic(rng, size, size)
        t[0] = rng.uniform(0.0, size)
        t[1] = rng.uniform(0.0, size)
        t[5] = min(t[5], 30.0)
        truth.append(t)
        init.append(perturb_sersic(rng, t))
        h = int(math.ceil(4 * t[5] + 3 * psf_sigma + 2))
        x0, x1 = max(0, int(t[0]) - h), min(size, int(t[0]) + h + 1)
        y0, y1 = max(0, int(t[1]) - h), min(size, int(t[1]) + h + 1)
        windows.append(((x0, x1), (y0, y1)))
    psf = gaussian_stamp(psf_sigma, psf_width)
    return np.array(truth), np.array(init), windows, psf


def bulge_disk_field(seed: int, size: int = 2048, n_pairs: int = 500, fwhm: float = 3.0, beta: float = 3.5,
                     psf_width: int = 65):
    """Bulge + disk field: ``n_pairs`` galaxies with uniform centres on a ``size``^2 image, each a
    Sersic bulge (n ~ U(2, 6)) and an exponential disk sharing its centre, both with the other
    parameters from the single-stamp distributions; a ``psf_width``^2 Moffat PSF (FWHM ``fwhm``
    px, beta ``beta``); a square window of half-size 4 max(Re) + 2 FWHM + 2 px per pair (clipped
    to the image).  Initial values: the truth perturbed by 10 % (same rule as the stamps, the
    shared centre moved once).  Returns (truth [n, 11] = cx, cy, bulge q, PA, n, Re, Ie, disk q,
    PA, Re, Ie; init [n, 11]; windows; psf)."""
    rng = np.random.default_rng(seed)
    truth, init, windows = [], [], []
    for _ in range(n_pairs):
        b = draw_sersic(rng, size, size)
        b[0] = rng.uniform(0.0, size)
        b[1] = rng.uniform(0.0, size)
        b[4] = rng.uniform(2.0, 6.0)
        dsk = draw_sersic(rng, size, size)
        bi = perturb_sersic(rng, b)
        bi[4] = float(np.clip(b[4] * (1 + 0.1 * rng.uniform(-1, 1)), 0.4, 7.5))
        di = perturb_sersic(rng, dsk)
        truth.append(np.r_[b[:7], dsk[2], dsk[3], dsk[5], dsk[6]])
        init.append(np.r_[bi[:7], di[2], di[3], di[5], di[6]])
        h = int(math.ceil(4 * max(b[5], dsk[5]) + 2 * fwhm + 2))
        x0, x1 = max(0, int(b[0]) - h), min(size, int(b[0]) + h + 1)
        y0, y1 = max(0, int(b[1]) - h), min(size, int(b[1]) + h + 1)
        windows.append(((x0, x1), (y0, y1)))
    psf = moffat_stamp(beta, moffat_rd(fwhm, beta), psf_width)
    return np.array(truth), np.array(init), windows, psf


def bulge_disk_sources(rows, windows):
    """Scene sources (bulge, then its disk linked to the bulge's centre) of ``bulge_disk_field``
    rows."""
    from .scene import SceneSource

    out = []
    for k, (r, w) in enumerate(zip(rows, windows)):
        cx, cy, bq, bpa, bn, bre, bie, dq, dpa, dre, die = [float(v) for v in r]
        out.append(SceneSource("sersic", [cx, cy, bq, bpa, bn, bre, bie], w))
        out.append(SceneSource("exponential", [cx, cy, dq, dpa, 1.0, dre, die], w, link_center=2 * k))
    return out
