"""FP64 numpy restatement of the moments initialiser (``ap_moments_init``), test
infrastructure only: the checker of the kernel and the initial values of the CPU arm.

The reference's own initial values come from ``Galaxy_Model.initialize`` (centre of light,
``Angle_COM_PA``, isophote q; models/galaxy_model_object.py:60-113) and a Nelder-Mead fit of a
binned radial profile (models/_shared_methods.py:116-166); the library's fallback for the
learned proposal is this simpler moments estimate, restated here step by step.
"""

from __future__ import annotations

import math

import numpy as np

BINS = 64


def moments_init(data: np.ndarray, sky: float, sigma: float, sky_F: float = 0.0) -> np.ndarray:
    """[cx, cy, q, PA, n, Re, Ie, F] of one square stamp (pixel scale 1, pixel (i, j) centre at
    (i + 0.5, j + 0.5))."""
    d = np.asarray(data, dtype=np.float64)
    ny, nx = d.shape
    w = d - sky
    use = w > sigma
    yy, xx = np.mgrid[0:ny, 0:nx]
    x = xx + 0.5
    y = yy + 0.5
    S = np.sum(w[use])
    cx = np.sum((w * x)[use]) / S if S > 0 else nx / 2
    cy = np.sum((w * y)[use]) / S if S > 0 else ny / 2
    dx, dy = x - cx, y - cy
    Mxx = np.sum((w * dx * dx)[use])
    Myy = np.sum((w * dy * dy)[use])
    Mxy = np.sum((w * dx * dy)[use])
    tr, det = Mxx + Myy, Mxx * Myy - Mxy * Mxy
    disc = math.sqrt(max(tr * tr / 4 - det, 0.0))
    l1, l2 = tr / 2 + disc, max(tr / 2 - disc, 1e-12)
    q = math.sqrt(l2 / l1) if l1 > 0 else 0.7
    q = min(max(q, 0.1), 0.95)
    theta = 0.5 * math.atan2(2 * Mxy, Mxx - Myy)
    pa = math.fmod(theta + math.pi / 2 + 2 * math.pi, math.pi)
    # elliptical radius in the model's frame (major axis at PA - pi/2 from +x)
    ca, sa = math.cos(pa - math.pi / 2), math.sin(pa - math.pi / 2)
    u = dx * ca + dy * sa
    v = (-dx * sa + dy * ca) / q
    r = np.sqrt(u * u + v * v)
    rmax = 0.75 * nx
    k = np.minimum(BINS - 1, (r / rmax * BINS).astype(np.int64))
    hist_f = np.bincount(k.ravel(), weights=w.ravel(), minlength=BINS)
    hist_n = np.bincount(k.ravel(), minlength=BINS).astype(np.float64)
    tot = hist_f.sum()
    cum, re, kre = 0.0, 5.0, 0
    for i in range(BINS):
        prev = cum
        cum += hist_f[i]
        if tot > 0 and cum >= 0.5 * tot:
            frac = (0.5 * tot - prev) / hist_f[i] if hist_f[i] > 0 else 0.5
            re = (i + frac) * rmax / BINS
            kre = i
            break
    re = max(re, 1.0)
    ie = hist_f[kre] / hist_n[kre] if (hist_n[kre] > 0 and hist_f[kre] > 0) else max(tot, 1.0) / 1000.0
    return np.array([cx, cy, q, pa, 2.0, re, math.log10(max(ie, 1e-6)), sky_F])
