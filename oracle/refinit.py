"""Initial values of a Sérsic / exponential galaxy the way the reference's ``initialize()`` finds
them, restated in float64 numpy.

Test infrastructure only (the checker of the CUDA initialiser, never a product path).  Parity is
pinned by ``tests/golden/init_*.npz``: the reference's own ``model.initialize()`` run on seeded
noisy stamps (``tests/golden/make_golden.py``).

The chain (reference files, AstroPhot 0.x):

1. centre: the window centre, then an iterated centre of light in a small box
   (``models/model_object.py:180-233``, ``utils/initialize/center.py:8-49``);
2. PA: the flux-weighted mean of 2θ about the centre (``models/galaxy_model_object.py:60-98``,
   ``utils/angle_operations.py:35-56``);
3. q: the axis ratio, among 15 samples in [0.2, 0.9], whose isophote has the smallest second
   Fourier amplitude (``models/galaxy_model_object.py:99-113``,
   ``utils/initialize/initialize.py:8-113``, ``utils/isophote/extract.py:10-218``,
   ``utils/interpolate.py:232-273``);
4. n, Re, Ie: Nelder–Mead on the log of a 10-bin median profile
   (``models/_shared_methods.py:71-166``, ``models/sersic_model.py:33-38``,
   ``models/exponential_model.py:32-37``, ``utils/parametric_profiles.py:21-36, 77-86``);
5. every value written through the soft-limit setter (``param/parameter.py:452-477``).

Reference quirks kept: the isophotes are centred on the TRANSPOSED centre pixel (the reference
passes ``(y, x)`` where ``_iso_extract`` reads ``(x, y)``); the centre of light works on the raw
data (sky included) and returns the box centre of the step before convergence; the exponential
initialiser hands ``exponential_np`` its arguments in swapped order, so "Re" receives the fitted
amplitude and "Ie" the log10 of the fitted scale length.  The bootstrap uncertainties the
reference also draws (10 extra Nelder–Mead runs on resampled bins, ``np.random``) are not
restated: they set no value.
"""

from __future__ import annotations

import numpy as np

SOFTENING = 1e-3
NORTH = np.pi / 2.0  # ``Image_Header.north`` (image/image_header.py:36): PA is counted from +y
Q_SAMPLES = np.linspace(0.2, 0.9, 15)
LIMITS = {"q": (0.0, 1.0), "n": (0.36, 8.0), "Re": (0.0, None)}


def soft_set(v, lo, hi):
    """``Parameter._soft_set_val_self`` (``param/parameter.py:452-477``): 1e-3 inside the limits."""
    if lo is not None:
        v = max(v, lo + 1e-3)
    if hi is not None:
        v = min(v, hi - 1e-3)
    return v


def iqr_half(v):
    """``scipy.stats.iqr(v, rng=(16, 84)) / 2`` with numpy's linear percentiles."""
    p = np.percentile(np.asarray(v, dtype=np.float64), [16, 84])
    return (p[1] - p[0]) / 2


# -- 1. centre of light ---------------------------------------------------------------------

def centre_of_light(row, col, image):
    """``center_of_mass`` (``utils/initialize/center.py:8-49``): (row, col) of the light-weighted
    centre in a ``w x w`` box, iterated until it moves by less than 0.1 px (L1); the box centre
    of the step BEFORE the converged one is returned; the start if the box leaves the image."""
    ny, nx = image.shape
    w = max(min(int(min(image.shape) / 10), 30), 6)
    w += w % 2
    xx, yy = np.meshgrid(np.arange(w), np.arange(w))
    start = (row, col)
    c = np.array([row, col], dtype=np.float64)
    for _ in range(100):
        r0 = int(round(c[0]) - w / 2)
        r1 = int(round(c[0]) + w / 2)
        c0 = int(round(c[1]) - w / 2)
        c1 = int(round(c[1]) + w / 2)
        if r0 < 0 or c0 < 0 or r1 >= ny or c1 >= nx:
            return np.array(start, dtype=np.float64)
        box = image[r0:r1, c0:c1]
        den = np.sum(box)
        new = np.array([r0 + np.sum(box * yy) / den, c0 + np.sum(box * xx) / den])
        if np.sum(np.abs(c - new)) < 0.1:
            break
        c = new
    return c


# -- 2. position angle ----------------------------------------------------------------------

def angular_centre_pa(flux, X, Y):
    """``Angle_COM_PA`` (``utils/angle_operations.py:35-56``): half the angle of the flux-weighted
    mean of (cos 2θ, sin 2θ), mod π."""
    theta = np.arctan2(Y, X)
    cs = np.sum(flux * np.cos(2 * theta)) / np.sum(flux)
    sn = np.sum(flux * np.sin(2 * theta)) / np.sum(flux)
    return np.arctan2(sn, cs) / 2 % np.pi


# -- 3. isophotes ---------------------------------------------------------------------------

def sigma_clip_upper(v, iterations=10, nsigma=5.0):
    """``Sigma_Clip_Upper`` (``utils/isophote/extract.py:10-28``): iterate lim = median +
    nsigma * iqr/2 over the values below lim until lim repeats."""
    v2 = np.sort(v)
    old, lim = 0.0, np.inf
    i = 0
    while i < iterations and old != lim:
        sel = v2[v2 < lim]
        med = np.median(sel) if sel.size else np.nan
        rng = iqr_half(sel) if sel.size else np.nan
        old = lim
        lim = med + rng * nsigma
        i += 1
    return lim


def lanczos_at(img, X, Y, scale=5):
    """``interpolate_Lanczos`` (``utils/interpolate.py:232-273``): normalised separable Lanczos
    window of 2*scale taps per axis, clipped at the image edge."""
    ny, nx = img.shape
    out = np.empty(len(X))
    k = np.arange(-scale + 1, scale + 1)
    for i in range(len(X)):
        fx, fy = np.floor(X[i]), np.floor(Y[i])
        bx0, bx1 = max(0, int(round(fx - scale + 1))), min(nx, int(round(fx + scale + 1)))
        by0, by1 = max(0, int(round(fy - scale + 1))), min(ny, int(round(fy + scale + 1)))
        tx = k - X[i] + fx
        ty = k - Y[i] + fy
        Lx = (np.sinc(tx) * np.sinc(tx / scale))[bx0 - int(round(fx - scale + 1)) : 2 * scale + bx1 - int(round(fx + scale + 1))]
        Ly = (np.sinc(ty) * np.sinc(ty / scale))[by0 - int(round(fy - scale + 1)) : 2 * scale + by1 - int(round(fy + scale + 1))]
        L = np.ones((by1 - by0, bx1 - bx0)) * Lx * Ly.reshape((Ly.size, -1))
        out[i] = np.sum(img[by0:by1, bx0:bx1] * L) / np.sum(L)
    return out


def periodic_interp(x, xp, fp, period):
    """``np.interp(x, xp, fp, period=period)``: xp sorted mod period and wrapped by one sample at
    each end."""
    xp = np.asarray(xp) % period
    x = np.asarray(x) % period
    o = np.argsort(xp, kind="stable")
    xp, fp = xp[o], np.asarray(fp)[o]
    xp = np.concatenate((xp[-1:] - period, xp, xp[0:1] + period))
    fp = np.concatenate((fp[-1:], fp, fp[0:1]))
    return np.interp(x, xp, fp)


def iso_extract(img, sma, q, pa, cx, cy, nsigma=3.0, interp_mask=False):
    """``_iso_extract`` (``utils/isophote/extract.py:107-218``) with sigma clipping on: fluxes at
    N = max(15, int(0.9 * 2π sma)) points of the ellipse (Lanczos below sma 30, nearest pixel
    above), points off the image dropped; values above the clip limit are dropped, or with
    ``interp_mask`` replaced by periodic interpolation in angle."""
    ny, nx = img.shape
    N = max(15, int(0.9 * 2 * np.pi * sma))
    theta = np.linspace(0, 2 * np.pi * (1.0 - 1.0 / N), N)
    theta = np.arctan(q * np.tan(theta)) + np.pi * (np.cos(theta) < 0)
    ellip = 1.0 - q
    rs = (1 - ellip) / (np.abs((1 - ellip) * np.cos(theta)) ** 2 + np.abs(np.sin(theta)) ** 2) ** (1.0 / 2)
    X, Y = sma * (rs * np.cos(theta)), sma * (rs * np.sin(theta))
    s, c = np.sin(pa), np.cos(pa)
    X, Y = c * X - s * Y, c * Y + s * X
    theta = (theta + pa) % (2 * np.pi)
    X, Y = X + cx, Y + cy
    keep = (X >= 0) & (X < nx - 1) & (Y >= 0) & (Y < ny - 1)
    if not np.all(keep):
        X, Y, theta = X[keep], Y[keep], theta[keep]
    if sma < 30:
        flux = lanczos_at(img, X, Y, 5)
    else:
        flux = img[np.rint(Y).astype(np.int32), np.rint(X).astype(np.int32)]
    if len(flux) > 30:
        choose = flux < sigma_clip_upper(flux, 10, nsigma)
        if np.sum(choose) <= 0:
            return flux
        if interp_mask:
            flux = flux.copy()
            flux[~choose] = periodic_interp(theta[~choose], theta[choose], flux[choose], 2 * np.pi)
            return flux
        return flux[choose]
    return flux


def isophote_radius(img, cx, cy, threshold, pa, q):
    """The growth loop of ``isophotes`` (``utils/initialize/initialize.py:22-44``): radii
    1.2^k until the 80 % quantile of a (clipped) isophote falls below ``threshold`` (from the
    fifth radius on) or the radius reaches half the larger image side."""
    radii = [1.0]
    while radii[-1] < max(img.shape) / 2:
        radii.append(radii[-1] * (1 + 0.2))
        v = iso_extract(img, radii[-1], q, pa, cx, cy)
        if len(v) < 3:
            continue
        if np.quantile(v, 0.8) < threshold and len(radii) > 4:
            break
    return radii[-1]


def isophote_q(img, cx, cy, threshold, pa, q_samples=Q_SAMPLES):
    """``isophotes`` at one radius for each sampled q (``utils/initialize/initialize.py:46-113``)
    and the reference's choice (``galaxy_model_object.py:109-111``): the q whose isophote has
    the smallest |c2| / (N (max(0, median) + iqr/2)), c2 the second DFT coefficient."""
    R = isophote_radius(img, cx, cy, threshold, pa, float(np.max(q_samples)))
    amp = []
    for qi in q_samples:
        v = iso_extract(img, R, qi, pa, cx, cy, interp_mask=True)
        if len(v) < 3:
            amp.append(None)
            continue
        c2 = np.fft.fft(v)[2]
        flux = np.median(v)
        noise = iqr_half(v)
        amp.append(np.abs(c2) / (len(v) * (max(0, flux) + noise)))
    good = [i for i, a in enumerate(amp) if a is not None]
    if not good:
        raise ValueError("no isophote could be sampled")
    amp = [amp[good[-1]] if a is None else a for a in amp]
    return int(np.argmin(amp)), R, np.array(amp)


# -- 4. binned profile + Nelder-Mead --------------------------------------------------------

def sample_profile(dat, X, Y, pa, q, pixel_area):
    """``_sample_image`` (``models/_shared_methods.py:71-118``): median flux in 11 log-spaced
    radius edges of the inclined radius, made positive, monotone beyond the fifth bin, log10,
    empty bins interpolated.  ``dat`` is already mask-filled and edge-median subtracted."""
    c, s = np.cos(-pa), np.sin(-pa)
    Xr, Yr = c * X - s * Y, s * X + c * Y
    R = np.sqrt(Xr**2 + (Yr / q) ** 2 + SOFTENING**2).ravel()
    edges = np.logspace(np.log10(R.min() * 0.9), np.log10(R.max() * 1.1), 11)
    b = np.searchsorted(edges, R, side="right") - 1
    v = dat.ravel()
    I = np.array([np.median(v[b == i]) if np.any(b == i) else np.nan for i in range(10)]) / pixel_area
    Rc = (edges[:-1] + edges[1:]) / 2
    I[I <= 0] = np.min(I[np.isfinite(I) & (I > 0)])
    for i in range(5, len(I)):
        if I[i] >= I[i - 1] and np.isfinite(I[i - 1]):
            I[i] = I[i - 1] - np.abs(I[i - 1] * 0.1)
    I = np.log10(I)
    ok = np.isfinite(I)
    if not np.all(ok):
        I[~ok] = np.interp(Rc[~ok], Rc[ok], I[ok])
    return Rc, I


def sersic_b(n):
    """``sersic_n_to_b`` (``utils/conversions/functions.py:7-22``)."""
    return 2 * n - 1 / 3 + 4 / (405 * n) + 46 / (25515 * n**2) + 131 / (1148175 * n**3) - 2194697 / (30690717750 * n**4)


def profile_log(kind, R, x):
    """log10 of the profile the reference fits: ``sersic_np(R, n, Re, 10**Ie)`` (1e6 when a
    parameter is not positive) or ``exponential_np(R, Re, 10**Ie)`` called with swapped
    arguments (amplitude ``x[0]``, scale length ``10**x[1]``)."""
    with np.errstate(all="ignore"):
        if kind == "sersic":
            n, Re, Ie = x[0], x[1], 10 ** x[2]
            if n <= 0 or Re <= 0 or Ie <= 0:
                return np.log10(np.ones(len(R)) * 1e6)
            return np.log10(Ie * np.exp(-sersic_b(n) * ((R / Re) ** (1 / n) - 1)))
        amp, Rs = x[0], 10 ** x[1]
        return np.log10(amp * np.exp(-sersic_b(1.0) * (R / Rs - 1.0)))


def profile_objective(kind, R, I, x):
    """``optim`` (``models/_shared_methods.py:139-142``): mean squared log residual without the
    two largest."""
    with np.errstate(all="ignore"):
        r = (I - profile_log(kind, R, x)) ** 2
        return np.mean(np.sort(r)[:-2])


def nelder_mead(f, x0, xatol=1e-4, fatol=1e-4, maxiter=None):
    """Nelder–Mead as ``scipy.optimize.minimize(method="Nelder-Mead")`` runs it by default
    (the Lagarias, Reeds, Wright & Wright 1998 form: reflection 1, expansion 2, outside and
    inside contraction 1/2, shrink 1/2; first simplex x0 with each coordinate scaled by 1.05, or
    set to 2.5e-4 where it is 0; stop when every vertex is within ``xatol`` of the best and every
    value within ``fatol``, or after 200 N iterations / evaluations).
    Returns (x, success, evaluations)."""
    x0 = np.asarray(x0, dtype=np.float64)
    N = len(x0)
    maxiter = 200 * N if maxiter is None else maxiter
    maxfev = maxiter
    calls = [0]

    class _Spent(Exception):
        pass

    def F(x):
        if calls[0] >= maxfev:
            raise _Spent
        calls[0] += 1
        return f(x.copy())

    sim = np.empty((N + 1, N))
    sim[0] = x0
    for k in range(N):
        y = x0.copy()
        y[k] = 1.05 * y[k] if y[k] != 0 else 0.00025
        sim[k + 1] = y
    fs = np.empty(N + 1)
    for k in range(N + 1):
        fs[k] = F(sim[k])
    o = np.argsort(fs, kind="stable")
    sim, fs = sim[o], fs[o]
    it = 1
    while calls[0] < maxfev and it < maxiter:
        try:
            if np.max(np.abs(sim[1:] - sim[0])) <= xatol and np.max(np.abs(fs[0] - fs[1:])) <= fatol:
                break
            xbar = np.add.reduce(sim[:-1], 0) / N
            xr = 2 * xbar - sim[-1]
            fr = F(xr)
            if fr < fs[0]:
                xe = 3 * xbar - 2 * sim[-1]
                fe = F(xe)
                if fe < fr:
                    sim[-1], fs[-1] = xe, fe
                else:
                    sim[-1], fs[-1] = xr, fr
            elif fr < fs[-2]:
                sim[-1], fs[-1] = xr, fr
            else:
                shrink = False
                if fr < fs[-1]:
                    xc = 1.5 * xbar - 0.5 * sim[-1]
                    fc = F(xc)
                    if fc <= fr:
                        sim[-1], fs[-1] = xc, fc
                    else:
                        shrink = True
                else:
                    xcc = 0.5 * xbar + 0.5 * sim[-1]
                    fcc = F(xcc)
                    if fcc < fs[-1]:
                        sim[-1], fs[-1] = xcc, fcc
                    else:
                        shrink = True
                if shrink:
                    for j in range(1, N + 1):
                        sim[j] = sim[0] + 0.5 * (sim[j] - sim[0])
                        fs[j] = F(sim[j])
            it += 1
        except _Spent:
            pass
        o = np.argsort(fs, kind="stable")
        sim, fs = sim[o], fs[o]
    success = not (calls[0] >= maxfev or it >= maxiter)
    return sim[0].copy(), success, calls[0]


# -- the whole chain ------------------------------------------------------------------------

def initialize(data, kind="sersic", scale=1.0, origin=(0.0, 0.0), mask=None, given=None):
    """Values a ``Sersic_Galaxy`` / ``Exponential_Galaxy`` gets from ``initialize()`` on ``data``
    (rows = y, columns = x; pixel (i, j) centre at ((i + 0.5) scale + origin_x,
    (j + 0.5) scale + origin_y)); north = π/2.  ``given`` holds the parameters that already have
    values (center, PA, q, n, Re, Ie): the centre of light is skipped when the centre is given,
    PA and q are computed only where missing, and the profile fit starts from the given values
    and writes only the missing ones (``_shared_methods.py:129-166``).
    Returns a dict with center (x, y), q, PA, (n,) Re, Ie and diagnostics."""
    given = {} if given is None else dict(given)
    data = np.asarray(data, dtype=np.float64)
    ny, nx = data.shape
    ox, oy = origin
    area = scale * scale
    # 1. centre (model_object.py:199-233)
    if "center" in given:
        centre = np.asarray(given["center"], dtype=np.float64)
    else:
        centre = np.array([ox + nx * scale / 2, oy + ny * scale / 2])
        icx, icy = (centre[0] - ox) / scale - 0.5, (centre[1] - oy) / scale - 0.5
        com = centre_of_light(icy, icx, data)
        if not (np.any(com < 0) or np.any(com >= np.array(data.shape))):
            centre = np.array([(com[1] + 0.5) * scale + ox, (com[0] + 0.5) * scale + oy])
    # 2. PA (galaxy_model_object.py:65-98)
    dat = data.copy()
    if mask is not None:
        dat[mask] = np.median(dat[~mask])
    edge = np.concatenate((dat[:, 0], dat[:, -1], dat[0, :], dat[-1, :]))
    edge_average = np.nanmedian(edge)
    edge_scatter = iqr_half(edge[np.isfinite(edge)])
    X, Y = np.meshgrid((np.arange(nx) + 0.5) * scale + ox, (np.arange(ny) + 0.5) * scale + oy)
    X, Y = X - centre[0], Y - centre[1]
    if "PA" in given:
        PA = float(given["PA"])
    else:
        w = dat - edge_average
        if mask is not None:
            seg = ~mask
            pa = angular_centre_pa(w[seg], X[seg], Y[seg])
        else:
            pa = angular_centre_pa(w, X, Y)
        PA = (pa + NORTH) % np.pi
        PA = 0.0 + (PA - 0.0) % np.pi  # cyclic soft set
    pa = PA - NORTH  # the angle the isophotes and the inclined transform use
    # 3. q (galaxy_model_object.py:99-113) on the transposed centre pixel
    R_iso, amps = None, None
    if "q" in given:
        q = float(given["q"])
    else:
        icx, icy = (centre[0] - ox) / scale - 0.5, (centre[1] - oy) / scale - 0.5
        qi, R_iso, amps = isophote_q(data - edge_average, icy, icx, 3 * edge_scatter, pa)
        q = soft_set(float(Q_SAMPLES[qi]), *LIMITS["q"])
    # 4. profile (_shared_methods.py:123-166)
    dat = data.copy()
    if mask is not None:
        dat[mask] = np.median(dat[~mask])
    edge = np.concatenate((dat[:, 0], dat[:, -1], dat[0, :], dat[-1, :]))
    dat -= np.median(edge)
    names = ["n", "Re", "Ie"] if kind == "sersic" else ["Re", "Ie"]
    out = dict(center=centre, q=q, PA=PA, iso_R=R_iso, iso_amp=amps)
    for k in names:
        if k in given:
            out[k] = float(given[k])
    if all(k in given for k in names):
        return out
    Rc, I = sample_profile(dat, X, Y, pa, q, area)
    x0 = [2.0, Rc[4], I[4]] if kind == "sersic" else [Rc[4], I[4]]
    x0 = [float(given[k]) if k in given else v for k, v in zip(names, x0)]
    x, ok, calls = nelder_mead(lambda v: profile_objective(kind, Rc, I, v), x0)
    fit = x if ok else np.asarray(x0)
    out.update(profile_R=Rc, profile_I=I, x0=np.asarray(x0), nm_success=ok, nm_calls=calls)
    for k, v in zip(names, fit):
        if k in given:
            continue
        out[k] = soft_set(float(v), *LIMITS[k]) if k in LIMITS else float(v)
    return out
