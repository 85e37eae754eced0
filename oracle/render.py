"""float64 numpy restatement of AstroPhot's model-image rendering and its
forward-mode Jacobian.  TEST INFRASTRUCTURE ONLY (see ``oracle/__init__``).

Every stage follows the reference's own operation order so that the
data-dependent integration masks (``select``) come out the same as the
reference's.  The Jacobian is the analytic derivative of the same graph
that the reference differentiates with ``torch.autograd.functional.jacobian
(strategy="forward-mode")`` (``astrophot/models/_model_methods.py:325-340``):
the masks are constants, the bilinear PSF shift is differentiated with
respect to the centre, and the representation transforms are chained on
top.

Coordinates: image arrays are ``[ny, nx]`` (row = y).  Windows carry the
pixel-scale matrix ``P`` and the reference points in (x, y) order, exactly
like ``astrophot/image/wcs.py:432-584`` (``PPCS``).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field, replace
from typing import Dict, List, Optional, Tuple

import numpy as np
from scipy.special import gammaln, roots_legendre

NORTH = math.pi / 2  # astrophot/image/image_header.py:36

# ----------------------------------------------------------------------------
# parameters and their (value <-> representation) maps
# ----------------------------------------------------------------------------

# (limits, cyclic) per parameter name; astrophot/models/galaxy_model_object.py:44-53,
# astrophot/models/sersic_model.py:61-65, exponential_model.py:58-61, flatsky_model.py:23-25
PARAM_SPECS = {
    "center": ((None, None), False),
    "q": ((0.0, 1.0), False),
    "PA": ((0.0, math.pi), True),
    "n": ((0.36, 8.0), False),
    "Re": ((0.0, None), False),
    "Ie": ((None, None), False),
    "F": ((None, None), False),
    # Moffat (models/moffat_model.py:88-92); its n takes KIND_SPECS' limits
    "Rd": ((0.0, None), False),
    "I0": ((None, None), False),
    # Gaussian_PSF (models/gaussian_model.py:272-275)
    "sigma": ((0.0, None), False),
    "flux": ((None, None), False),
}

# per-kind overrides of PARAM_SPECS: Moffat_PSF's n, models/moffat_model.py:89
KIND_SPECS = {"moffat": {"n": ((0.1, 10.0), False)}}


def _spec(name, kind=None):
    return KIND_SPECS.get(kind, {}).get(name, PARAM_SPECS[name])

PARAM_ORDER = {
    # astrophot/models/model_object.py:61, galaxy_model_object.py:53,
    # sersic_model.py:66, exponential_model.py:62, flatsky_model.py:26
    "sersic": ("center", "q", "PA", "n", "Re", "Ie"),
    "exponential": ("center", "q", "PA", "Re", "Ie"),
    "flat_sky": ("F",),
    # psf_model_object.py:45, moffat_model.py:93
    "moffat": ("center", "n", "Rd", "I0"),
    # gaussian_model.py:276
    "gaussian": ("center", "sigma", "flux"),
}


def value_to_rep(name: str, val, kind=None):
    """``boundaries`` / ``cyclic_boundaries``: utils/conversions/optimization.py:6-14,50-54."""
    (lo, hi), cyclic = _spec(name, kind)
    val = np.asarray(val, dtype=np.float64)
    if cyclic:
        return lo + np.mod(val - lo, hi - lo)
    if lo is None and hi is None:
        return val
    if lo is None:
        return val - 1.0 / (val - hi)
    if hi is None:
        return val - 1.0 / (val - lo)
    return np.tan((val - lo) * np.pi / (hi - lo) - np.pi / 2)


def rep_to_value(name: str, rep, kind=None):
    """``inv_boundaries`` / ``cyclic_boundaries``: utils/conversions/optimization.py:17-25,50-54."""
    (lo, hi), cyclic = _spec(name, kind)
    rep = np.asarray(rep, dtype=np.float64)
    if cyclic:
        return lo + np.mod(rep - lo, hi - lo)
    if lo is None and hi is None:
        return rep
    if lo is None:
        return (rep + hi - np.sqrt((rep - hi) ** 2 + 4)) * 0.5
    if hi is None:
        return (rep + lo + np.sqrt((rep - lo) ** 2 + 4)) * 0.5
    return (np.arctan(rep) + np.pi / 2) * (hi - lo) / np.pi + lo


def drep_dvalue(name: str, rep, kind=None):
    """d(value)/d(representation), i.e. ``d_inv_boundaries_dval``
    (utils/conversions/optimization.py:40-47); 1 for cyclic and free parameters
    (forward-mode AD of ``remainder`` has unit slope)."""
    (lo, hi), cyclic = _spec(name, kind)
    rep = np.asarray(rep, dtype=np.float64)
    if cyclic or (lo is None and hi is None):
        return np.ones_like(rep)
    if lo is None:
        return 0.5 - 0.5 * (rep - hi) / np.sqrt((rep - hi) ** 2 + 4)
    if hi is None:
        return 0.5 + 0.5 * (rep - lo) / np.sqrt((rep - lo) ** 2 + 4)
    return (hi - lo) / (np.pi * (rep**2 + 1))


def check_limits(name: str, val, kind=None) -> None:
    """``Parameter_Node._set_val_self`` limit check, astrophot/param/parameter.py:436-450."""
    (lo, hi), cyclic = _spec(name, kind)
    if cyclic:
        return
    val = np.asarray(val)
    if lo is not None and not np.all(val > lo):
        raise ValueError(f"{name} has lower limit {lo}")
    if hi is not None and not np.all(val < hi):
        raise ValueError(f"{name} has upper limit {hi}")


# ----------------------------------------------------------------------------
# 1-D profiles and closed forms
# ----------------------------------------------------------------------------


def sersic_b(n):
    """utils/conversions/functions.py:7-22."""
    return (
        2 * n
        - 1 / 3
        + 4 / (405 * n)
        + 46 / (25515 * n**2)
        + 131 / (1148175 * n**3)
        - 2194697 / (30690717750 * n**4)
    )


def sersic_db(n):
    """d b(n) / d n of :func:`sersic_b`."""
    return (
        2.0
        - 4 / (405 * n**2)
        - 2 * 46 / (25515 * n**3)
        - 3 * 131 / (1148175 * n**4)
        + 4 * 2194697 / (30690717750 * n**5)
    )


def sersic_total_flux(Ie_lin, n, Re, q):
    """``sersic_Ie_to_flux_torch``, utils/conversions/functions.py:168-190."""
    bn = sersic_b(n)
    return 2 * np.pi * Ie_lin * Re**2 * q * n * (np.exp(bn) * bn ** (-2 * n)) * np.exp(gammaln(2 * n))


# ----------------------------------------------------------------------------
# geometry (astrophot/image/wcs.py PPCS, astrophot/image/window_object.py)
# ----------------------------------------------------------------------------


@dataclass
class Window:
    """Pixel grid on the tangent plane: ``xy = P (ij - ref_ij) + ref_xy``
    (wcs.py:561-584).  ``nx, ny`` is ``pixel_shape``."""

    nx: int
    ny: int
    P: np.ndarray = field(default_factory=lambda: np.eye(2))
    ref_ij: np.ndarray = field(default_factory=lambda: np.array([-0.5, -0.5]))
    ref_xy: np.ndarray = field(default_factory=lambda: np.zeros(2))

    def __post_init__(self):
        self.P = np.asarray(self.P, dtype=np.float64).reshape(2, 2)
        self.ref_ij = np.asarray(self.ref_ij, dtype=np.float64).copy()
        self.ref_xy = np.asarray(self.ref_xy, dtype=np.float64).copy()

    @staticmethod
    def from_scale(nx, ny, scale=1.0, origin=(0.0, 0.0)):
        return Window(nx, ny, np.eye(2) * float(scale), np.array([-0.5, -0.5]), np.array(origin, float))

    @property
    def pixel_area(self):
        return abs(np.linalg.det(self.P))

    @property
    def pixel_length(self):
        return math.sqrt(self.pixel_area)

    def copy(self):
        return replace(self, P=self.P.copy(), ref_ij=self.ref_ij.copy(), ref_xy=self.ref_xy.copy())

    def pixel_to_plane(self, i, j):
        i = np.asarray(i, dtype=np.float64)
        j = np.asarray(j, dtype=np.float64)
        di = i - self.ref_ij[0]
        dj = j - self.ref_ij[1]
        return (
            self.P[0, 0] * di + self.P[0, 1] * dj + self.ref_xy[0],
            self.P[1, 0] * di + self.P[1, 1] * dj + self.ref_xy[1],
        )

    def plane_to_pixel(self, x, y):
        Pi = np.linalg.inv(self.P)
        dx = np.asarray(x, float) - self.ref_xy[0]
        dy = np.asarray(y, float) - self.ref_xy[1]
        return (
            Pi[0, 0] * dx + Pi[0, 1] * dy + self.ref_ij[0],
            Pi[1, 0] * dx + Pi[1, 1] * dy + self.ref_ij[1],
        )

    def meshgrid(self):
        """``get_coordinate_meshgrid``, window_object.py:390-405."""
        ii, jj = np.meshgrid(np.arange(self.nx, dtype=float), np.arange(self.ny, dtype=float), indexing="xy")
        return self.pixel_to_plane(ii, jj)

    def corner_meshgrid(self):
        """``get_coordinate_corner_meshgrid``, window_object.py:407-426."""
        ii, jj = np.meshgrid(
            np.arange(self.nx + 1, dtype=float) - 0.5, np.arange(self.ny + 1, dtype=float) - 0.5, indexing="xy"
        )
        return self.pixel_to_plane(ii, jj)

    def simps_meshgrid(self):
        """``get_coordinate_simps_meshgrid``, window_object.py:428-460."""
        ii, jj = np.meshgrid(
            0.5 * np.arange(2 * self.nx + 1, dtype=float) - 0.5,
            0.5 * np.arange(2 * self.ny + 1, dtype=float) - 0.5,
            indexing="xy",
        )
        return self.pixel_to_plane(ii, jj)

    def rescale_pixel(self, scale):
        """window_object.py:233-239."""
        w = self.copy()
        w.P = self.P * scale
        w.nx = int(self.nx // scale)
        w.ny = int(self.ny // scale)
        w.ref_ij = (self.ref_ij + 0.5) / scale - 0.5
        return w

    def pad_pixel(self, bx, by):
        """window_object.py:367-388 (two-value form)."""
        self.nx += 2 * bx
        self.ny += 2 * by
        self.ref_ij = self.ref_ij + np.array([bx, by], float)
        return self

    def pixel_shift(self, shift):
        """window_object.py:284-290."""
        self.ref_ij = self.ref_ij - shift
        return self


@dataclass
class PSF:
    """A PSF stamp (odd shape) on its own pixel grid (``PSF_Image``,
    astrophot/image/psf_image.py:17-93)."""

    data: np.ndarray
    scale: float = 1.0

    @property
    def border(self) -> Tuple[int, int]:
        """``psf_border_int`` = ceil((1 + flip(shape)) / 2), psf_image.py:71-93 -> (bx, by)."""
        ky, kx = self.data.shape
        return int(math.ceil((1 + kx) / 2)), int(math.ceil((1 + ky) / 2))

    @property
    def pixel_length(self):
        return float(self.scale)


@dataclass
class Component:
    """One AstroPhot component model and its sampling knobs
    (class attributes at astrophot/models/model_object.py:64-95)."""

    kind: str  # "sersic" | "exponential" | "flat_sky"
    params: Dict[str, np.ndarray]
    psf_mode: str = "none"
    psf_convolve_mode: str = "fft"
    psf_subpixel_shift: str = "bilinear"
    sampling_mode: str = "midpoint"
    sampling_tolerance: float = 1e-2
    integrate_mode: str = "threshold"
    integrate_max_depth: int = 3
    integrate_gridding: int = 5
    integrate_quad_level: int = 3
    softening: float = 1e-3
    # sampling_mode "midpoint_center" (the single-Sersic stamp configuration's "midpoint sampling
    # plus 3 x 3 supersampling within 2 px of the centre"; no such mode in the reference)
    center_quad_level: int = 3
    center_radius: float = 2.0
    # pixel count the integration threshold divides by (None: the working window's).  A windowed
    # source of a group is evaluated by the reference on the group's window; a Sersic source
    # rendered on its own window with the group's working pixel count gives the same pixels.
    thr_numel: Optional[float] = None
    locked: Tuple[str, ...] = ()
    # pixel window [[x0, x1], [y0, y1]] inside the group's window (Model.window given in pixels,
    # models/core_model.py:313-325 -> Window.crop_to_pixel); None = the whole window
    window: Optional[Tuple[Tuple[int, int], Tuple[int, int]]] = None

    def __post_init__(self):
        self.params = {k: np.asarray(v, dtype=np.float64) for k, v in self.params.items()}
        if self.kind == "flat_sky":  # Sky_Model forces these, sky_model_object.py:21-35
            self.psf_mode = "none"
            self.integrate_mode = "none"

    @property
    def param_names(self):
        return PARAM_ORDER[self.kind]

    def free_slots(self) -> List[Tuple[str, int]]:
        """(name, element) pairs in ``vector_values`` order, skipping locked nodes."""
        out = []
        for name in self.param_names:
            if name in self.locked:
                continue
            size = 2 if name == "center" else 1
            out += [(name, k) for k in range(size)]
        return out


# ----------------------------------------------------------------------------
# brightness evaluation with analytic partials
# ----------------------------------------------------------------------------

GRAD_KEYS = ("X", "Y", "q", "PA", "n", "Re", "Ie", "F", "Rd", "I0", "sigma", "flux")


def eval_brightness(comp: Component, X, Y, pixel_area, grad: bool):
    """Brightness at plane offsets (X, Y) from the centre.

    Sersic/exponential: ``transformed_evaluate_model`` (models/_shared_methods.py:286-296) ->
    ``inclined_transform_coordinates`` (:301-307, ``Rotate_Cartesian``
    utils/conversions/coordinates.py:5-13) -> ``radius_metric`` (models/_model_methods.py:38-40)
    -> ``sersic_torch`` / ``exponential_torch`` (utils/parametric_profiles.py:7-18, 63-74).
    Flat sky: ``Flat_Sky.evaluate_model`` (models/flatsky_model.py:53-55).

    Returns (I, partials) where partials maps GRAD_KEYS to arrays (d I / d key, with X and Y
    the sample coordinates relative to the centre).
    """
    p = comp.params
    if comp.kind == "flat_sky":
        I = np.ones_like(X) * (pixel_area * 10 ** p["F"])
        if not grad:
            return I, None
        return I, {"F": I * np.log(10.0)}
    if comp.kind == "moffat":
        # Moffat_PSF: radial_evaluate_model on untransformed coordinates
        # (models/_shared_methods.py:275-283, psf_model_object.py:140-142) -> moffat_torch
        # (utils/parametric_profiles.py:89-100) with I0 * pixel_area (_shared_methods.py:355-361)
        n, Rd = p["n"], p["Rd"]
        R = np.sqrt(X**2 + Y**2 + comp.softening**2)
        w = 1 + (R / Rd) ** 2
        I = (pixel_area * 10 ** p["I0"]) / w**n
        if not grad:
            return I, None
        dI_dR = -I * n * 2 * R / (Rd * Rd * w)
        return I, {"n": -I * np.log(w), "Rd": I * n * 2 * R * R / (Rd**3 * w), "I0": I * np.log(10.0),
                   "X": dI_dR * X / R, "Y": dI_dR * Y / R}
    if comp.kind == "gaussian":
        # Gaussian_PSF: radial_evaluate_model -> gaussian_torch (utils/parametric_profiles.py:39-48)
        # with 10^flux * pixel_area (models/_shared_methods.py:403-408)
        sig = p["sigma"]
        R = np.sqrt(X**2 + Y**2 + comp.softening**2)
        I = (pixel_area * 10 ** p["flux"]) / np.sqrt(2 * np.pi * sig**2) * np.exp(-0.5 * (R / sig) ** 2)
        if not grad:
            return I, None
        dI_dR = -I * R / sig**2
        return I, {"sigma": I * (R * R / sig**3 - 1 / sig), "flux": I * np.log(10.0), "X": dI_dR * X / R,
                   "Y": dI_dR * Y / R}

    q = p["q"]
    PA = p["PA"]
    theta = -(PA - NORTH)
    s = np.sin(theta)
    c = np.cos(theta)
    Xr = c * X - s * Y
    Yr0 = s * X + c * Y
    Yr = Yr0 / q
    R = np.sqrt(Xr**2 + Yr**2 + comp.softening**2)
    Re = p["Re"]
    amp = pixel_area * 10 ** p["Ie"]
    if comp.kind == "sersic":
        n = p["n"]
        bn = sersic_b(n)
        t = np.power(R / Re, 1 / n)
        I = amp * np.exp(-bn * (t - 1))
    elif comp.kind == "exponential":
        bn = sersic_b(1.0)
        I = amp * np.exp(-bn * ((R / Re) - 1.0))
    else:
        raise ValueError(comp.kind)
    if not grad:
        return I, None

    out = {}
    if comp.kind == "sersic":
        dI_dR = -I * bn * t / (n * R)
        out["Re"] = I * bn * t / (n * Re)
        out["n"] = I * (-sersic_db(n) * (t - 1) + bn * t * np.log(R / Re) / (n * n))
    else:
        dI_dR = -I * bn / Re
        out["Re"] = I * bn * R / (Re * Re)
    out["Ie"] = I * np.log(10.0)
    # R^2 = Xr^2 + (Yr0/q)^2 + eps^2;  dXr/dPA = Yr0, dYr0/dPA = -Xr
    out["q"] = dI_dR * (-(Yr * Yr) / (q * R))
    out["PA"] = dI_dR * (Xr * Yr0 * (1.0 - 1.0 / (q * q)) / R)
    out["X"] = dI_dR * ((Xr * c + Yr * s / q) / R)
    out["Y"] = dI_dR * ((-Xr * s + Yr * c / q) / R)
    return I, out


def _zero_grad(shape):
    return {k: np.zeros(shape) for k in GRAD_KEYS}


def _fill_grad(g):
    full = {}
    for k in GRAD_KEYS:
        full[k] = g[k] if (g is not None and k in g) else None
    return full


class Sampled:
    """A value array plus its partials (None entries mean identically zero)."""

    def __init__(self, val, grad=None):
        self.val = val
        self.grad = grad  # dict or None

    def wsum(self, weights, axis=-1):
        g = None
        if self.grad is not None:
            g = {k: (None if v is None else np.sum(v * weights, axis=axis)) for k, v in self.grad.items()}
        return Sampled(np.sum(self.val * weights, axis=axis), g)


def _eval(comp, X, Y, pixel_area, grad):
    I, g = eval_brightness(comp, X, Y, pixel_area, grad)
    return Sampled(I, _fill_grad(g) if grad else None)


# ----------------------------------------------------------------------------
# sub-pixel quadrature (astrophot/utils/operations.py)
# ----------------------------------------------------------------------------


def quad_table(n, P):
    """operations.py:105-120."""
    abscissa, weights = roots_legendre(n)
    Xg, Yg = np.meshgrid(abscissa, abscissa, indexing="xy")
    W = np.outer(weights, weights) / 4.0
    st = np.stack((Xg, Yg)).reshape(2, -1) / 2.0
    XY = P @ st
    return XY[0], XY[1], W.reshape(-1)


def displacement_grid(N, P):
    """operations.py:94-102."""
    px = np.linspace(-(N - 1) / (2 * N), (N - 1) / (2 * N), N)
    PX, PY = np.meshgrid(px, px, indexing="xy")
    XY = P @ np.stack((PX, PY)).reshape(2, -1)
    return XY[0], XY[1]


def single_quad_integrate(comp, X, Y, P, pixel_area, quad_level, grad):
    """operations.py:123-147: (res, ref) with ref the middle sample."""
    aX, aY, w = quad_table(quad_level, P)
    Xs = X[..., None] + aX
    Ys = Y[..., None] + aY
    S = _eval(comp, Xs, Ys, pixel_area, grad)
    ref = S.val[..., (quad_level**2) // 2]
    return S.wsum(w), ref


def grid_integrate(comp, X, Y, P, pixel_area, quad_level, gridding, depth, max_depth, reference, grad):
    """operations.py:150-247, including the ``reference * gridding**2`` threshold passed down
    to the finer level (:241) while ``pixel_area`` shrinks by ``gridding**2`` (:232)."""
    res, ref = single_quad_integrate(comp, X, Y, P, pixel_area, quad_level, grad)
    if depth >= max_depth:
        return res
    select = np.abs(res.val - ref) > reference
    out_val = res.val.copy()
    out_grad = None if res.grad is None else {k: (None if v is None else v.copy()) for k, v in res.grad.items()}
    if np.any(select):
        sx, sy = displacement_grid(gridding, P)
        subX = X[select][:, None] + sx
        subY = Y[select][:, None] + sy
        sub = grid_integrate(
            comp,
            subX,
            subY,
            P / gridding,
            pixel_area / gridding**2,
            quad_level,
            gridding,
            depth + 1,
            max_depth,
            reference * gridding**2,
            grad,
        )
        out_val[select] = sub.val.sum(axis=-1)
        if out_grad is not None:
            for k in GRAD_KEYS:
                if sub.grad[k] is not None:
                    out_grad[k][select] = sub.grad[k].sum(axis=-1)
    return Sampled(out_val, out_grad)


# ----------------------------------------------------------------------------
# sampling modes (astrophot/models/_model_methods.py:82-184)
# ----------------------------------------------------------------------------


def _laplacian_replicate(img):
    """conv2d with ``curvature_kernel`` (utils/interpolate.py:332-343), ``valid``, then
    ``replicate`` pad by 1 (models/_model_methods.py:89-97)."""
    ny, nx = img.shape
    if ny < 3 or nx < 3:
        raise ValueError("curvature stencil needs at least 3x3 pixels")
    c = img[1:-1, 1:-1]
    lap = img[:-2, 1:-1] + img[1:-1, :-2] + (-4.0) * c + img[1:-1, 2:] + img[2:, 1:-1]
    return np.pad(lap, 1, mode="edge")


def _conv_valid_stride(img, kernel, stride):
    kh, kw = kernel.shape
    ny = (img.shape[0] - kh) // stride + 1
    nx = (img.shape[1] - kw) // stride + 1
    out = np.zeros((ny, nx))
    for v in range(kh):
        for u in range(kw):
            out += kernel[v, u] * img[v : v + stride * (ny - 1) + 1 : stride, u : u + stride * (nx - 1) + 1 : stride]
    return out


SIMPSONS_KERNEL = np.array([[1.0, 4.0, 1.0], [4.0, 16.0, 4.0], [1.0, 4.0, 1.0]]) / 36.0  # interpolate.py:346-355


def _map_sampled(S: Sampled, fn):
    g = None
    if S.grad is not None:
        g = {k: (None if v is None else fn(v)) for k, v in S.grad.items()}
    return Sampled(fn(S.val), g)


def sample_init(comp, win: Window, center, grad):
    """``_sample_init``, models/_model_methods.py:82-148 -> (reference image, deep Sampled)."""
    mode = comp.sampling_mode
    if mode == "midpoint":
        cx, cy = win.meshgrid()
        S = _eval(comp, cx - center[0], cy - center[1], win.pixel_area, grad)
        curv = _laplacian_replicate(S.val)
        return S.val + curv, S
    if mode == "simpsons":
        cx, cy = win.simps_meshgrid()
        D = _eval(comp, cx - center[0], cy - center[1], win.pixel_area, grad)
        mid = D.val[1::2, 1::2]
        simps = _map_sampled(D, lambda a: _conv_valid_stride(a, SIMPSONS_KERNEL, 2))
        return mid, simps
    if mode.startswith("quad"):
        level = int(mode[mode.find(":") + 1 :])
        cx, cy = win.meshgrid()
        res, ref = single_quad_integrate(comp, cx - center[0], cy - center[1], win.P, win.pixel_area, level, grad)
        return ref, res
    if mode == "midpoint_center":
        return sample_midpoint_center(comp, win, center, grad)
    if mode == "trapezoid":
        cx, cy = win.corner_meshgrid()
        D = _eval(comp, cx - center[0], cy - center[1], win.pixel_area, grad)
        trapz = _map_sampled(D, lambda a: _conv_valid_stride(a, np.full((2, 2), 0.25), 1))
        curv = _laplacian_replicate(trapz.val)
        return trapz.val + curv, trapz
    raise ValueError(f"unknown sampling mode: {mode}")


# squared pixel distances up to radius^2 + CENTER_R2_SLACK count as inside: with the sub-pixel
# shift the pixel centres sit at whole-pixel offsets from the model centre, and a pixel exactly
# at the radius must not fall out by the rounding of its coordinates
CENTER_R2_SLACK = 1e-6


def center_select(win: Window, X, Y, radius):
    """Pixels whose centres lie within ``radius`` pixels of the model centre (plane offsets X, Y
    mapped back to pixel units by the inverse pixel-scale matrix)."""
    Pinv = np.linalg.inv(win.P)
    di = Pinv[0, 0] * X + Pinv[0, 1] * Y
    dj = Pinv[1, 0] * X + Pinv[1, 1] * Y
    return di * di + dj * dj <= radius * radius + CENTER_R2_SLACK


def sample_midpoint_center(comp, win: Window, center, grad):
    """Midpoint sampling with the pixels near the centre integrated by Gauss-Legendre
    quadrature: the midpoint image (``_sample_init`` "midpoint", models/_model_methods.py:84-87)
    with the pixels whose centres lie within ``center_radius`` pixels of the model centre
    replaced by ``single_quad_integrate`` (utils/operations.py:123-147) at
    ``center_quad_level``.  Returns (reference image, deep Sampled) like ``sample_init``; the
    adaptive integration does not run in this mode (its reference image is the curvature
    estimate of the midpoint image, as for "midpoint")."""
    if comp.integrate_mode != "none":
        raise ValueError("sampling_mode midpoint_center needs integrate_mode none")
    cx, cy = win.meshgrid()
    X, Y = cx - center[0], cy - center[1]
    S = _eval(comp, X, Y, win.pixel_area, grad)
    curv = _laplacian_replicate(S.val)
    sel = center_select(win, X, Y, comp.center_radius)
    if np.any(sel):
        res, _ = single_quad_integrate(comp, X[sel], Y[sel], win.P, win.pixel_area, comp.center_quad_level, grad)
        S.val[sel] = res.val
        if grad:
            for k in GRAD_KEYS:
                if res.grad[k] is not None:
                    if S.grad[k] is None:
                        S.grad[k] = np.zeros_like(S.val)
                    S.grad[k][sel] = res.grad[k]
    return S.val + curv, S


def integrate_reference(comp, deep_val):
    """``_integrate_reference``: models/_model_methods.py:151-152 (sum / numel), overridden by
    ``Sersic_Galaxy._integrate_reference`` (models/sersic_model.py:87-89, total flux / numel)."""
    numel = deep_val.size if comp.thr_numel is None else comp.thr_numel
    if comp.kind == "sersic":
        p = comp.params
        tot = sersic_total_flux(10 ** p["Ie"], p["n"], p["Re"], p["q"])
        return tot / numel
    return np.sum(deep_val) / numel


def sample_integrate(comp, deep: Sampled, reference, win: Window, center, grad):
    """``_sample_integrate``, models/_model_methods.py:155-184."""
    if comp.integrate_mode == "none":
        return deep, None
    if comp.integrate_mode != "threshold":
        raise ValueError(f"unknown integrate mode {comp.integrate_mode}")
    cx, cy = win.meshgrid()
    X = cx - center[0]
    Y = cy - center[1]
    ref = integrate_reference(comp, deep.val)
    error = np.abs(deep.val - reference)
    select = error > comp.sampling_tolerance * ref
    if np.any(select):
        sub = grid_integrate(
            comp,
            X[select],
            Y[select],
            win.P,
            win.pixel_area,
            comp.integrate_quad_level,
            comp.integrate_gridding,
            1,
            comp.integrate_max_depth,
            comp.sampling_tolerance * ref,
            grad,
        )
        deep.val[select] = sub.val
        if grad:
            for k in GRAD_KEYS:
                if sub.grad[k] is not None:
                    if deep.grad[k] is None:
                        deep.grad[k] = np.zeros_like(deep.val)
                    deep.grad[k][select] = sub.grad[k]
    return deep, select


# ----------------------------------------------------------------------------
# PSF shift and convolution
# ----------------------------------------------------------------------------


def shift_psf_bilinear(psf: np.ndarray, shift, grad: bool):
    """``_shift_psf`` bilinear (models/_model_methods.py:187-207) using ``interp2d``
    (utils/interpolate.py:282-329), kept padded by 1, plus d/d(shift_x), d/d(shift_y)."""
    pad = np.pad(psf, 1)
    h, w = pad.shape
    x = np.arange(w, dtype=float)[None, :] - shift[0] + np.zeros((h, 1))
    y = np.arange(h, dtype=float)[:, None] - shift[1] + np.zeros((1, w))
    x0 = np.floor(x).astype(np.int64)
    y0 = np.floor(y).astype(np.int64)
    x1 = x0 + 1
    y1 = y0 + 1
    x0 = np.clip(x0, 0, w - 2)
    x1 = np.clip(x1, 1, w - 1)
    y0 = np.clip(y0, 0, h - 2)
    y1 = np.clip(y1, 1, h - 1)
    fa = pad[y0, x0]
    fb = pad[y1, x0]
    fc = pad[y0, x1]
    fd = pad[y1, x1]
    wa = (x1 - x) * (y1 - y)
    wb = (x1 - x) * (y - y0)
    wc = (x - x0) * (y1 - y)
    wd = (x - x0) * (y - y0)
    out = fa * wa + fb * wb + fc * wc + fd * wd
    if not grad:
        return out, None, None
    # dx/dshift_x = -1, dy/dshift_y = -1
    dsx = -(fa * (-(y1 - y)) + fb * (-(y - y0)) + fc * (y1 - y) + fd * (y - y0))
    dsy = -(fa * (-(x1 - x)) + fb * (x1 - x) + fc * (-(x - x0)) + fd * (x - x0))
    return out, dsx, dsy


def _lanczos_1d(shift, order):
    """Lanczos weights f(a - order + shift), f(t) = sinc(t) sinc(t / order), a = 0..2 order, and
    their shift derivatives (``_shift_Lanczos_kernel_torch``, utils/interpolate.py:145-163, with
    dx = -shift; f is even, so the reference's sign flip of the argument changes nothing)."""
    t = np.arange(-order, order + 1, dtype=float) + shift

    def sinc_d(u):
        x = np.pi * u
        small = np.abs(x) < 1e-4
        xs = np.where(small, 1.0, x)
        v = np.where(small, 1.0 - x * x / 6.0, np.sin(xs) / xs)
        dv = np.where(small, np.pi * (-x / 3.0), np.pi * (np.cos(xs) - np.sin(xs) / xs) / xs)
        return v, dv

    s1, d1 = sinc_d(t)
    s2, d2 = sinc_d(t / order)
    return s1 * s2, d1 * s2 + s1 * d2 / order


def shift_psf_lanczos(psf: np.ndarray, shift, order: int, grad: bool):
    """``_shift_psf`` "lanczos:order" (models/_model_methods.py:209-227): the PSF zero-padded by
    ``order`` and cross-correlated ("same") with Lx (x) Ly, kept padded, plus d/d(shift_x),
    d/d(shift_y).  The kernel is left unnormalised: the caller renormalises the shifted PSF,
    which cancels the reference's normalisation of the kernel."""
    k = int(order)
    lx, dlx = _lanczos_1d(shift[0], k)
    ly, dly = _lanczos_1d(shift[1], k)
    pad = np.pad(psf, k)
    big = np.pad(pad, k)  # the "same" correlation's zero border
    h, w = pad.shape

    def corr(wx, wy):
        out = np.zeros((h, w))
        for b in range(2 * k + 1):
            for a in range(2 * k + 1):
                out += wy[b] * wx[a] * big[b : b + h, a : a + w]
        return out

    out = corr(lx, ly)
    if not grad:
        return out, None, None
    return out, corr(dlx, ly), corr(lx, dly)


def convolve_fft_semantics(img, kern):
    """``fft_convolve_torch(img, psf, img_prepadded=True)`` (utils/operations.py:9-36): circular
    convolution at the image size, rolled by -(k-1)/2 -- written as the equivalent direct sum."""
    ky, kx = kern.shape
    cy, cx = (ky - 1) // 2, (kx - 1) // 2
    out = np.zeros_like(img)
    for v in range(ky):
        for u in range(kx):
            if kern[v, u] != 0.0:
                out += kern[v, u] * np.roll(img, shift=(v - cy, u - cx), axis=(0, 1))
    return out


def convolve_direct_semantics(img, kern):
    """``conv2d(img, flip(psf), padding="same")`` (models/_model_methods.py:247-255): zero-padded."""
    ky, kx = kern.shape
    cy, cx = (ky - 1) // 2, (kx - 1) // 2
    ny, nx = img.shape
    padded = np.pad(img, ((cy, cy), (cx, cx)))
    out = np.zeros_like(img)
    for v in range(ky):
        for u in range(kx):
            if kern[v, u] != 0.0:
                out += kern[v, u] * padded[2 * cy - v : 2 * cy - v + ny, 2 * cx - u : 2 * cx - u + nx]
    return out


# ----------------------------------------------------------------------------
# Component_Model.sample + jacobian (astrophot/models/model_object.py:258-375)
# ----------------------------------------------------------------------------


@dataclass
class Rendered:
    model: np.ndarray  # [ny, nx]
    jac: Optional[Dict[Tuple[str, int], np.ndarray]]  # value-space partials keyed (name, element)
    select: Optional[np.ndarray] = None
    working_shape: Tuple[int, int] = (0, 0)


def sample_component(comp: Component, win: Window, psf: Optional[PSF] = None, grad: bool = False,
                     psf_dirs: Optional[dict] = None) -> Rendered:
    """Render one component on ``win`` (its own window) and, when ``grad``, the value-space
    Jacobian with respect to every parameter element (locked ones included; the caller
    selects).  Follows ``Component_Model.sample`` (models/model_object.py:258-375).
    ``psf_dirs`` {name: d psf / d theta} (a live PSF model's parameters) adds the columns
    ("psf", name): the pre-convolution image convolved with the derivative of the shifted,
    renormalised kernel (models/_model_methods.py:233-243) along each."""
    p = comp.params
    center = p["center"] if "center" in p else np.zeros(2)
    center_partials_from_coords = True
    if comp.psf_mode == "full" and comp.kind != "flat_sky":
        if psf is None:
            raise ValueError("psf_mode full needs a PSF")
        upscale = int(round(win.pixel_length / psf.pixel_length))
        work = win.rescale_pixel(1 / upscale) if upscale != 1 else win.copy()
        bx, by = psf.border
        work.pad_pixel(bx, by)
        lanczos = "lanczos" in comp.psf_subpixel_shift
        if comp.psf_subpixel_shift != "none":
            if comp.psf_subpixel_shift != "bilinear" and not lanczos:
                raise ValueError(f"unsupported subpixel shift {comp.psf_subpixel_shift}")
            pcx, pcy = work.plane_to_pixel(center[0], center[1])
            pc = np.array([pcx, pcy])
            shift = pc - np.round(pc)
            work.pixel_shift(shift)
            center_partials_from_coords = False
        else:
            shift = None
        reference, deep = sample_init(comp, work, center, grad)
        deep, select = sample_integrate(comp, deep, reference, work, center, grad)
        if shift is not None and lanczos:
            order = int(comp.psf_subpixel_shift[comp.psf_subpixel_shift.find(":") + 1 :])
            spsf, dsx, dsy = shift_psf_lanczos(psf.data, shift, order, grad)
        elif shift is not None:
            spsf, dsx, dsy = shift_psf_bilinear(psf.data, shift, grad)
        else:
            spsf, dsx, dsy = psf.data.copy(), None, None
        norm = np.sum(spsf)
        kern = spsf / norm
        conv = convolve_fft_semantics if comp.psf_convolve_mode == "fft" else convolve_direct_semantics
        if comp.psf_convolve_mode not in ("fft", "direct"):
            raise ValueError(f"unrecognized psf_convolve_mode: {comp.psf_convolve_mode}")
        ny, nx = deep.val.shape

        def finish(a):
            return _reduce(conv(a, kern)[by : ny - by, bx : nx - bx], upscale)

        model = finish(deep.val)
        jac = None
        if grad:
            jac = _component_partials(comp, deep, finish, center_partials_from_coords, work)
            if shift is not None:
                # d kern / d shift through the renormalisation (models/_model_methods.py:243)
                dk = []
                for d in (dsx, dsy):
                    dk.append(d / norm - spsf * np.sum(d) / norm**2)
                Pi = np.linalg.inv(work.P)  # d shift / d center = P^-1 (plane_to_pixel)
                dmod = [_reduce(conv(deep.val, k)[by : ny - by, bx : nx - bx], upscale) for k in dk]
                jac[("center", 0)] = dmod[0] * Pi[0, 0] + dmod[1] * Pi[1, 0]
                jac[("center", 1)] = dmod[0] * Pi[0, 1] + dmod[1] * Pi[1, 1]
            for name, D in (psf_dirs or {}).items():
                if shift is None:
                    SD = D
                elif lanczos:
                    SD = shift_psf_lanczos(D, shift, order, False)[0]
                else:
                    SD = shift_psf_bilinear(D, shift, False)[0]
                dk = SD / norm - spsf * np.sum(SD) / norm**2
                jac[("psf", name)] = _reduce(conv(deep.val, dk)[by : ny - by, bx : nx - bx], upscale)
        return Rendered(model, jac, select, (ny, nx))

    reference, deep = sample_init(comp, win.copy(), center, grad)
    deep, select = sample_integrate(comp, deep, reference, win.copy(), center, grad)
    model = deep.val
    jac = _component_partials(comp, deep, lambda a: a, True, win) if grad else None
    return Rendered(model, jac, select, model.shape)


def _reduce(img, upscale):
    """``Image.reduce``: sum upscale x upscale blocks (image/image_object.py:327-350)."""
    if upscale == 1:
        return img
    ny, nx = img.shape
    MS, NS = ny // upscale, nx // upscale
    return img[: MS * upscale, : NS * upscale].reshape(MS, upscale, NS, upscale).sum(axis=(1, 3))


def _component_partials(comp, deep: Sampled, finish, center_from_coords, win):
    jac = {}
    g = deep.grad
    zero = np.zeros_like(deep.val)
    for name in comp.param_names:
        if name == "center":
            if center_from_coords:
                gx = g["X"] if g["X"] is not None else zero
                gy = g["Y"] if g["Y"] is not None else zero
                # X = x - cx, Y = y - cy
                jac[("center", 0)] = finish(-gx)
                jac[("center", 1)] = finish(-gy)
            else:
                jac[("center", 0)] = finish(zero)
                jac[("center", 1)] = finish(zero)
        else:
            gv = g[name] if g[name] is not None else zero
            jac[(name, 0)] = finish(gv)
    return jac


def sub_window(win: Window, pix) -> Window:
    """The window of pixels [[x0, x1], [y0, y1]] of ``win`` (``crop_to_pixel``)."""
    (x0, x1), (y0, y1) = pix
    w = win.copy()
    w.nx, w.ny = int(x1 - x0), int(y1 - y0)
    w.ref_ij = win.ref_ij - np.array([x0, y0], dtype=np.float64)
    return w


def sample_group_parts(components: List[Component], win: Window, psf: Optional[PSF], grad=False):
    """Each component added into ``win`` (``Group_Model.sample``, models/group_model_object.py:
    183-231) and, when ``grad``, its value-space partials placed on ``win``.

    Reference quirk reproduced: inside a group a component with its own pixel window is
    *evaluated on the group's window* (``model(window=group window)`` makes the working window
    the group's, models/model_object.py:290-296, with the integration threshold and the PSF
    convolution of that larger window) and only its own window is added
    (``make_model_image`` = target[self.window & window], core_model.py:193-204); its Jacobian
    is evaluated on its own window (``self.window & window``, models/_model_methods.py:293-298).
    """
    total = np.zeros((win.ny, win.nx))
    parts = []
    for comp in components:
        if comp.window is None:
            r = sample_component(comp, win, psf, grad)
            total += r.model
            parts.append(r.jac)
            continue
        (x0, x1), (y0, y1) = comp.window
        if grad:
            r = sample_component(comp, sub_window(win, comp.window), psf, True)
            total[y0:y1, x0:x1] += r.model
            full = {}
            for key, v in r.jac.items():
                f = np.zeros((win.ny, win.nx))
                f[y0:y1, x0:x1] = v
                full[key] = f
            parts.append(full)
        else:
            r = sample_component(comp, win, psf, False)
            total[y0:y1, x0:x1] += r.model[y0:y1, x0:x1]
            parts.append(None)
    return total, parts


def sample_group(components: List[Component], win: Window, psf: Optional[PSF], grad=False, links=None):
    """``Group_Model.sample`` / ``jacobian`` (models/group_model_object.py:183-283): the model is
    the sum of the components and the Jacobian columns are the components' free parameters in
    order (``vector_identities``).  ``links`` maps (component, name) of a parameter whose node
    points at another component's node (``value = node``, param/parameter.py:480-496) to that
    (component, name): the linked node leaves the vector and its partials add into the column
    of the node it points at (``Jacobian_Image`` merges columns by identity,
    image/jacobian_image.py:36-37, 79-118)."""
    links = links or {}
    total, parts = sample_group_parts(components, win, psf, grad)
    if not grad:
        return total, None
    cols = []
    for ci, comp in enumerate(components):
        for (name, k) in comp.free_slots():
            if (ci, name) in links:
                continue
            col = parts[ci][(name, k)].copy()
            for (cj, nj), target in links.items():
                if target == (ci, name):
                    col += parts[cj][(nj, k)]
            cols.append(col)
    J = np.stack(cols, axis=-1) if cols else None
    return total, J


def gaussian_psf(sigma, img_width, pixelscale, upsample=4, normalize=True):
    """utils/initialize/construct_psf.py:8-35."""
    assert img_width % 2 == 1
    N = img_width * upsample
    g = np.linspace(-(N - 1) * pixelscale / (2 * upsample), (N - 1) * pixelscale / (2 * upsample), N)
    XX, YY = np.meshgrid(g, g)
    ZZ = np.exp(-0.5 * (XX**2 + YY**2) / sigma**2)
    ZZ = ZZ.reshape(img_width, upsample, img_width, upsample).sum(axis=(1, 3)) / (upsample**2)
    return ZZ / np.sum(ZZ) if normalize else ZZ


def moffat_psf(n, Rd, img_width, pixelscale, upsample=4, normalize=True):
    """utils/initialize/construct_psf.py:38-65."""
    assert img_width % 2 == 1
    N = img_width * upsample
    g = np.linspace(-(N - 1) * pixelscale / (2 * upsample), (N - 1) * pixelscale / (2 * upsample), N)
    XX, YY = np.meshgrid(g, g)
    ZZ = 1.0 / (1.0 + (XX**2 + YY**2) / (Rd**2)) ** n
    ZZ = ZZ.reshape(img_width, upsample, img_width, upsample).sum(axis=(1, 3)) / (upsample**2)
    return ZZ / np.sum(ZZ) if normalize else ZZ
