"""Fitted parametric PSFs restated in float64 numpy.  TEST INFRASTRUCTURE ONLY (the checker
of the CUDA path's live PSF models; see ``oracle/__init__``).

* ``render_psf``: a Moffat (models/moffat_model.py:71-120) or Gaussian
  (models/gaussian_model.py:255-290) PSF model sampled on its PSF image and normalised to unit sum
  (``PSF_Model.sample``, astrophot/models/psf_model_object.py:180-264, with the class knobs of
  psf_model_object.py:50-80: Simpson sampling, tolerance 1e-3, threshold integration), and the
  derivatives of the normalised image with respect to the PSF parameters.
* ``LivePSFProblem``: a galaxy convolved with that live PSF, the PSF's free parameters joining
  the galaxy's in one LM vector (``set_aux_psf``, models/model_object.py:133-149; the PSF image
  is sampled from its parameters at every evaluation, model_object.py:306-312).  The linked PSF
  node is added to the galaxy's parameters before the galaxy's own, so the PSF parameters lead
  the vector.  It has the interface ``LMOracle`` expects.

Pinned by ``tests/golden/auxpsf_48.npz`` (Moffat) and ``auxpsf_gauss_48.npz`` (Gaussian),
recorded from the reference itself.
"""

from __future__ import annotations

import copy
from typing import Dict, Optional, Sequence

import numpy as np

from .render import PSF, Component, Window, check_limits, drep_dvalue, rep_to_value, sample_component, value_to_rep

# PSF_Model class attributes (astrophot/models/psf_model_object.py:50-80)
PSF_KNOBS = dict(sampling_mode="simpsons", sampling_tolerance=1e-3, integrate_mode="threshold",
                 integrate_max_depth=3, integrate_gridding=5, integrate_quad_level=3, softening=1e-3)
PSF_ORDER = {"moffat": ("n", "Rd", "I0"), "gaussian": ("sigma", "flux")}
DEFAULT_FREE = {"moffat": ("n", "Rd"), "gaussian": ("sigma",)}


def psf_window(kx: int, ky: int, scale: float = 1.0) -> Window:
    """The pixel grid of a PSF_Image: centred on the plane origin (image/psf_image.py:17-60)."""
    return Window(kx, ky, np.eye(2) * float(scale), np.array([(kx - 1) / 2, (ky - 1) / 2]), np.zeros(2))


def render_psf(params: Dict[str, float], shape, scale: float = 1.0, grad: bool = False,
               free: Optional[Sequence[str]] = None, kind: str = "moffat"):
    """(K / sum K, {name: d(K / sum K) / d name}) of a Moffat or Gaussian PSF model on a
    ``shape`` = (ky, kx) PSF image."""
    ky, kx = shape
    free = DEFAULT_FREE[kind] if free is None else free
    comp = Component(kind, {"center": np.zeros(2), **{k: params[k] for k in PSF_ORDER[kind]}}, **PSF_KNOBS)
    r = sample_component(comp, psf_window(kx, ky, scale), None, grad)
    S = np.sum(r.model)
    Kn = r.model / S
    if not grad:
        return Kn, {}
    dK = {}
    for name in free:
        d = r.jac[(name, 0)]
        dK[name] = d / S - Kn * np.sum(d) / S
    return Kn, dK


class LivePSFProblem:
    """One galaxy (``psf_mode`` "full") with a live Moffat or Gaussian PSF (``psf_kind``) on
    ``window``, against data ``Y`` with weights ``W``; ``sky`` (counts per pixel) is a locked
    flat sky of the same group (``Group_Model`` of the galaxy and a ``Flat_Sky``,
    models/group_model_object.py:183-231, flatsky_model.py:53-55)."""

    def __init__(self, galaxy: Component, window: Window, psf_params: Dict[str, float], psf_shape,
                 Y: np.ndarray, W: Optional[np.ndarray] = None, psf_scale: float = 1.0,
                 psf_free: Optional[Sequence[str]] = None, mask: Optional[np.ndarray] = None,
                 psf_kind: str = "moffat", sky: float = 0.0):
        self.galaxy = copy.deepcopy(galaxy)
        self.window = window
        self.psf_params = {k: float(v) for k, v in psf_params.items()}
        self.psf_shape = tuple(psf_shape)
        self.psf_scale = float(psf_scale)
        self.psf_kind = psf_kind
        self.sky = float(sky)
        self.psf_free = tuple(DEFAULT_FREE[psf_kind] if psf_free is None else psf_free)
        self.Y, self.W, self.mask = Y, W, mask
        self.slots = [("psf", name, 0) for name in self.psf_free] + [("gal", name, k)
                                                                    for name, k in self.galaxy.free_slots()]

    def _kind(self, who):
        return self.psf_kind if who == "psf" else None

    def _get(self, who, name, k):
        if who == "psf":
            return self.psf_params[name]
        return float(np.atleast_1d(self.galaxy.params[name])[k])

    def values(self):
        return np.array([self._get(*s) for s in self.slots])

    def representation(self):
        return np.array([value_to_rep(name, self._get(who, name, k), self._kind(who)) for who, name, k in self.slots])

    def set_representation(self, rep):
        for (who, name, k), r in zip(self.slots, rep):
            v = float(rep_to_value(name, r, self._kind(who)))
            check_limits(name, v, self._kind(who))
            if who == "psf":
                self.psf_params[name] = v
            elif name == "center":
                arr = np.array(self.galaxy.params["center"], dtype=float).copy()
                arr[k] = v
                self.galaxy.params["center"] = arr
            else:
                self.galaxy.params[name] = np.asarray(v, dtype=float)

    def psf_image(self, grad=False):
        return render_psf(self.psf_params, self.psf_shape, self.psf_scale, grad, self.psf_free, self.psf_kind)

    def forward(self, rep):
        self.set_representation(rep)
        K, _ = self.psf_image()
        return sample_component(self.galaxy, self.window, PSF(K, self.psf_scale)).model.reshape(-1) + self.sky

    def jacobian_values(self):
        K, dK = self.psf_image(grad=True)
        r = sample_component(self.galaxy, self.window, PSF(K, self.psf_scale), True, psf_dirs=dK)
        cols = [r.jac[("psf", name)] if who == "psf" else r.jac[(name, k)] for who, name, k in self.slots]
        return np.stack(cols, axis=-1)

    def jacobian(self, rep):
        """Representation-space Jacobian [N, P]."""
        self.set_representation(rep)
        J = self.jacobian_values()
        scale = np.array([drep_dvalue(name, r, self._kind(who)) for (who, name, k), r in zip(self.slots, rep)])
        return J.reshape(-1, J.shape[-1]) * scale[None, :]
