"""Pixel grids, windows and image containers of the render path
(``astrophot/image/``: ``window_object.py``, ``target_image.py``, ``psf_image.py``,
``model_image.py``, ``jacobian_image.py``, ``wcs.py`` PPCS).

A window is a rectangle of pixels on a plane grid ``xy = P (ij - ref_ij) + ref_xy``
(``image/wcs.py:561-584``).  Model windows given as ``[[xmin, xmax], [ymin, ymax]]`` are
sub-rectangles of their target's grid (``crop_to_pixel``, ``window_object.py:358-365``).
Pixel data are float64 host tensors ``[ny, nx]``.
"""

from __future__ import annotations

import ast

import math
from typing import Optional

import numpy as np
import torch

from . import config
from .errors import InvalidWindow, SpecificationConflict

__all__ = ("Window", "Target_Image", "PSF_Image", "Model_Image", "Jacobian_Image")


def _t(v, dtype=None):
    return torch.as_tensor(np.asarray(v), dtype=dtype or config.ap_dtype)


class Window:
    """``pixel_shape`` = (nx, ny); ``pixelscale`` 2x2; ``reference_imageij`` /
    ``reference_imagexy`` pin the grid to the plane (default (-0.5, -0.5) and (0, 0))."""

    def __init__(self, pixel_shape=None, pixelscale=1.0, reference_imageij=(-0.5, -0.5), reference_imagexy=(0.0, 0.0),
                 origin=None, **kwargs):
        if pixel_shape is None:
            raise InvalidWindow("Window needs pixel_shape")
        self.pixel_shape = np.array([int(round(float(v))) for v in pixel_shape], dtype=np.int64)
        P = np.asarray(pixelscale, dtype=np.float64)
        self.pixelscale = np.eye(2) * float(P) if P.size == 1 else P.reshape(2, 2).copy()
        self.reference_imageij = np.asarray(reference_imageij, dtype=np.float64).copy()
        self.reference_imagexy = np.asarray(reference_imagexy if origin is None else origin, dtype=np.float64).copy()

    # geometry
    @property
    def pixel_area(self):
        return abs(np.linalg.det(self.pixelscale))

    @property
    def pixel_length(self):
        return math.sqrt(self.pixel_area)

    def copy(self):
        return Window(self.pixel_shape.copy(), self.pixelscale.copy(), self.reference_imageij.copy(),
                      self.reference_imagexy.copy())

    def pixel_to_plane(self, i, j):
        d = np.array([np.asarray(i, float) - self.reference_imageij[0], np.asarray(j, float) - self.reference_imageij[1]])
        P = self.pixelscale
        return P[0, 0] * d[0] + P[0, 1] * d[1] + self.reference_imagexy[0], P[1, 0] * d[0] + P[1, 1] * d[1] + self.reference_imagexy[1]

    def plane_to_pixel(self, x, y):
        Pi = np.linalg.inv(self.pixelscale)
        dx, dy = np.asarray(x, float) - self.reference_imagexy[0], np.asarray(y, float) - self.reference_imagexy[1]
        return Pi[0, 0] * dx + Pi[0, 1] * dy + self.reference_imageij[0], Pi[1, 0] * dx + Pi[1, 1] * dy + self.reference_imageij[1]

    @property
    def origin(self):
        return np.array(self.pixel_to_plane(-0.5, -0.5))

    @property
    def center(self):
        return np.array(self.pixel_to_plane(self.pixel_shape[0] / 2 - 0.5, self.pixel_shape[1] / 2 - 0.5))

    @property
    def shape(self):
        P = self.pixelscale
        return np.array([np.linalg.norm(P @ [self.pixel_shape[0], 0]), np.linalg.norm(P @ [0, self.pixel_shape[1]])])

    def geometry_row(self):
        """The 8 doubles of this window for ``ap_batch_create``."""
        return np.r_[self.pixelscale.ravel(), self.reference_imageij, self.reference_imagexy]

    # sub-rectangles on a common grid
    def offset_in(self, other):
        """Integer pixel offset (di, dj) of this window's (0, 0) pixel in ``other``'s grid."""
        i, j = other.plane_to_pixel(*self.pixel_to_plane(0, 0))
        return int(round(float(i))), int(round(float(j)))

    def crop_to_pixel(self, pixels):
        """``[[xmin, xmax], [ymin, ymax]]`` in this window's pixels (window_object.py:358-365)."""
        pixels = np.asarray(pixels, dtype=np.float64)
        self.reference_imageij = self.reference_imageij - pixels[:, 0]
        self.pixel_shape = np.array([int(pixels[0, 1] - pixels[0, 0]), int(pixels[1, 1] - pixels[1, 0])])
        return self

    def __and__(self, other):
        di, dj = other.offset_in(self)
        i0, j0 = max(0, di), max(0, dj)
        i1 = min(self.pixel_shape[0], di + other.pixel_shape[0])
        j1 = min(self.pixel_shape[1], dj + other.pixel_shape[1])
        return self.copy().crop_to_pixel([[i0, max(i0, i1)], [j0, max(j0, j1)]])

    def __or__(self, other):
        di, dj = other.offset_in(self)
        i0, j0 = min(0, di), min(0, dj)
        i1 = max(self.pixel_shape[0], di + other.pixel_shape[0])
        j1 = max(self.pixel_shape[1], dj + other.pixel_shape[1])
        return self.copy().crop_to_pixel([[i0, i1], [j0, j1]])

    def get_self_indices(self, other):
        """Index slices (rows, cols) of ``other`` inside this window (window_object.py:241-261)."""
        di, dj = other.offset_in(self)
        return (slice(max(0, dj), min(self.pixel_shape[1], dj + other.pixel_shape[1])),
                slice(max(0, di), min(self.pixel_shape[0], di + other.pixel_shape[0])))

    def __eq__(self, other):
        return (isinstance(other, Window) and np.array_equal(self.pixel_shape, other.pixel_shape)
                and np.allclose(self.pixelscale, other.pixelscale) and other.offset_in(self) == (0, 0))

    def get_state(self):
        return {"pixel_shape": self.pixel_shape.tolist(), "pixelscale": self.pixelscale.tolist(),
                "reference_imageij": self.reference_imageij.tolist(), "reference_imagexy": self.reference_imagexy.tolist()}

    def __repr__(self):
        return f"Window(pixel_shape={self.pixel_shape.tolist()}, origin={self.origin.tolist()})"


class PSF_Image:
    """An odd-shaped PSF stamp (``image/psf_image.py:17-93``)."""

    def __init__(self, data=None, pixelscale=1.0, **kwargs):
        self.data = _t(data)
        if any(s % 2 != 1 for s in self.data.shape):
            raise SpecificationConflict(f"psf must have odd shape, not {tuple(self.data.shape)}")
        P = np.asarray(pixelscale, dtype=np.float64)
        self.pixelscale = np.eye(2) * float(P) if P.size == 1 else P.reshape(2, 2)

    @property
    def pixel_length(self):
        return math.sqrt(abs(np.linalg.det(self.pixelscale)))

    @property
    def psf_border_int(self):
        ky, kx = self.data.shape
        return np.array([math.ceil((1 + kx) / 2), math.ceil((1 + ky) / 2)])

    def normalize(self):
        self.data /= torch.sum(self.data)


class _Image:
    def __init__(self, data, window: Window):
        self.data = data
        self.window = window

    @property
    def pixel_area(self):
        return self.window.pixel_area

    @property
    def pixelscale(self):
        return self.window.pixelscale

    def flatten(self, attribute="data"):
        return getattr(self, attribute).reshape(-1)

    def plane_to_pixel(self, x, y=None):
        if y is None:
            x, y = x
        return np.array(self.window.plane_to_pixel(x, y))

    def pixel_to_plane(self, i, j=None):
        if j is None:
            i, j = i
        return np.array(self.window.pixel_to_plane(i, j))


class Target_Image(_Image):
    """Data with optional variance/weight, mask and PSF (``image/target_image.py:17-342``)."""

    def __init__(self, data=None, pixelscale=1.0, psf=None, variance=None, weight=None, mask=None, zeropoint=None,
                 origin=None, window=None, psf_upscale=1, filename=None, **kwargs):
        if filename is not None:
            self._load_states(filename)
            return
        data = _t(data)
        if window is None:
            window = Window((data.shape[1], data.shape[0]), pixelscale, origin=origin)
        super().__init__(data, window)
        self.zeropoint = zeropoint
        self._weight = None
        if weight is not None:
            self.weight = weight
        elif variance is not None:
            self.variance = variance
        self._mask = None if mask is None else torch.as_tensor(np.asarray(mask), dtype=torch.bool)
        if torch.any(torch.isnan(self.data)):
            nanm = torch.isnan(self.data)
            self._mask = nanm if self._mask is None else (self._mask | nanm)
        if psf is None or isinstance(psf, PSF_Image):
            self.psf = psf
        else:
            self.psf = PSF_Image(psf, pixelscale=self.window.pixelscale / psf_upscale)

    @property
    def has_variance(self):
        return self._weight is not None

    has_weight = has_variance

    @property
    def weight(self):
        return self._weight if self._weight is not None else torch.ones_like(self.data)

    @weight.setter
    def weight(self, w):
        w = _t(w)
        if w.shape != self.data.shape:
            raise SpecificationConflict(f"weight/variance must have same shape as data ({tuple(w.shape)} vs {tuple(self.data.shape)})")
        self._weight = w

    @property
    def variance(self):
        if self._weight is None:
            return torch.ones_like(self.data)
        return torch.where(self._weight == 0, torch.inf, 1 / self._weight)

    @variance.setter
    def variance(self, v):
        self.weight = 1 / _t(v)

    @property
    def has_mask(self):
        return self._mask is not None

    @property
    def mask(self):
        return self._mask if self._mask is not None else torch.zeros_like(self.data, dtype=torch.bool)

    @property
    def has_psf(self):
        return self.psf is not None

    def __getitem__(self, window: Window):
        """The part of this target inside ``window`` (same grid)."""
        sub = self.window & window
        rows, cols = self.window.get_self_indices(sub)
        out = Target_Image(self.data[rows, cols].clone(), window=sub, psf=self.psf, zeropoint=self.zeropoint)
        if self._weight is not None:
            out._weight = self._weight[rows, cols].clone()
        if self._mask is not None:
            out._mask = self._mask[rows, cols].clone()
        return out

    def model_image(self, window: Optional[Window] = None):
        w = self.window if window is None else window
        return Model_Image(torch.zeros((int(w.pixel_shape[1]), int(w.pixel_shape[0])), dtype=config.ap_dtype), w.copy())

    def copy(self):
        out = Target_Image(self.data.clone(), window=self.window.copy(), psf=self.psf, zeropoint=self.zeropoint)
        out._weight = None if self._weight is None else self._weight.clone()
        out._mask = None if self._mask is None else self._mask.clone()
        return out

    # -- FITS (image/image_object.py:400-428, image/target_image.py:503-532) -------------------
    @staticmethod
    def _window_keys(w: Window, shape_xy):
        return {"PROJ": "gnomonic", "REFRADEC": str([0.0, 0.0]), "REFPLNXY": str([0.0, 0.0]),
                "PXLSCALE": str(np.asarray(w.pixelscale, dtype=np.float64).tolist()),
                "REFIMGIJ": str(np.asarray(w.reference_imageij, dtype=np.float64).tolist()),
                "REFIMGXY": str(np.asarray(w.reference_imagexy, dtype=np.float64).tolist()),
                "PXL_SHPE": str([float(v) for v in shape_xy])}

    def get_fits_state(self):
        """[(data, header)]: PRIMARY (with the window and zeropoint keys), WEIGHT, MASK, PSF."""
        head = self._window_keys(self.window, self.window.pixel_shape)
        if self.zeropoint is not None:
            head["ZEROPNT"] = str(float(self.zeropoint))
        head["IMAGE"] = "PRIMARY"
        states = [(self.data.detach().cpu().numpy().astype(np.float64), head)]
        if self.has_weight:
            states.append((self._weight.detach().cpu().numpy().astype(np.float64), {"IMAGE": "WEIGHT"}))
        if self.has_mask:
            states.append((self._mask.detach().cpu().numpy().astype(np.int64), {"IMAGE": "MASK"}))
        if self.has_psf:
            ky, kx = self.psf.data.shape
            pw = Window((kx, ky), self.psf.pixelscale)
            ph = self._window_keys(pw, (kx, ky))
            ph["IMAGE"] = "PSF"
            states.append((self.psf.data.detach().cpu().numpy().astype(np.float64), ph))
        return states

    def save(self, filename=None, overwrite=True):
        """Write the HDU list the reference writes (primary image + WEIGHT / MASK / PSF images)."""
        import os

        from .fits_io import write_hdus

        if filename is None:
            return self.get_fits_state()
        if os.path.exists(filename) and not overwrite:
            raise OSError(f"{filename} exists")
        write_hdus(filename, self.get_fits_state())
        return self.get_fits_state()

    def _load_states(self, filename):
        from .fits_io import read_hdus

        hdus = read_hdus(filename)
        prim = next((d, h) for d, h in hdus if str(h.get("IMAGE", "")).strip() == "PRIMARY")
        data, head = prim
        lit = ast.literal_eval  # the reference writes Python list literals into these keys
        P = np.array(lit(str(head["PXLSCALE"])), dtype=np.float64)
        shape = [int(round(v)) for v in lit(str(head["PXL_SHPE"]))]
        w = Window(shape, P, reference_imageij=lit(str(head["REFIMGIJ"])), reference_imagexy=lit(str(head["REFIMGXY"])))
        _Image.__init__(self, _t(np.asarray(data, dtype=np.float64)), w)
        self.zeropoint = float(lit(str(head["ZEROPNT"]))) if "ZEROPNT" in head else None
        self._weight = None
        self._mask = None
        self.psf = None
        for d, h in hdus:
            tag = str(h.get("IMAGE", "")).strip()
            if tag == "WEIGHT":
                self._weight = _t(np.asarray(d, dtype=np.float64))
            # the reference's set_fits_state looks for "mask" in lower case while it writes
            # "MASK" (image/target_image.py:517, 529): a saved mask does not come back on load
            if tag == "mask":
                self._mask = torch.as_tensor(np.asarray(d, dtype=bool))
            if tag == "PSF":
                Pp = np.array(lit(str(h["PXLSCALE"])), dtype=np.float64)
                self.psf = PSF_Image(np.asarray(d, dtype=np.float64), pixelscale=Pp)

    def load(self, filename):
        self._load_states(filename)


class Model_Image(_Image):
    """Model pixels on a window (``image/model_image.py``); ``+=`` adds by window overlap
    (``image/image_object.py:450-457``)."""

    def __init__(self, data=None, window: Window = None, **kwargs):
        if data is None:
            data = torch.zeros((int(window.pixel_shape[1]), int(window.pixel_shape[0])), dtype=config.ap_dtype)
        super().__init__(_t(data), window)

    def __iadd__(self, other):
        if isinstance(other, _Image):
            rs, cs = self.window.get_self_indices(other.window)
            ro, co = other.window.get_self_indices(self.window)
            self.data[rs, cs] += other.data[ro, co]
        else:
            self.data += other
        return self

    def blank_copy(self):
        return Model_Image(torch.zeros_like(self.data), self.window.copy())

    def copy(self):
        return Model_Image(self.data.clone(), self.window.copy())


class Jacobian_Image(_Image):
    """d(model)/d(parameter) planes ``[ny, nx, P]`` with the parameter identities
    (``image/jacobian_image.py:13-118``)."""

    def __init__(self, parameters, data, window: Window, **kwargs):
        super().__init__(_t(data), window)
        self.parameters = list(parameters)

    def flatten(self, attribute="data"):
        d = getattr(self, attribute)
        return d.reshape(-1, d.shape[-1])

    def __iadd__(self, other):
        """Columns merged by parameter identity; shared parameters sum."""
        rs, cs = self.window.get_self_indices(other.window)
        ro, co = other.window.get_self_indices(self.window)
        for k, pid in enumerate(other.parameters):
            if pid not in self.parameters:
                self.parameters.append(pid)
                self.data = torch.cat([self.data, torch.zeros((*self.data.shape[:2], 1), dtype=self.data.dtype)], dim=-1)
            self.data[rs, cs, self.parameters.index(pid)] += other.data[ro, co, k]
        return self
