"""Helpers mirroring ``astrophot.utils`` for the render path: PSF stamp constructors
(``utils/initialize/construct_psf.py:8-65``), the Sersic b(n) polynomial
(``utils/conversions/functions.py:7-22``) and the segmentation-map window helpers
(``utils/initialize/segmentation_map.py``, in ``segmap.py``)."""

from types import SimpleNamespace

from .synthetic import gaussian_stamp as _gaussian_stamp
from .synthetic import moffat_stamp as _moffat_stamp


def moffat_psf(n, Rd, img_width, pixelscale, upsample=4, normalize=True):
    """4x4 super-sampled Moffat stamp with index n (beta) and core radius Rd, normalised."""
    return _moffat_stamp(n, Rd, img_width, pixelscale, upsample)


def gaussian_psf(sigma, img_width, pixelscale, upsample=4, normalize=True):
    """4x4 super-sampled Gaussian stamp, normalised."""
    return _gaussian_stamp(sigma, img_width, pixelscale, upsample)


def sersic_n_to_b(n):
    return (2 * n - 1 / 3 + 4 / (405 * n) + 46 / (25515 * n**2) + 131 / (1148175 * n**3)
            - 2194697 / (30690717750 * n**4))


from . import segmap as _segmap  # noqa: E402

initialize = SimpleNamespace(moffat_psf=moffat_psf, gaussian_psf=gaussian_psf,
                             segmentation_map=_segmap,
                             **{name: getattr(_segmap, name) for name in _segmap.__all__})
conversions = SimpleNamespace(functions=SimpleNamespace(sersic_n_to_b=sersic_n_to_b))
