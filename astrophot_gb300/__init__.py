"""GB300-native render + Levenberg-Marquardt path for AstroPhot models.

Drop-in surface (mirrors ``astrophot``): ``models`` (``AstroPhot_Model`` factory,
``Sersic_Galaxy``, ``Exponential_Galaxy``, ``Flat_Sky``, ``Group_Model``), ``image``
(``Target_Image``, ``PSF_Image``, ``Window``, ``Model_Image``, ``Jacobian_Image``),
``param`` (``Parameter_Node`` and its contexts), ``fit`` (``LM``, ``BatchLM``, ``Iter_LM``), ``errors``,
``utils`` and ``AP_config``.  Every render, Jacobian and fit runs in the CUDA library
(``libastrophot_gb300.so``, C ABI in ``include/astrophot_gb300.h``); using them without the
built library raises ImportError.
"""

from . import config as AP_config  # noqa: F401
from . import autograd, errors, fit, image, models, param, utils  # noqa: F401

__version__ = "0.1.0"
