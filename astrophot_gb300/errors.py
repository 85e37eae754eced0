"""Exception types the drop-in keeps raising, with the reference's names and hierarchy
(``astrophot/errors/base.py:6-30``, ``fit.py:6``, ``param.py:6``, ``models.py:6-22``,
``image.py:9-40``)."""


class AstroPhotError(Exception):
    """Base exception for all AstroPhot processes."""


class NameNotAllowed(AstroPhotError):
    """Invalid name of an AstroPhot object."""


class SpecificationConflict(AstroPhotError):
    """Conflicting or ambiguous inputs (unknown sampling / integration / PSF modes)."""


class OptimizeStop(AstroPhotError):
    """Raised to stop an optimisation (LM found no step that improves chi^2)."""


class InvalidParameter(AstroPhotError):
    """A parameter was assigned incorrectly, e.g. outside its limits."""


class InvalidModel(AstroPhotError):
    """A model object is inappropriate for this use."""


class InvalidTarget(AstroPhotError):
    """A target object was assigned incorrectly."""


class UnrecognizedModel(AstroPhotError):
    """Unknown model_type string."""


class InvalidWindow(AstroPhotError):
    """A window is misspecified."""


class ConflicingWCS(InvalidWindow):
    """Windows compared with WCS prescriptions that do not agree."""


class InvalidData(AstroPhotError):
    """An image cannot determine the data it holds."""


class InvalidImage(AstroPhotError):
    """An image object cannot be used as given."""
