"""Model classes with the reference's construction API (``astrophot/models/``).

``AstroPhot_Model(model_type=...)`` builds ``Sersic_Galaxy`` ("sersic galaxy model"),
``Exponential_Galaxy`` ("exponential galaxy model"), ``Flat_Sky`` ("flat sky model"),
``Moffat_PSF`` ("moffat psf model", a live PSF when given as a galaxy's ``psf``) or
``Group_Model`` ("group model") with the same parameters, limits, sampling knobs and
defaults as the reference (``models/core_model.py:98-115``, ``model_object.py:57-111``,
``galaxy_model_object.py:44-53``, ``sersic_model.py:61-66``, ``exponential_model.py:58-62``,
``flatsky_model.py:23-26``, ``sky_model_object.py:16-35``, ``group_model_object.py``).

Every image, Jacobian and fit is computed by the CUDA library through its C ABI
(``_native``): a galaxy, alone or in a group with a flat sky, is one stamp of a
``StampBatch`` whose window is the model's window.  There is no CPU fallback.
"""

from __future__ import annotations

import math
from copy import deepcopy
from typing import Optional

import numpy as np
import torch

from . import config
from .errors import InvalidTarget, NameNotAllowed, SpecificationConflict, UnrecognizedModel, InvalidWindow
from .image import Jacobian_Image, Model_Image, PSF_Image, Target_Image, Window
from .param import Param_SoftLimits, Param_Unlock, Parameter_Node

__all__ = (
    "AstroPhot_Model",
    "Component_Model",
    "Galaxy_Model",
    "Sersic_Galaxy",
    "Exponential_Galaxy",
    "Sky_Model",
    "Flat_Sky",
    "Group_Model",
    "PSF_Model",
    "Moffat_PSF",
    "Gaussian_PSF",
)

# full parameter-vector slots of the C ABI
SLOT = {"center": (0, 1), "q": (2,), "PA": (3,), "n": (4,), "Re": (5,), "Ie": (6,), "F": (7,)}


def _all_subclasses(cls):
    return set(cls.__subclasses__()).union(s for c in cls.__subclasses__() for s in _all_subclasses(c))


class AstroPhot_Model:
    """Factory and common plumbing (``models/core_model.py:26-502``)."""

    model_type = "model"
    model_names = []
    special_kwargs = ["parameters", "filename", "model_type", "usable"]
    usable = False

    def __new__(cls, *, filename=None, model_type=None, **kwargs):
        if model_type is not None:
            for M in _all_subclasses(AstroPhot_Model):
                if M.model_type == model_type:
                    return super(AstroPhot_Model, cls).__new__(M)
            raise UnrecognizedModel(f"Unknown AstroPhot model type: {model_type}")
        return super().__new__(cls)

    def __init__(self, *, name=None, target=None, window=None, locked=False, **kwargs):
        self._window = None
        self._target = None
        self.name = name
        self.parameters = Parameter_Node(self.name)
        self.target = target
        self.window = window
        self._locked = locked
        self.mask = kwargs.get("mask", None)
        for k, v in kwargs.items():
            if k in self.special_kwargs:
                continue
            setattr(self, k, v)

    # names --------------------------------------------------------------------------------
    @property
    def name(self):
        return self._name

    @name.setter
    def name(self, name):
        if name is None:
            i = 0
            while f"{self.model_type} [{i}]" in AstroPhot_Model.model_names:
                i += 1
            name = f"{self.model_type} [{i}]"
        if ":" in name or "|" in name:
            raise NameNotAllowed("characters '|' and ':' are reserved for internal model operations")
        self._name = name
        AstroPhot_Model.model_names.append(name)

    # target / window ---------------------------------------------------------------------
    @property
    def target(self):
        return self._target

    @target.setter
    def target(self, tar):
        if not (tar is None or isinstance(tar, Target_Image)):
            raise InvalidTarget("AstroPhot_Model target must be a Target_Image instance.")
        self._target = tar

    @property
    def window(self):
        if self._window is None:
            if self.target is None:
                raise ValueError("This model has no target or window, these must be provided by the user")
            return self.target.window.copy()
        return self._window

    @window.setter
    def window(self, window):
        if window is None:
            self._window = None
        elif isinstance(window, Window):
            self._window = window
        elif len(window) == 2:
            self._window = self.target.window.copy().crop_to_pixel(window)
        else:
            raise InvalidWindow(f"Unrecognized window format: {window}")

    @property
    def locked(self):
        return self._locked

    @locked.setter
    def locked(self, val):
        self._locked = val

    def __getitem__(self, key):
        return self.parameters[key]

    def __contains__(self, key):
        return key in self.parameters

    def make_model_image(self, window: Optional[Window] = None):
        w = self.window if window is None else (self.window & window)
        return self.target.model_image(w)

    def __call__(self, image=None, parameters=None, window=None, as_representation=False, **kwargs):
        """``core_model.py:484-502``: a tensor ``parameters`` is written into the model first."""
        if isinstance(parameters, (torch.Tensor, np.ndarray, list, tuple)):
            if as_representation:
                self.parameters.vector_set_representation(parameters)
            else:
                self.parameters.vector_set_values(parameters)
            parameters = None
        return self.sample(image=image, window=window, parameters=parameters, **kwargs)

    # the model's own render components (one galaxy and/or one flat sky)
    def _components(self):
        return [self]

    # reverse-mode center gradients as the reference's autograd gives them under PSF shift
    # (sub-pixel PSF shift path + sampling-coordinate path); False = the render's derivative
    reference_center_gradient = True

    def negative_log_likelihood(self, parameters=None, as_representation=False):
        """``core_model.py:220-256``: sum over unmasked pixels of W (model - data)^2 / 2.

        A ``parameters`` tensor that requires grad makes the result differentiable: its
        backward is the library's adjoint (``ap_render_vjp``) of the CUDA render."""
        if isinstance(parameters, torch.Tensor) and parameters.requires_grad:
            return _NLLFunction.apply(parameters, self, bool(as_representation))
        if parameters is not None:
            (self.parameters.vector_set_representation if as_representation else self.parameters.vector_set_values)(parameters)
        model = self.sample()
        data = self.target[self.window]
        r = (model.data - data.data) ** 2 * data.weight
        if data.has_mask:
            r = r[torch.logical_not(data.mask)]
        return torch.sum(r) / 2.0

    def get_state(self):
        return {"name": self.name, "model_type": self.model_type, "parameters": self.parameters.get_state()}

    @classmethod
    def List_Model_Names(cls, usable=None):
        return sorted(M.model_type for M in _all_subclasses(cls) if usable is None or M.usable is usable)


class Component_Model(AstroPhot_Model):
    """Single-component model with the reference's sampling knobs (``model_object.py:25-111``)."""

    parameter_specs = {"center": {"units": "arcsec", "uncertainty": [0.1, 0.1]}}
    _parameter_order = ("center",)
    psf_mode = "none"
    psf_convolve_mode = "fft"
    psf_subpixel_shift = "bilinear"
    sampling_mode = "midpoint"
    sampling_tolerance = 1e-2
    integrate_mode = "threshold"
    integrate_max_depth = 3
    integrate_gridding = 5
    integrate_quad_level = 3
    jacobian_chunksize = 10
    image_chunksize = 1000
    softening = 1e-3
    usable = False

    def __init__(self, *, name=None, **kwargs):
        self._psf = None
        super().__init__(name=name, **kwargs)
        specs = self.build_parameter_specs(kwargs.get("parameters", None))
        for p in self.__class__._parameter_order:
            spec = specs[p]
            if isinstance(spec, Parameter_Node):
                self.parameters.link(spec)
            else:
                self.parameters.link(Parameter_Node(p, **spec))
        self._plans = {}

    @classmethod
    def build_parameter_specs(cls, user_specs=None):
        """``_model_methods.py:43-65``."""
        specs = {}
        for base in reversed(cls.__mro__):
            if "parameter_specs" in base.__dict__:
                specs.update(deepcopy(base.__dict__["parameter_specs"]))
        if isinstance(user_specs, dict):
            for p, v in user_specs.items():
                if isinstance(v, Parameter_Node):
                    specs[p] = v
                elif isinstance(v, dict):
                    specs[p].update(v)
                else:
                    specs[p]["value"] = v
        return specs

    @property
    def psf(self):
        if self._psf is None:
            return None if self.target is None else self.target.psf
        return self._psf

    @psf.setter
    def psf(self, val):
        if val is None or isinstance(val, PSF_Image):
            self._psf = val
        elif isinstance(val, PSF_Model):
            self.set_aux_psf(val)
        else:
            self._psf = PSF_Image(val, pixelscale=self.target.pixelscale)

    def set_aux_psf(self, aux_psf, add_parameters=True):
        """``set_aux_psf`` (``model_object.py:133-149``): a PSF model sampled at every evaluation,
        its parameters linked into this model's (ahead of the model's own, which are added
        after the constructor's keyword arguments)."""
        self._psf = aux_psf
        if add_parameters:
            self.parameters.link(aux_psf.parameters)

    @torch.no_grad()
    def initialize(self, target=None, parameters=None, **kwargs):
        """Centre defaults to the window centre (``model_object.py:180-205``); the reference's
        profile heuristics are not part of this path, so other parameters must be given."""
        c = self.parameters["center"]
        if c.value is None:
            with Param_Unlock(c), Param_SoftLimits(c):
                c.value = self.window.center
        missing = [p for p in self._parameter_order if self.parameters[p].value is None]
        if missing:
            raise SpecificationConflict(f"{self.name}: parameters without values: {sorted(set(missing))}")

    # ---- rendering through the C ABI ----------------------------------------------------
    def sample(self, image=None, window=None, parameters=None):
        """``Component_Model.sample`` (``model_object.py:258-375``) on the CUDA path."""
        return _sample_structure(self, [self], image, window)

    def jacobian(self, parameters=None, as_representation=False, window=None, pass_jacobian=None, **kwargs):
        """``_model_methods.py:260-347``: d(model)/d(vector) on the model window."""
        if parameters is not None:
            (self.parameters.vector_set_representation if as_representation else self.parameters.vector_set_values)(parameters)
        return _jacobian_structure(self, [self], as_representation, window)


class Galaxy_Model(Component_Model):
    """q in (0, 1), PA cyclic in [0, pi) (``galaxy_model_object.py:21-53``)."""

    model_type = f"galaxy {Component_Model.model_type}"
    parameter_specs = {
        "q": {"units": "b/a", "limits": (0, 1), "uncertainty": 0.03},
        "PA": {"units": "radians", "limits": (0, math.pi), "cyclic": True, "uncertainty": 0.06},
    }
    _parameter_order = Component_Model._parameter_order + ("q", "PA")
    usable = False

    @torch.no_grad()
    def initialize(self, target=None, parameters=None, **kwargs):
        """``initialize()`` of a Sérsic / exponential galaxy on the CUDA path
        (``ap_reference_init``): every parameter without a value gets the reference's own
        heuristic value, the centre of light (``model_object.py:180-233``), the angular centre
        PA and the flattest-isophote q (``galaxy_model_object.py:60-113``), and n / Re / Ie from
        Nelder-Mead on the binned median profile (``_shared_methods.py:123-166``); parameters
        with values are inputs.  Uncertainties are left as they are."""
        from . import _native as N

        order = self._parameter_order
        missing = [p for p in order if self.parameters[p].value is None]
        if not missing:
            return
        target = self.target if target is None else target
        area = target[self.window]
        c = self.parameters["center"]
        if c.value is None and c.locked:  # model_object.py:209-210: the window centre, no search
            with Param_Unlock(c), Param_SoftLimits(c):
                c.value = self.window.center
        vec = np.zeros((1, 8))
        known = 0
        for name in order:
            node = self.parameters[name]
            if node.value is None:
                continue
            for k, slot in enumerate(SLOT[name]):
                vec[0, slot] = float(node.value.reshape(-1)[k])
                known |= 1 << slot
        opts = N.make_options(profile=self.profile, free_mask=0x7F if self.profile == "sersic" else 0x6F)
        w = area.window
        batch = N.StampBatch([tuple(w.pixel_shape)], None, w.geometry_row()[None, :], opts, config.ap_device)
        data = batch.pack([area.data.detach().cpu().numpy()])
        mask = batch.pack([area.mask.detach().cpu().numpy()], torch.uint8) if area.has_mask else None
        out, status = batch.reference_init(data, mask, torch.tensor(vec), known)
        if int(status.item()) & (N.INIT_NO_ISOPHOTE | N.INIT_NO_PROFILE):
            raise ValueError(f"{self.name}: unable to recover isophotes or a radial profile, provide initial values")
        out = out.cpu().numpy()[0]
        for name in missing:
            node = self.parameters[name]
            val = out[list(SLOT[name])] if len(SLOT[name]) > 1 else out[SLOT[name][0]]
            with Param_Unlock(node), Param_SoftLimits(node):
                node.value = torch.as_tensor(val, dtype=config.ap_dtype)


class PSF_Model(Component_Model):
    """A point-source profile sampled on a PSF image (``psf_model_object.py:21-264``): centred on
    the image's (0, 0), Simpson sampling at tolerance 1e-3 with threshold integration, the
    image normalised to unit sum.  Its target is a ``PSF_Image``."""

    parameter_specs = {"center": {"units": "arcsec", "value": (0.0, 0.0), "uncertainty": (0.1, 0.1),
                                  "locked": True}}
    _parameter_order = ("center",)
    model_type = f"psf {AstroPhot_Model.model_type}"
    sampling_mode = "simpsons"
    sampling_tolerance = 1e-3
    normalize_psf = True
    usable = False

    @property
    def target(self):
        return self._target

    @target.setter
    def target(self, tar):
        if not (tar is None or isinstance(tar, PSF_Image)):
            raise InvalidTarget("PSF_Model target must be a PSF_Image instance.")
        self._target = tar

    _live_kind = None  # LivePSF kind of a concrete PSF model

    def initialize(self, target=None, parameters=None, **kwargs):
        missing = [p for p in self._parameter_order[1:] if self.parameters[p].value is None]
        if missing:
            raise SpecificationConflict(f"{self.name}: parameters without values: {missing}")

    def live_psf(self, device=None):
        """A :class:`~astrophot_gb300.scene.LivePSF` at the current values; its free parameters
        are the unlocked ones of the profile's parameters."""
        from .scene import LivePSF

        if self._live_kind is None:
            raise NotImplementedError(f"{self.model_type} has no CUDA sampler")
        if self.normalize_psf is not True:
            raise NotImplementedError("an unnormalised PSF model is not supported by the CUDA path")
        if self.sampling_mode not in ("midpoint", "simpsons", "trapezoid") and not self.sampling_mode.startswith("quad"):
            raise SpecificationConflict(f"unknown sampling mode: {self.sampling_mode}")
        p = self.parameters
        names = self._parameter_order[1:]
        vals = {k: float(p[k].value.item()) for k in names}
        free = tuple(k for k in names if not p[k].locked)
        knobs = {k: getattr(self, k) for k in ("sampling_mode", "sampling_tolerance", "integrate_mode",
                                               "integrate_max_depth", "integrate_gridding", "integrate_quad_level",
                                               "softening")}
        return LivePSF(vals, tuple(self.target.data.shape), self.target.pixel_length, free, knobs,
                       config.ap_device if device is None else device, kind=self._live_kind)

    def sample(self, image=None, window=None, parameters=None):
        """``PSF_Model.sample``: the normalised PSF image, sampled on the GPU."""
        if isinstance(parameters, (torch.Tensor, np.ndarray, list, tuple)):
            self.parameters.vector_set_values(parameters)
        img = self.live_psf().image()
        return PSF_Image(torch.as_tensor(img, dtype=config.ap_dtype), pixelscale=self.target.pixelscale)

    def jacobian(self, parameters=None, as_representation=False, window=None, pass_jacobian=None, **kwargs):
        """d(normalised PSF image) / d(free parameters): [ky, kx, n_free]."""
        if parameters is not None:
            (self.parameters.vector_set_representation if as_representation else self.parameters.vector_set_values)(parameters)
        live = self.live_psf()
        _, dK = live.render(True)
        if dK is None:
            return torch.zeros(live.ky, live.kx, 0, dtype=config.ap_dtype)
        J = dK.cpu().numpy().astype(np.float64).reshape(-1, live.ky, live.kx).transpose(1, 2, 0)
        if as_representation:
            J = J * live.drep(live.representation())[None, None, :]
        return torch.as_tensor(J, dtype=config.ap_dtype)


class Moffat_PSF(PSF_Model):
    """I(R) = 10^I0 / (1 + (R/Rd)^2)^n on the PSF image (``moffat_model.py:71-120``), I0 locked
    at 0 by default.  As a galaxy's ``psf`` it is a live PSF: re-sampled from its parameters at
    every evaluation and fitted with the galaxy (``astrophot_gb300.scene.LivePSF``)."""

    model_type = f"moffat {PSF_Model.model_type}"
    parameter_specs = {
        "n": {"units": "none", "limits": (0.1, 10), "uncertainty": 0.05},
        "Rd": {"units": "arcsec", "limits": (0, None)},
        "I0": {"units": "log10(flux/arcsec^2)", "value": 0.0, "locked": True},
    }
    _parameter_order = PSF_Model._parameter_order + ("n", "Rd", "I0")
    _live_kind = "moffat"
    usable = True


class Gaussian_PSF(PSF_Model):
    """I(R) = 10^flux exp(-R^2 / (2 sigma^2)) / sqrt(2 pi sigma^2) on the PSF image
    (``gaussian_model.py:255-290``), flux locked at 0 by default; live like ``Moffat_PSF``."""

    model_type = f"gaussian {PSF_Model.model_type}"
    parameter_specs = {
        "sigma": {"units": "arcsec", "limits": (0, None)},
        "flux": {"units": "log10(flux)", "value": 0.0, "locked": True},
    }
    _parameter_order = PSF_Model._parameter_order + ("sigma", "flux")
    _live_kind = "gaussian"
    usable = True


class Sersic_Galaxy(Galaxy_Model):
    """I(R) = 10^Ie exp(-b(n) ((R/Re)^(1/n) - 1)) (``sersic_model.py:41-91``)."""

    model_type = f"sersic {Galaxy_Model.model_type}"
    parameter_specs = {
        "n": {"units": "none", "limits": (0.36, 8), "uncertainty": 0.05},
        "Re": {"units": "arcsec", "limits": (0, None)},
        "Ie": {"units": "log10(flux/arcsec^2)"},
    }
    _parameter_order = Galaxy_Model._parameter_order + ("n", "Re", "Ie")
    usable = True
    profile = "sersic"

    def total_flux(self, parameters=None, window=None):
        """``sersic_Ie_to_flux_torch`` (``utils/conversions/functions.py:168-190``)."""
        p = self.parameters
        n, Re, q, Ie = (p[k].value.item() for k in ("n", "Re", "q", "Ie"))
        bn = 2 * n - 1 / 3 + 4 / (405 * n) + 46 / (25515 * n**2) + 131 / (1148175 * n**3) - 2194697 / (30690717750 * n**4)
        return torch.tensor(2 * math.pi * 10**Ie * Re**2 * q * n * math.exp(bn) * bn ** (-2 * n) * math.exp(math.lgamma(2 * n)),
                            dtype=config.ap_dtype)


class Exponential_Galaxy(Galaxy_Model):
    """I(R) = 10^Ie exp(-b(1) (R/Re - 1)) (``exponential_model.py:40-74``)."""

    model_type = f"exponential {Galaxy_Model.model_type}"
    parameter_specs = {
        "Ie": {"units": "log10(flux/arcsec^2)"},
        "Re": {"units": "arcsec", "limits": (0, None)},
    }
    _parameter_order = Galaxy_Model._parameter_order + ("Re", "Ie")
    usable = True
    profile = "exponential"


class Sky_Model(Component_Model):
    """Locked centre, no PSF, no integration (``sky_model_object.py:6-35``)."""

    model_type = f"sky {Component_Model.model_type}"
    parameter_specs = {"center": {"units": "arcsec", "locked": True, "uncertainty": 0.0}}
    usable = False

    @property
    def psf_mode(self):
        return "none"

    @psf_mode.setter
    def psf_mode(self, val):
        pass

    @property
    def integrate_mode(self):
        return "none"

    @integrate_mode.setter
    def integrate_mode(self, val):
        pass


class Flat_Sky(Sky_Model):
    """pixel_area * 10^F everywhere (``flatsky_model.py:13-55``)."""

    model_type = f"flat {Sky_Model.model_type}"
    parameter_specs = {"F": {"units": "log10(flux/arcsec^2)"}}
    _parameter_order = Sky_Model._parameter_order + ("F",)
    usable = True

    @torch.no_grad()
    def initialize(self, target=None, parameters=None, **kwargs):
        c = self.parameters["center"]
        if c.value is None:
            with Param_Unlock(c), Param_SoftLimits(c):
                c.value = self.window.center
        F = self.parameters["F"]
        if F.value is None:
            with Param_Unlock(F), Param_SoftLimits(F):
                F.value = math.log10(abs(float(torch.median(self.target[self.window].data))) / self.target.pixel_area)


class Group_Model(AstroPhot_Model):
    """Sum of sub-models; its ``psf_mode`` is pushed onto every sub-model when they are added
    (``group_model_object.py:88, 292-297``)."""

    model_type = f"group {AstroPhot_Model.model_type}"
    usable = True

    def __init__(self, *, name=None, models=None, **kwargs):
        self._psf_mode = "none"
        self.models = {}
        super().__init__(name=name, **kwargs)
        if models is not None:
            self.add_model(models)
        self._plans = {}

    def add_model(self, model):
        if isinstance(model, (list, tuple)):
            for m in model:
                self.add_model(m)
            return
        if model.name in self.models and self.models[model.name] is not model:
            raise KeyError(f"{self.name} already has model with name {model.name}, every model must have a unique name.")
        self.models[model.name] = model
        self.parameters.link(model.parameters)
        self.psf_mode = self.psf_mode
        if model.target is None:
            model.target = self.target
        self._window = None
        self._plans = {}

    @property
    def psf_mode(self):
        return self._psf_mode

    @psf_mode.setter
    def psf_mode(self, value):
        self._psf_mode = value
        for m in getattr(self, "models", {}).values():
            m.psf_mode = value

    @property
    def window(self):
        if self._window is not None:
            return self._window
        w = None
        for m in self.models.values():
            if m.locked:
                continue
            w = m.window.copy() if w is None else (w | m.window)
        if w is None:
            return self.target.window.copy()
        return w

    @window.setter
    def window(self, window):
        AstroPhot_Model.window.fset(self, window)

    def __iter__(self):
        return iter(self.models.values())

    @torch.no_grad()
    def initialize(self, target=None, parameters=None, **kwargs):
        for m in self.models.values():
            m.initialize()

    def _components(self):
        return list(self.models.values())

    def sample(self, image=None, window=None, parameters=None):
        return _sample_structure(self, list(self.models.values()), image, window)

    def jacobian(self, parameters=None, as_representation=False, pass_jacobian=None, window=None, **kwargs):
        if parameters is not None:
            (self.parameters.vector_set_representation if as_representation else self.parameters.vector_set_values)(parameters)
        return _jacobian_structure(self, list(self.models.values()), as_representation, window)


# ----------------------------------------------------------------------------------------
# mapping supported structures onto one stamp of the C ABI
# ----------------------------------------------------------------------------------------


class _Structure:
    """A galaxy (Sersic or exponential) and/or a flat sky rendered on one window."""

    def __init__(self, owner, components):
        gals = [c for c in components if isinstance(c, (Sersic_Galaxy, Exponential_Galaxy))]
        skies = [c for c in components if isinstance(c, Flat_Sky)]
        if len(gals) + len(skies) != len(components) or len(gals) > 1 or len(skies) > 1:
            raise NotImplementedError(
                "the CUDA render path covers one Sersic or exponential galaxy, optionally with one flat sky")
        self.owner = owner
        self.gal = gals[0] if gals else None
        self.sky = skies[0] if skies else None
        g = self.gal
        if g is not None:
            if g.psf_mode not in ("none", "full"):
                raise SpecificationConflict(f"unknown psf_mode {g.psf_mode}")
            if g.psf_mode == "full" and g.psf_convolve_mode not in ("fft", "direct"):
                raise ValueError(f"unrecognized psf_convolve_mode: {g.psf_convolve_mode}")
            if g.psf_mode == "full" and g.psf_subpixel_shift not in ("bilinear", "none"):
                from . import _native as N

                N.lanczos_order(g.psf_subpixel_shift)  # "lanczos:k", or SpecificationConflict
                if "lanczos" not in g.psf_subpixel_shift:
                    raise SpecificationConflict(f"unrecognized subpixel shift method: {g.psf_subpixel_shift}")

    def options(self):
        from . import _native as N

        g = self.gal
        free = 0
        if g is not None:
            for name, slots in SLOT.items():
                if name in g.parameters and not g.parameters[name].locked:
                    for sl in slots:
                        free |= 1 << sl
        if self.sky is not None and not self.sky.parameters["F"].locked:
            free |= 1 << 7
        if g is None:
            return N.make_options(profile="sersic", sampling_mode="midpoint", integrate_mode="none", psf_mode="none",
                                  free_mask=free, has_sky=True)
        return N.make_options(
            profile=g.profile, sampling_mode=g.sampling_mode, integrate_mode=g.integrate_mode, psf_mode=g.psf_mode,
            psf_subpixel_shift=g.psf_subpixel_shift, integrate_max_depth=g.integrate_max_depth,
            integrate_gridding=g.integrate_gridding, integrate_quad_level=g.integrate_quad_level,
            sampling_tolerance=g.sampling_tolerance, softening=g.softening, free_mask=free,
            has_sky=self.sky is not None, psf_convolve_mode=g.psf_convolve_mode)

    def full_params(self):
        v = np.zeros(8)
        g = self.gal
        if g is None:
            v[:7] = [0.0, 0.0, 0.5, 0.0, 1.0, 1.0, -np.inf]
        else:
            p = g.parameters
            v[0:2] = p["center"].value.numpy()
            v[2] = p["q"].value.item()
            v[3] = p["PA"].value.item()
            v[4] = p["n"].value.item() if "n" in p else 1.0
            v[5] = p["Re"].value.item()
            v[6] = p["Ie"].value.item()
        if self.sky is not None:
            v[7] = self.sky.parameters["F"].value.item()
        return v

    def vector_order(self):
        """For each element of ``owner.parameters.vector_values()``, its full-vector slot."""
        out = []
        comps = [c for c in ([self.gal] if self.gal is not None else []) + ([self.sky] if self.sky is not None else [])]
        slot_of = {}
        for c in comps:
            for name, slots in SLOT.items():
                if name in c.parameters:
                    slot_of[c.parameters[name].identity] = slots
        for node in self.owner.parameters.flat(include_locked=False).values():
            slots = slot_of[node.identity]
            mask = node.vector_mask().numpy()
            out += [sl for sl, m in zip(slots, mask) if m]
        return out


def _plan(owner, struct: _Structure, window: Window):
    from . import _native as N

    opts = struct.options()
    psf = struct.gal.psf if (struct.gal is not None and struct.gal.psf_mode == "full") else None
    if psf is not None and abs(psf.pixel_length - window.pixel_length) > 1e-9 * window.pixel_length:
        raise SpecificationConflict("PSFs finer than the image pixels are not supported by the CUDA path")
    key = (tuple(window.pixel_shape), tuple(window.geometry_row()), None if psf is None else (id(psf), tuple(psf.data.shape)),
           bytes(opts))
    plans = owner.__dict__.setdefault("_plans", {})
    if key not in plans:
        batch = N.StampBatch([tuple(window.pixel_shape)], None if psf is None else [(psf.data.shape[1], psf.data.shape[0])],
                             window.geometry_row()[None, :], opts, config.ap_device)
        psf_d = None if psf is None else batch.pack_psf([psf.data.numpy()])
        plans.clear()
        plans[key] = (batch, psf_d)
    return plans[key]


def _sample_structure(owner, components, image, window):
    if _needs_scene(owner, components):
        return _sample_scene(owner, components, image, window)
    struct = _Structure(owner, components)
    w = owner.window if window is None else (owner.window & window)
    if image is None:
        image = owner.target.model_image(w)
    batch, psf_d = _plan(owner, struct, w)
    out = batch.render(torch.tensor(struct.full_params()[None, :]), psf_d)
    img = Model_Image(torch.as_tensor(batch.unpack(out)[0], dtype=config.ap_dtype), w.copy())
    image += img
    return image


def _jacobian_structure(owner, components, as_representation, window):
    if _needs_scene(owner, components):
        return _jacobian_scene(owner, components, as_representation, window)
    struct = _Structure(owner, components)
    w = owner.window if window is None else (owner.window & window)
    batch, psf_d = _plan(owner, struct, w)
    _, jac = batch.jacobian(torch.tensor(struct.full_params()[None, :]), psf_d, as_representation=as_representation)
    ny, nx = int(w.pixel_shape[1]), int(w.pixel_shape[0])
    J = jac.cpu().numpy().reshape(batch.n_free, ny, nx).astype(np.float64)
    # compact C-ABI columns (full-vector slot order) -> the model's vector order
    compact = [i for i in range(8) if batch.options.free_mask & (1 << i)]
    order = struct.vector_order()
    cols = [J[compact.index(sl)] for sl in order]
    data = np.stack(cols, -1) if cols else np.zeros((ny, nx, 0))
    return Jacobian_Image(owner.parameters.vector_identities(), data, w.copy())


class _NLLFunction(torch.autograd.Function):
    """nll(vector) with the adjoint of the CUDA render as its backward: d nll / d vector =
    sum_pixels W (model - data) d model / d vector over unmasked pixels."""

    @staticmethod
    def forward(ctx, vec, owner, as_representation):
        v = vec.detach().to("cpu", config.ap_dtype)
        (owner.parameters.vector_set_representation if as_representation else owner.parameters.vector_set_values)(v)
        ctx.owner, ctx.as_rep = owner, as_representation
        comps = owner._components()
        if _needs_scene(owner, comps):
            scene = _make_scene(owner, comps)
            rep = scene.representation()
            model = scene.forward(rep).to(torch.float64)
            r = model - scene.data.to(torch.float64)
            wt = scene.weight.to(torch.float64)
            if scene.mask is not None:
                keep = scene.mask == 0
                r = torch.where(keep, r, torch.zeros_like(r))
                wt = torch.where(keep, wt, torch.zeros_like(wt))
            g = wt * r
            ctx.scene, ctx.rep, ctx.g = scene, rep, g
            return (0.5 * torch.sum(g * r)).to("cpu", vec.dtype)
        ctx.scene = None
        struct = _Structure(owner, comps)
        w = owner.window
        batch, psf_d = _plan(owner, struct, w)
        params = torch.tensor(struct.full_params()[None, :])
        model = batch.render(params, psf_d).to(torch.float64)
        data = owner.target[w]
        d = batch.pack([data.data.numpy()], torch.float64)
        wt = batch.pack([data.weight.numpy()], torch.float64)
        r = model - d
        if data.has_mask:
            keep = torch.logical_not(batch.pack([data.mask.numpy().astype(np.uint8)], torch.uint8).bool())
            r = torch.where(keep, r, torch.zeros_like(r))
            wt = torch.where(keep, wt, torch.zeros_like(wt))
        g = wt * r
        ctx.struct = struct
        ctx.batch, ctx.psf_d, ctx.params, ctx.g = batch, psf_d, params, g
        return (0.5 * torch.sum(g * r)).to("cpu", vec.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        if ctx.scene is not None:
            grad = ctx.scene.vjp(ctx.rep, ctx.g.to(torch.float32), as_representation=ctx.as_rep,
                                 reference_center=bool(ctx.owner.reference_center_gradient))
            return grad.to(config.ap_dtype) * grad_out.to("cpu", config.ap_dtype), None, None
        batch = ctx.batch
        gc = batch.vjp(ctx.params, ctx.psf_d, ctx.g.to(torch.float32), as_representation=ctx.as_rep,
                       reference_center=bool(ctx.owner.reference_center_gradient))[0].cpu()
        compact = [i for i in range(8) if batch.options.free_mask & (1 << i)]
        grad = torch.tensor([float(gc[compact.index(sl)]) for sl in ctx.struct.vector_order()], dtype=config.ap_dtype)
        return grad * grad_out.to("cpu", config.ap_dtype), None, None


# ----------------------------------------------------------------------------------------
# groups of several galaxies on one image: scenes (astrophot_gb300.scene)
# ----------------------------------------------------------------------------------------
def _galaxies(components):
    return [c for c in components if isinstance(c, (Sersic_Galaxy, Exponential_Galaxy))]


def _psf_upscale(psf, window) -> int:
    """round(image pixel / PSF pixel) (models/model_object.py:313); 1 for no PSF or a PSF model."""
    if psf is None or isinstance(psf, PSF_Model):
        return 1
    ratio = float(window.pixel_length) / float(psf.pixel_length)
    u = int(round(ratio))
    if u < 1 or abs(ratio - u) > 1e-6 * ratio:
        raise SpecificationConflict("the PSF's pixels must divide the image's pixels on the CUDA path")
    return u


def _needs_scene(owner, components):
    """More than one galaxy, a galaxy whose own window is not the group's window, or a galaxy
    convolved with a live PSF model or a PSF image finer than the image pixels."""
    gals = _galaxies(components)
    if len(gals) > 1:
        return True
    if gals and gals[0].psf_mode == "full" and isinstance(gals[0].psf, PSF_Model):
        return True
    if gals and gals[0].psf_mode == "full" and _psf_upscale(gals[0].psf, owner.window) > 1:
        return True
    if gals and gals[0] is not owner and gals[0]._window is not None and not (gals[0].window == owner.window):
        return True
    return False


_KNOBS = ("sampling_mode", "sampling_tolerance", "integrate_mode", "integrate_max_depth", "integrate_gridding",
          "integrate_quad_level", "softening", "psf_subpixel_shift", "psf_convolve_mode", "psf_mode")


def _scene_spec(owner, components):
    from .scene import SceneSource

    w = owner.window
    gals = _galaxies(components)
    skies = [c for c in components if isinstance(c, Flat_Sky)]
    if len(gals) + len(skies) != len(components) or len(skies) > 1:
        raise NotImplementedError("the scene path covers Sersic / exponential galaxies and one flat sky")
    sky, sky_free = 0.0, {}
    if skies:
        F = skies[0].parameters["F"]
        if F.locked:
            sky = float(w.pixel_area) * 10.0 ** float(F.value.item())
        else:
            # a free F: one image-wide column of the joint vector, after the galaxies listed
            # before the sky (the group's parameter order follows its model list)
            sky_free = dict(sky_F=float(F.value.item()),
                            sky_after=sum(1 for c in components[: components.index(skies[0])] if c in gals))
    # the scene's settings are the first galaxy's; a galaxy whose own differ carries them as its
    # source's options (its own stamp batch).  The PSF mode and the PSF are shared.
    knobs = {k: getattr(gals[0], k) for k in _KNOBS}
    if any(g.psf_mode != knobs["psf_mode"] for g in gals[1:]):
        raise NotImplementedError("galaxies of one group must share their psf_mode on the CUDA path")
    psf = gals[0].psf if knobs["psf_mode"] == "full" else None
    if psf is not None and any(g.psf is not psf for g in gals[1:]):
        raise NotImplementedError("galaxies of one group must share one PSF on the CUDA path")
    if isinstance(psf, PSF_Model) and psf._live_kind is None:
        raise NotImplementedError("the CUDA path's live PSF models are Moffat and Gaussian PSFs")
    center_owner = {}
    sources = []
    for gi, g in enumerate(gals):
        p = g.parameters
        c = p["center"]
        link = None
        if isinstance(c._value, Parameter_Node):
            target = c._value
            if id(target) not in center_owner:
                raise NotImplementedError("a linked centre must point at the centre of an earlier galaxy of the group")
            link = center_owner[id(target)]
        else:
            center_owner[id(c)] = gi
        vals = [float(v) for v in c.value.numpy()] + [
            p["q"].value.item(), p["PA"].value.item(), p["n"].value.item() if "n" in p else 1.0, p["Re"].value.item(),
            p["Ie"].value.item()]
        locked = tuple(sl for name, slots in SLOT.items() if name in p and name != "F"
                       for sl in slots if p[name].locked and not (name == "center" and link is not None))
        di, dj = g.window.offset_in(w)
        win = ((di, di + int(g.window.pixel_shape[0])), (dj, dj + int(g.window.pixel_shape[1])))
        own = {k: getattr(g, k) for k in _KNOBS if k != "psf_mode" and getattr(g, k) != knobs[k]}
        sources.append(SceneSource(g.profile, vals, win, link, locked, options=own or None))
    opts = {k: knobs[k] for k in _KNOBS if k != "psf_mode"}
    return w, sources, psf, sky, sky_free, opts


def _make_scene(owner, components, with_data=True):
    from .scene import Scene

    w, sources, psf, sky, sky_free, opts = _scene_spec(owner, components)
    if abs(w.pixelscale[0, 1]) > 0 or abs(w.pixelscale[1, 0]) > 0 or abs(w.pixelscale[0, 0] - w.pixelscale[1, 1]) > 0:
        raise NotImplementedError("scenes need a square, axis-aligned pixel grid on the CUDA path")
    nx, ny = int(w.pixel_shape[0]), int(w.pixel_shape[1])
    origin = w.pixel_to_plane(-0.5, -0.5)
    if with_data:
        tgt = owner.target[w]
        data, weight = tgt.data.numpy(), tgt.weight.numpy()
        mask = tgt.mask.numpy() if tgt.has_mask else None
    else:
        data = weight = np.zeros((ny, nx))
        mask = None
    live = psf.live_psf() if isinstance(psf, PSF_Model) else None
    if live is not None and abs(live.scale - float(w.pixelscale[0, 0])) > 1e-9 * live.scale:
        raise NotImplementedError("a live PSF needs the image's pixel scale on the CUDA path")
    scene = Scene(nx, ny, sources, None if (psf is None or live is not None) else psf.data.numpy(), data, weight,
                  mask=mask, sky=sky, scale=float(w.pixelscale[0, 0]), options=opts,
                  origin=(float(origin[0]), float(origin[1])), device=config.ap_device, psf_model=live,
                  psf_upscale=_psf_upscale(psf, w), **sky_free)
    if scene.P != len(owner.parameters.vector_values()):
        raise NotImplementedError("this parameter structure has no joint-vector mapping on the CUDA path")
    return scene


def _sample_scene(owner, components, image, window):
    w = owner.window if window is None else (owner.window & window)
    if window is not None and not (w == owner.window):
        raise NotImplementedError("sampling a sub-window of a multi-galaxy group is not supported by the CUDA path")
    scene = _make_scene(owner, components, with_data=False)
    img = scene.forward(scene.representation()).cpu().numpy().reshape(scene.ny, scene.nx).astype(np.float64)
    if image is None:
        image = owner.target.model_image(w)
    image += Model_Image(torch.as_tensor(img, dtype=config.ap_dtype), w.copy())
    return image


def _jacobian_scene(owner, components, as_representation, window):
    w = owner.window
    scene = _make_scene(owner, components, with_data=False)
    J = scene.jacobian_image(scene.representation(), as_representation=as_representation)
    return Jacobian_Image(owner.parameters.vector_identities(), J, w.copy())
