"""Generate the golden vectors in this folder by running the reference itself.

Run with ``ASTROPHOT_REFERENCE=<path of the reference checkout>`` set:

    python tests/golden/make_golden.py          # every case
    python tests/golden/make_golden.py init     # only the initial-value cases
    python tests/golden/make_golden.py iter     # the initial-value and Iter_LM cases
    python tests/golden/make_golden.py segmap   # only the segmentation-map case
    python tests/golden/make_golden.py auxpsf   # only the live-PSF-model case
    python tests/golden/make_golden.py center   # only the centre-supersampling cases
    python tests/golden/make_golden.py psfstamps  # only the Moffat / Gaussian PSF stamps
    python tests/golden/make_golden.py freesky    # only the group with a free flat sky
    python tests/golden/make_golden.py knobs      # only the group with per-galaxy sampling settings
    python tests/golden/make_golden.py upscale    # only the PSF finer than the image pixels
    python tests/golden/make_golden.py groupupscale  # only the group with that PSF
    python tests/golden/make_golden.py lanczos    # only the Lanczos PSF shifts

The reference (AstroPhot 0.x) is imported through a ``sys.modules`` shim for
the optional packages it imports at module level but never calls on this
path (astropy, yaml, h5py, matplotlib, pyro, requests, tqdm).  Everything
runs in float64 on the CPU (``AP_config.ap_dtype``).  Each case stores the
inputs (data, PSF, parameters, knobs) together with the reference's outputs,
so the oracle and the CUDA path are checked on exactly the same arrays.
"""

from __future__ import annotations

import importlib.abc
import importlib.machinery
import json
import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from astrophot_gb300 import synthetic  # noqa: E402

REFERENCE = os.environ.get("ASTROPHOT_REFERENCE")


class _StubObj:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _StubObj()

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _StubObj()

    def __mro_entries__(self, bases):
        return (object,)


class _StubModule(types.ModuleType):
    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _StubObj()


class _StubFinder(importlib.abc.MetaPathFinder, importlib.abc.Loader):
    ROOTS = ("astropy", "yaml", "h5py", "matplotlib", "pyro", "requests", "tqdm")

    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in self.ROOTS:
            return importlib.machinery.ModuleSpec(fullname, self, is_package=True)
        return None

    def create_module(self, spec):
        m = _StubModule(spec.name)
        m.__path__ = []
        return m

    def exec_module(self, module):
        pass


def import_reference():
    if not REFERENCE:
        raise SystemExit("set ASTROPHOT_REFERENCE to the reference checkout (the folder holding astrophot/)")
    sys.meta_path.insert(0, _StubFinder())
    sys.path.insert(0, REFERENCE)
    import astrophot as ap  # noqa: E402

    return ap


# --------------------------------------------------------------------------
# case definitions (inputs only)
# --------------------------------------------------------------------------

MOFFAT_25 = ("moffat", 3.5, 3.0, 25)


def psf_array(spec, scale=1.0):
    if spec is None:
        return None
    kind = spec[0]
    if kind == "moffat":
        _, beta, fwhm, width = spec
        return synthetic.moffat_stamp(beta, synthetic.moffat_rd(fwhm, beta) * scale, width, scale)
    if kind == "gaussian":
        _, sigma, width = spec
        return synthetic.gaussian_stamp(sigma * scale, width, scale)
    raise ValueError(kind)


RENDER_CASES = {
    "sersic_psf_64": dict(
        kind="sersic",
        nx=64,
        ny=64,
        scale=1.0,
        psf=MOFFAT_25,
        params={"center": [31.7, 32.4], "q": 0.55, "PA": 0.9, "n": 2.5, "Re": 8.0, "Ie": 1.2},
        knobs={"psf_mode": "full"},
    ),
    "sersic_psf_n4": dict(
        kind="sersic",
        nx=48,
        ny=40,
        scale=1.0,
        psf=("moffat", 3.5, 2.5, 11),
        params={"center": [20.2, 23.9], "q": 0.35, "PA": 2.8, "n": 4.2, "Re": 4.0, "Ie": 0.8},
        knobs={"psf_mode": "full"},
    ),
    "sersic_psf_direct": dict(
        kind="sersic",
        nx=64,
        ny=64,
        scale=1.0,
        psf=MOFFAT_25,
        params={"center": [31.7, 32.4], "q": 0.55, "PA": 0.9, "n": 2.5, "Re": 8.0, "Ie": 1.2},
        knobs={"psf_mode": "full", "psf_convolve_mode": "direct"},
    ),
    # the Lanczos sub-pixel shifts of the PSF ("lanczos:3" and "lanczos:2")
    "sersic_psf_lanczos3": dict(
        kind="sersic",
        nx=64,
        ny=64,
        scale=1.0,
        psf=MOFFAT_25,
        params={"center": [31.7, 32.4], "q": 0.55, "PA": 0.9, "n": 2.5, "Re": 8.0, "Ie": 1.2},
        knobs={"psf_mode": "full", "psf_subpixel_shift": "lanczos:3"},
    ),
    "exp_psf_lanczos2": dict(
        kind="exponential",
        nx=48,
        ny=48,
        scale=1.0,
        psf=("gaussian", 1.5, 13),
        params={"center": [23.6, 24.2], "q": 0.6, "PA": 1.7, "Re": 7.0, "Ie": 1.5},
        knobs={"psf_mode": "full", "psf_subpixel_shift": "lanczos:2", "psf_convolve_mode": "direct"},
    ),
    "sersic_nopsf": dict(
        kind="sersic",
        nx=40,
        ny=48,
        scale=1.0,
        psf=None,
        params={"center": [17.3, 26.6], "q": 0.7, "PA": 0.3, "n": 1.3, "Re": 6.0, "Ie": 1.0},
        knobs={},
    ),
    "sersic_nopsf_quad3": dict(
        kind="sersic",
        nx=40,
        ny=48,
        scale=1.0,
        psf=None,
        params={"center": [17.3, 26.6], "q": 0.7, "PA": 0.3, "n": 1.3, "Re": 6.0, "Ie": 1.0},
        knobs={"sampling_mode": "quad:3"},
    ),
    "sersic_nopsf_simpsons": dict(
        kind="sersic",
        nx=40,
        ny=48,
        scale=1.0,
        psf=None,
        params={"center": [17.3, 26.6], "q": 0.7, "PA": 0.3, "n": 1.3, "Re": 6.0, "Ie": 1.0},
        knobs={"sampling_mode": "simpsons"},
    ),
    "sersic_nopsf_trapezoid": dict(
        kind="sersic",
        nx=40,
        ny=48,
        scale=1.0,
        psf=None,
        params={"center": [17.3, 26.6], "q": 0.7, "PA": 0.3, "n": 1.3, "Re": 6.0, "Ie": 1.0},
        knobs={"sampling_mode": "trapezoid"},
    ),
    "sersic_nopsf_noint": dict(
        kind="sersic",
        nx=40,
        ny=48,
        scale=1.0,
        psf=None,
        params={"center": [17.3, 26.6], "q": 0.7, "PA": 0.3, "n": 1.3, "Re": 6.0, "Ie": 1.0},
        knobs={"integrate_mode": "none"},
    ),
    "exp_psf": dict(
        kind="exponential",
        nx=48,
        ny=48,
        scale=1.0,
        psf=("gaussian", 1.5, 13),
        params={"center": [23.6, 24.2], "q": 0.6, "PA": 1.7, "Re": 7.0, "Ie": 1.5},
        knobs={"psf_mode": "full"},
    ),
    # the single-Sersic stamp configuration's sampling: midpoint, plus 3 x 3 Gauss-Legendre on
    # the pixels within 2 px of the centre, no adaptive integration (see center_supersample)
    "sersic_psf_center": dict(
        kind="sersic",
        nx=64,
        ny=64,
        scale=1.0,
        psf=MOFFAT_25,
        params={"center": [31.7, 32.4], "q": 0.55, "PA": 0.9, "n": 2.5, "Re": 8.0, "Ie": 1.2},
        knobs={"psf_mode": "full", "sampling_mode": "midpoint_center", "integrate_mode": "none"},
    ),
    "sersic_nopsf_center": dict(
        kind="sersic",
        nx=40,
        ny=48,
        scale=0.8,
        psf=None,
        params={"center": [14.1, 21.3], "q": 0.7, "PA": 0.3, "n": 3.3, "Re": 4.0, "Ie": 1.0},
        knobs={"sampling_mode": "midpoint_center", "integrate_mode": "none"},
    ),
    "sersic_scale08": dict(
        kind="sersic",
        nx=50,
        ny=60,
        scale=0.8,
        psf=("gaussian", 2.0, 11),
        params={"center": [19.66, 24.05], "q": 0.7, "PA": math.pi / 4, "n": 1.0, "Re": 12.0, "Ie": 0.0},
        knobs={"psf_mode": "full"},
    ),
}

LM_CASES = {
    # 64 x 64 single Sersic + locked sky 1.0, Moffat 25^2 (a smaller cousin of the 128^2 case)
    "lm_64": dict(size=64, seed=11, psf=MOFFAT_25),
    # the 128 x 128 single-Sersic stamp workload, two seeds
    "lm_c0_seed0": dict(size=128, seed=0, psf=MOFFAT_25),
    "lm_c0_seed1": dict(size=128, seed=1, psf=MOFFAT_25),
    # the same workload with its stated sampling: midpoint + 3 x 3 within 2 px of the centre
    "lm_c0center_seed2": dict(size=128, seed=2, psf=MOFFAT_25, sampling_mode="midpoint_center"),
}


def center_supersample(model, radius=2.0, quad_level=3):
    """Give a reference model the sampling "midpoint_center" by wrapping its ``_sample_init``:
    the reference's own midpoint sampling (models/_model_methods.py:84-98), with the pixels whose
    centres lie within ``radius`` pixels of the model centre replaced by the reference's own
    ``single_quad_integrate`` (utils/operations.py:123-147) at ``quad_level``.  The model keeps
    integrate_mode "none", so the integrated image is this deep image.  (A squared distance up
    to radius^2 + 1e-6 counts as inside, so pixel centres exactly on the circle stay in.)"""
    import torch
    from astrophot import AP_config
    from astrophot.utils.operations import single_quad_integrate

    plain = model._sample_init

    def _sample_init(image, parameters, center):
        reference, deep = plain(image=image, parameters=parameters, center=center)
        Coords = image.get_coordinate_meshgrid()
        X, Y = Coords - center[..., None, None]
        Pinv = torch.linalg.inv(image.header.pixelscale)
        di = Pinv[0, 0] * X + Pinv[0, 1] * Y
        dj = Pinv[1, 0] * X + Pinv[1, 1] * Y
        select = di * di + dj * dj <= radius * radius + 1e-6
        res, _ = single_quad_integrate(X=X[select], Y=Y[select], image_header=image.header,
                                       eval_brightness=model.evaluate_model, eval_parameters=parameters,
                                       dtype=AP_config.ap_dtype, device=AP_config.ap_device, quad_level=quad_level)
        deep[select] = res
        return reference, deep

    model._sample_init = _sample_init
    return model


# --------------------------------------------------------------------------
# reference drivers
# --------------------------------------------------------------------------


def ref_component(ap, case, target, name):
    model_type = {"sersic": "sersic galaxy model", "exponential": "exponential galaxy model"}[case["kind"]]
    kw = dict(case["knobs"])
    params = {k: (list(v) if isinstance(v, (list, tuple)) else v) for k, v in case["params"].items()}
    center = kw.get("sampling_mode") == "midpoint_center"
    if center:
        kw["sampling_mode"] = "midpoint"
    m = ap.models.AstroPhot_Model(name=name, model_type=model_type, target=target, parameters=params, **kw)
    return center_supersample(m) if center else m


def run_render_case(ap, key, case):

    psf = psf_array(case["psf"], case["scale"])
    target = ap.image.Target_Image(
        data=np.zeros((case["ny"], case["nx"])), pixelscale=case["scale"], psf=psf
    )
    model = ref_component(ap, case, target, f"golden {key}")
    img = model().data.detach().cpu().numpy()
    J_rep = model.jacobian(as_representation=True).data.detach().cpu().numpy()
    J_val = model.jacobian(as_representation=False).data.detach().cpu().numpy()
    rep = model.parameters.vector_representation().detach().cpu().numpy()
    val = model.parameters.vector_values().detach().cpu().numpy()
    out = dict(
        model=img,
        jac_rep=J_rep,
        jac_val=J_val,
        rep=rep,
        val=val,
        psf=np.zeros((0, 0)) if psf is None else psf,
        spec=json.dumps(case),
    )
    # sky groups: the same component plus a flat sky.  ``Group_Model`` pushes its own
    # ``psf_mode`` onto every sub-model when they are added (group_model_object.py:88,
    # :292-297), so the group is built with psf_mode="full"; the "quirk" entry keeps the
    # default group psf_mode ("none"), which silently turns the galaxy's PSF off.
    if key == "sersic_psf_64":
        for tag, lock, F, gmode in (
            ("locked", True, 0.0, "full"),
            ("free", False, 0.3, "full"),
            ("quirk", True, 0.0, None),
        ):
            sky = ap.models.AstroPhot_Model(
                name=f"golden sky {key} {tag}",
                model_type="flat sky model",
                target=target,
                parameters={"F": {"value": F, "locked": lock}},
            )
            sky.initialize()  # sets the (locked) sky centre to the window centre
            comp = ref_component(ap, case, target, f"golden {key} g {tag}")
            gkw = {} if gmode is None else {"psf_mode": gmode}
            group = ap.models.AstroPhot_Model(
                name=f"golden group {key} {tag}", model_type="group model", target=target, models=[comp, sky], **gkw
            )
            out[f"group_{tag}_model"] = group().data.detach().cpu().numpy()
            out[f"group_{tag}_jac_rep"] = group.jacobian(as_representation=True).data.detach().cpu().numpy()
    return out


def make_lm_data(ap, case):
    """Truth image from the reference (Sersic + sky 1.0), noise sigma = sqrt(model + 10)."""
    spec = synthetic.c0_stamp(case["seed"], size=case["size"])
    psf = psf_array(case["psf"])
    target = ap.image.Target_Image(data=np.zeros((spec.ny, spec.nx)), pixelscale=1.0, psf=psf)
    group = build_lm_group(ap, target, spec.truth, f"truth {case['seed']} {case['size']}",
                           case.get("sampling_mode", "midpoint"))
    truth_img = group().data.detach().cpu().numpy()
    data, weight = synthetic.add_noise(truth_img, spec.seed)
    return spec, psf, truth_img, data, weight


def build_lm_group(ap, target, vals, name, sampling_mode="midpoint"):
    cx, cy, q, PA, n, Re, Ie = [float(v) for v in vals]
    kw = {"integrate_mode": "none"} if sampling_mode == "midpoint_center" else {}
    gal = ap.models.AstroPhot_Model(
        name=f"{name} gal",
        model_type="sersic galaxy model",
        target=target,
        psf_mode="full",
        parameters={"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie},
        **kw,
    )
    if sampling_mode == "midpoint_center":
        center_supersample(gal)
    sky = ap.models.AstroPhot_Model(
        name=f"{name} sky",
        model_type="flat sky model",
        target=target,
        parameters={"F": {"value": 0.0, "locked": True}},
    )
    sky.initialize()  # sets the (locked) sky centre to the window centre
    return ap.models.AstroPhot_Model(
        name=f"{name} group", model_type="group model", target=target, models=[gal, sky], psf_mode="full"
    )


def run_lm_case(ap, key, case):
    spec, psf, truth_img, data, weight = make_lm_data(ap, case)
    target = ap.image.Target_Image(data=data, pixelscale=1.0, psf=psf, variance=1.0 / weight)
    group = build_lm_group(ap, target, spec.init, f"fit {key}", case.get("sampling_mode", "midpoint"))
    rep0 = group.parameters.vector_representation().detach().cpu().numpy().copy()
    res = ap.fit.LM(group, initial_state=rep0).fit()
    return dict(
        truth=spec.truth,
        init=spec.init,
        psf=psf,
        truth_model=truth_img,
        data=data,
        weight=weight,
        rep0=rep0,
        loss_history=np.array(res.loss_history),
        L_history=np.array(res.L_history),
        lambda_history=np.array(res.lambda_history),
        res=np.array(res.res()),
        final_values=group.parameters.vector_values().detach().cpu().numpy(),
        message=np.array(res.message),
        spec=json.dumps(case),
    )


VJP_CASES = {
    # negative_log_likelihood (models/core_model.py:220-256) and its autograd gradient with
    # respect to the representation vector, Sersic + Moffat 25^2, 96 x 96 crop
    "vjp_sersic_96": dict(size=96, seed=5, psf=MOFFAT_25, model="sersic"),
    # exponential, no PSF, a masked block of pixels (center gradients from the coordinates)
    "vjp_exp_mask_64": dict(size=64, seed=8, psf=None, model="exponential", mask=True),
}


def run_vjp_case(ap, key, case):
    import torch

    spec = synthetic.c0_stamp(case["seed"], size=case["size"])
    psf = psf_array(case["psf"]) if case["psf"] is not None else None
    psf_mode = "full" if psf is not None else "none"
    mtype = f"{case['model']} galaxy model"
    cx, cy, q, PA, n, Re, Ie = [float(v) for v in spec.truth]

    def params(cx, cy, q, PA, n, Re, Ie):
        p = {"center": [cx, cy], "q": q, "PA": PA, "Re": Re, "Ie": Ie}
        if case["model"] == "sersic":
            p["n"] = n
        return p

    kw = dict(pixelscale=1.0) if psf is None else dict(pixelscale=1.0, psf=psf)
    target = ap.image.Target_Image(data=np.zeros((spec.ny, spec.nx)), **kw)
    truth_model = ap.models.AstroPhot_Model(name=f"vjp truth {key}", model_type=mtype, target=target,
                                            psf_mode=psf_mode, parameters=params(cx, cy, q, PA, n, Re, Ie))
    truth_img = truth_model().data.detach().cpu().numpy()
    data, weight = synthetic.add_noise(truth_img, spec.seed)
    mask = np.zeros(data.shape, dtype=bool)
    if case.get("mask"):
        mask[5:17, 40:58] = True
        mask[::7, ::5] = True
    target = ap.image.Target_Image(data=data, variance=1.0 / weight, mask=mask, **kw)
    cx, cy, q, PA, n, Re, Ie = [float(v) for v in spec.init]
    model = ap.models.AstroPhot_Model(name=f"vjp {key}", model_type=mtype, target=target, psf_mode=psf_mode,
                                      parameters=params(cx, cy, q, PA, n, Re, Ie))
    rep = model.parameters.vector_representation().detach().clone().requires_grad_(True)
    nll = model.negative_log_likelihood(parameters=rep, as_representation=True)
    nll.backward()
    # the same gradient from the reference's forward-mode jacobian() (what its LM uses)
    rep0 = rep.detach().clone()
    J = model.jacobian(parameters=rep0, as_representation=True).data.detach().numpy().reshape(-1, len(rep0))
    m = model().data.detach().numpy().reshape(-1)
    keep = np.logical_not(mask.reshape(-1))
    grad_fwd = J[keep].T @ (weight.reshape(-1)[keep] * (m[keep] - data.reshape(-1)[keep]))
    return dict(data=data, weight=weight, mask=mask, psf=psf if psf is not None else np.zeros((0, 0)), init=spec.init,
                rep=rep.detach().numpy(), nll=np.array(nll.item()), grad=rep.grad.detach().numpy(), grad_fwd=grad_fwd,
                spec=json.dumps(case))


GROUP_CASES = {
    # Group_Model of four components with their own pixel windows on one 96 x 96 image
    # (models/group_model_object.py:183-283): a Sersic bulge and an exponential disk sharing
    # one centre node (parameter link, param/parameter.py value = node), two more Sersic
    # galaxies whose windows overlap the first pair's, a locked flat sky; group psf_mode
    # "full" with a 25 x 25 Moffat.  Recorded: model, representation Jacobian (linked columns
    # merged), vector names, and an LM trajectory.
    "group_linked_96": dict(size=96, seed=13, psf=MOFFAT_25, max_iter=12),
    # the same group with its flat sky free (F = 0.3 in the truth, started at 0.22): the sky's
    # F is the last entry of the joint vector, its Jacobian column image-wide
    "group_freesky_96": dict(size=96, seed=19, psf=MOFFAT_25, max_iter=12, sky_free=True, sky_F_truth=0.3,
                             sky_F_init=0.22),
    # the group with different sampling settings per galaxy (model attributes, per source in
    # GROUP_SOURCES order): the disk sampled by Simpson's rule, the east galaxy without adaptive
    # integration, the south galaxy by 3 x 3 Gauss-Legendre quadrature
    "group_knobs_96": dict(size=96, seed=23, psf=MOFFAT_25, max_iter=12,
                           knobs=[{}, {"sampling_mode": "simpsons"}, {"integrate_mode": "none"},
                                  {"sampling_mode": "quad:3"}]),
    # the group with a PSF image of pixels twice finer than the image's (the 25 x 25 Moffat of
    # FWHM 3" on 0.5" pixels): every galaxy sampled on its window rescaled to the PSF's grid
    "group_upscale_96": dict(size=96, seed=31, psf=MOFFAT_25, max_iter=12, psf_upscale=2),
}

GROUP_SOURCES = (
    # name, kind, window [[x0, x1], [y0, y1]], truth (cx, cy, q, PA, n, Re, Ie), link
    ("bulge", "sersic", [[8, 72], [10, 74]], (40.3, 42.6, 0.7, 0.8, 3.2, 5.0, 2.2), None),
    ("disk", "exponential", [[8, 72], [10, 74]], (40.3, 42.6, 0.45, 0.9, 1.0, 12.0, 1.3), "bulge"),
    ("east", "sersic", [[50, 96], [36, 90]], (72.4, 63.1, 0.6, 2.0, 1.5, 7.0, 1.8), None),
    ("south", "sersic", [[0, 44], [52, 96]], (21.2, 73.8, 0.8, 0.3, 2.5, 4.0, 2.0), None),
)


def group_source_params(kind, vals, linked):
    cx, cy, q, PA, n, Re, Ie = vals
    p = {"q": q, "PA": PA, "Re": Re, "Ie": Ie}
    if not linked:
        p["center"] = [cx, cy]
    if kind == "sersic":
        p["n"] = n
    return p


def group_init_values(vals):
    """Fixed 10-15 % perturbation of a truth vector (centre shifted by (0.8, -0.6) px)."""
    cx, cy, q, PA, n, Re, Ie = vals
    return (cx + 0.8, cy - 0.6, min(q * 1.1, 0.95), PA + 0.1, n * 0.85, Re * 1.15, Ie - 0.1)


def build_group(ap, target, values, tag, psf_mode="full", sky_F=0.0, sky_free=False, knobs=None):
    models = {}
    for i, ((name, kind, window, _, link), vals) in enumerate(zip(GROUP_SOURCES, values)):
        kw = dict(knobs[i]) if knobs else {}
        m = ap.models.AstroPhot_Model(name=f"{tag} {name}", model_type=f"{kind} galaxy model", target=target,
                                      window=window, parameters=group_source_params(kind, vals, link is not None),
                                      **kw)
        if link is not None:
            m.parameters["center"].value = models[link].parameters["center"]
        models[name] = m
    sky = ap.models.AstroPhot_Model(name=f"{tag} sky", model_type="flat sky model", target=target,
                                    parameters={"F": {"value": sky_F, "locked": not sky_free}})
    sky.initialize()  # sets the (unused) sky centre the sampler reads
    group = ap.models.AstroPhot_Model(name=f"{tag} group", model_type="group model", target=target,
                                      models=list(models.values()) + [sky], psf_mode=psf_mode)
    return group


def group_psf(ap, case):
    """The case's PSF array and the target's psf argument (a PSF_Image of finer pixels when the
    case has psf_upscale)."""
    u = case.get("psf_upscale", 1)
    if u == 1:
        psf = psf_array(case["psf"])
        return psf, psf
    _, beta, fwhm, width = case["psf"]
    psf = synthetic.moffat_stamp(beta, synthetic.moffat_rd(fwhm, beta), width, 1.0 / u)
    return psf, ap.image.PSF_Image(data=psf, pixelscale=1.0 / u)


def run_group_case(ap, key, case):
    N = case["size"]
    psf, psf_arg = group_psf(ap, case)
    target = ap.image.Target_Image(data=np.zeros((N, N)), pixelscale=1.0, psf=psf_arg)
    truth_vals = [src[3] for src in GROUP_SOURCES]
    sky_free = bool(case.get("sky_free", False))
    knobs = case.get("knobs")
    truth_group = build_group(ap, target, truth_vals, f"{key} truth", sky_F=case.get("sky_F_truth", 0.0),
                              sky_free=sky_free, knobs=knobs)
    truth_img = truth_group().data.detach().cpu().numpy()
    data, weight = synthetic.add_noise(truth_img, case["seed"])
    target = ap.image.Target_Image(data=data, pixelscale=1.0, psf=psf_arg, variance=1.0 / weight)
    init_vals = [group_init_values(v) for v in truth_vals]
    group = build_group(ap, target, init_vals, key, sky_F=case.get("sky_F_init", 0.0), sky_free=sky_free,
                        knobs=knobs)
    init_img = group().data.detach().cpu().numpy()
    jac = group.jacobian(as_representation=True).data.detach().cpu().numpy()
    names = [str(n) for n in group.parameters.vector_names()]
    rep0 = group.parameters.vector_representation().detach().cpu().numpy().copy()
    res = ap.fit.LM(group, initial_state=rep0, max_iter=case["max_iter"]).fit()
    return dict(
        psf=psf, data=data, weight=weight, truth_model=truth_img, init_model=init_img, jac_rep=jac,
        names=np.array(names), rep0=rep0, init_values=np.array(init_vals), truth_values=np.array(truth_vals),
        loss_history=np.array(res.loss_history), L_history=np.array(res.L_history),
        lambda_history=np.array(res.lambda_history), res=np.array(res.res()), message=np.array(res.message),
        spec=json.dumps(case),
    )


ITER_CASES = {
    # fit.Iter_LM over the group_linked_96 group from its perturbed start: the joint vector in
    # sequential chunks of 7 parameters, each chunk a full LM with the others fixed
    "iterlm_linked_96": dict(group="group_linked_96", chunks=7, method="sequential", max_iter=5),
}


def run_iter_case(ap, key, case):
    gcase = GROUP_CASES[case["group"]]
    N = gcase["size"]
    psf = psf_array(gcase["psf"])
    target = ap.image.Target_Image(data=np.zeros((N, N)), pixelscale=1.0, psf=psf)
    truth_vals = [src[3] for src in GROUP_SOURCES]
    truth_img = build_group(ap, target, truth_vals, f"{key} truth")().data.detach().cpu().numpy()
    data, weight = synthetic.add_noise(truth_img, gcase["seed"])
    target = ap.image.Target_Image(data=data, pixelscale=1.0, psf=psf, variance=1.0 / weight)
    group = build_group(ap, target, [group_init_values(v) for v in truth_vals], key)
    rep0 = group.parameters.vector_representation().detach().cpu().numpy().copy()
    res = ap.fit.Iter_LM(group, initial_state=rep0, chunks=case["chunks"], method=case["method"],
                         max_iter=case["max_iter"]).fit()
    return dict(rep0=rep0, loss_history=np.array(res.loss_history), lambda_history=np.array(res.lambda_history),
                res=np.array(res.res()), message=np.array(res.message), ndf=np.array(res.ndf), spec=json.dumps(case))


SEGMAP_CASES = {
    # the segmentation-map helpers (utils/initialize/segmentation_map.py) on a 240 x 200 image of
    # seven noisy Sersic galaxies whose segments (ids 1-6 and 9; 0 = background, skipped) are
    # their isophote regions above 3 sigma, one of them clipped at the image edge
    "segmap_240x200": dict(nx=240, ny=200, seed=31, noise=0.05),
}

SEGMAP_GALAXIES = (  # id, centre, q, PA, n, Re, Ie
    (1, (40.3, 52.7), 0.6, 0.4, 2.0, 6.0, 0.5),
    (2, (120.6, 95.2), 0.35, 2.1, 1.2, 10.0, 0.3),
    (3, (190.1, 40.8), 0.8, 1.0, 3.5, 5.0, 0.6),
    (4, (70.4, 160.3), 0.5, 2.8, 1.0, 8.0, 0.2),
    (5, (210.7, 150.9), 0.7, 0.2, 2.5, 7.0, 0.4),
    (6, (3.2, 110.5), 0.9, 1.6, 1.5, 6.0, 0.5),
    (9, (150.3, 175.6), 0.45, 1.3, 4.0, 4.0, 0.7),
)


def run_segmap_case(ap, key, case):
    from astrophot.utils.initialize import segmentation_map as sm

    rng = np.random.default_rng(case["seed"])
    nx, ny = case["nx"], case["ny"]
    blank = ap.image.Target_Image(data=np.zeros((ny, nx)), pixelscale=1.0)
    image = np.zeros((ny, nx))
    seg = np.zeros((ny, nx), dtype=np.int32)
    best = np.zeros((ny, nx))
    for sid, c, q, PA, n, Re, Ie in SEGMAP_GALAXIES:
        m = ap.models.AstroPhot_Model(name=f"{key} {sid}", model_type="sersic galaxy model", target=blank,
                                      parameters={"center": list(c), "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie})
        img = m().data.detach().cpu().numpy()
        image += img
        own = (img > 3 * case["noise"]) & (img > best)
        seg[own] = sid
        best = np.maximum(best, img)
    image = (image + case["noise"] * rng.normal(size=image.shape)).astype(np.float32).astype(np.float64)
    cen = sm.centroids_from_segmentation_map(seg, image)
    pas = sm.PA_from_segmentation_map(seg, image, cen)
    qs = sm.q_from_segmentation_map(seg, image, cen, pas)
    win = sm.windows_from_segmentation_map(seg)
    scaled = sm.scale_windows(win, image_shape=image.shape, expand_scale=1.5, expand_border=3)
    filt = sm.filter_windows(scaled, min_size=30, max_area=3800, min_flux=700.0, image=image)
    ids = np.array(sorted(int(i) for i in cen))
    return dict(
        seg=seg, image=image, ids=ids,
        centroids=np.array([cen[i] for i in ids]), pas=np.array([pas[i] for i in ids]),
        qs=np.array([qs[i] for i in ids]), windows=np.array([win[i] for i in ids]),
        scaled=np.array([scaled[i] for i in ids]), filtered_ids=np.array(sorted(int(i) for i in filt)),
        spec=json.dumps(case),
    )


ADJOINT_CASES = {
    # negative_log_likelihood().backward() of a Group_Model of three bulge (Sersic) + disk
    # (exponential) pairs sharing their centre node, each with its own window, on a 256 x 256
    # crop with a 65 x 65 Moffat PSF (FWHM 3, beta 3.5), locked sky: reverse-mode gradient
    # (grad) and the forward-mode jacobian() contracted with the residual (grad_fwd)
    "adjoint_bulge_disk_256": dict(size=256, seed=21, psf=("moffat", 3.5, 3.0, 65)),
}

ADJOINT_PAIRS = (
    # centre, window [[x0, x1], [y0, y1]], bulge (q, PA, n, Re, Ie), disk (q, PA, Re, Ie)
    ((80.3, 92.7), [[20, 150], [30, 160]], (0.8, 0.6, 3.5, 4.0, 2.0), (0.5, 0.7, 14.0, 1.1)),
    ((170.6, 150.2), [[100, 240], [80, 220]], (0.7, 2.2, 2.4, 6.0, 1.7), (0.35, 2.1, 18.0, 0.9)),
    ((120.4, 210.9), [[60, 190], [150, 256]], (0.9, 1.3, 4.5, 3.0, 2.3), (0.6, 1.4, 10.0, 1.3)),
)


def perturb_pair(c, b, dsk):
    cx, cy = c
    bq, bpa, bn, bre, bie = b
    dq, dpa, dre, die = dsk
    return ((cx + 0.7, cy - 0.5), (min(bq * 1.1, 0.95), bpa + 0.08, bn * 0.9, bre * 1.12, bie - 0.08),
            (min(dq * 1.1, 0.95), dpa - 0.06, dre * 0.9, die + 0.07))


def build_bulge_disk(ap, target, pairs, tag, perturb=False):
    models = []
    for k, (c, win, b, dsk) in enumerate(pairs):
        if perturb:
            c, b, dsk = perturb_pair(c, b, dsk)
        cx, cy = c
        bq, bpa, bn, bre, bie = b
        dq, dpa, dre, die = dsk
        bulge = ap.models.AstroPhot_Model(name=f"{tag} bulge {k}", model_type="sersic galaxy model", target=target,
                                          window=win, parameters={"center": [cx, cy], "q": bq, "PA": bpa, "n": bn,
                                                                  "Re": bre, "Ie": bie})
        disk = ap.models.AstroPhot_Model(name=f"{tag} disk {k}", model_type="exponential galaxy model",
                                         target=target, window=win,
                                         parameters={"q": dq, "PA": dpa, "Re": dre, "Ie": die})
        disk.parameters["center"].value = bulge.parameters["center"]
        models += [bulge, disk]
    sky = ap.models.AstroPhot_Model(name=f"{tag} sky", model_type="flat sky model", target=target,
                                    parameters={"F": {"value": 0.0, "locked": True}})
    sky.initialize()
    return ap.models.AstroPhot_Model(name=f"{tag} group", model_type="group model", target=target,
                                     models=models + [sky], psf_mode="full")


def run_adjoint_case(ap, key, case):
    N = case["size"]
    psf = psf_array(case["psf"])
    target = ap.image.Target_Image(data=np.zeros((N, N)), pixelscale=1.0, psf=psf)
    truth_img = build_bulge_disk(ap, target, ADJOINT_PAIRS, f"{key} truth")().data.detach().cpu().numpy()
    data, weight = synthetic.add_noise(truth_img, case["seed"])
    target = ap.image.Target_Image(data=data, pixelscale=1.0, psf=psf, variance=1.0 / weight)
    group = build_bulge_disk(ap, target, ADJOINT_PAIRS, key, perturb=True)
    names = [str(n) for n in group.parameters.vector_names()]
    rep = group.parameters.vector_representation().detach().clone().requires_grad_(True)
    nll = group.negative_log_likelihood(parameters=rep, as_representation=True)
    nll.backward()
    rep0 = rep.detach().clone()
    J = group.jacobian(parameters=rep0, as_representation=True).data.detach().cpu().numpy().reshape(-1, len(rep0))
    m = group().data.detach().cpu().numpy().reshape(-1)
    grad_fwd = J.T @ (weight.reshape(-1) * (m - data.reshape(-1)))
    init = [perturb_pair(c, b, dsk) for c, _, b, dsk in ADJOINT_PAIRS]
    return dict(psf=psf, data=data, weight=weight, names=np.array(names), rep=rep0.numpy(), nll=np.array(nll.item()),
                grad=rep.grad.detach().numpy(), grad_fwd=grad_fwd, model=m.reshape(N, N), spec=json.dumps(case),
                centers=np.array([i[0] for i in init]), bulges=np.array([i[1] for i in init]),
                disks=np.array([i[2] for i in init]), windows=np.array([w for _, w, _, _ in ADJOINT_PAIRS]))


# --------------------------------------------------------------------------
# the reference's initial-value heuristics (Model.initialize) on noisy stamps
# --------------------------------------------------------------------------

# truth rendered by the reference (PSF convolved) + flat sky, Gaussian noise; data rounded to
# float32 so every implementation reads the same numbers; ``mask`` names a mask pattern.
AUXPSF_CASES = {
    # a compact Sersic galaxy (Re 1.5 px, so the PSF shape is well constrained) on 48 x 48
    # convolved with a live Moffat PSF model on a 15 x 15 PSF image
    # (set_aux_psf, models/model_object.py:133-149): the PSF's n and Rd fitted with the galaxy
    "auxpsf_48": dict(size=48, psf_size=15, seed=21,
                      truth=dict(psf=dict(n=2.5, Rd=2.2), gal=[24.3, 23.6, 0.7, 1.0, 1.5, 1.5, 2.5]),
                      init=dict(psf=dict(n=2.0, Rd=2.6), gal=[24.0, 24.0, 0.75, 0.9, 1.8, 1.8, 2.4])),
    # the same galaxy with a live Gaussian PSF model (sigma fitted, flux locked)
    "auxpsf_gauss_48": dict(size=48, psf_size=15, seed=22, psf_kind="gaussian",
                            truth=dict(psf=dict(sigma=1.6), gal=[24.3, 23.6, 0.7, 1.0, 1.5, 1.5, 2.5]),
                            init=dict(psf=dict(sigma=2.0), gal=[24.0, 24.0, 0.75, 0.9, 1.8, 1.8, 2.4])),
}


def build_auxpsf(ap, target, psf_target, vals, tag, kind="moffat"):
    live = ap.models.AstroPhot_Model(name=f"psf {tag}", model_type=f"{kind} psf model", target=psf_target,
                                     parameters=dict(vals["psf"]))
    cx, cy, q, PA, n, Re, Ie = vals["gal"]
    gal = ap.models.AstroPhot_Model(name=f"gal {tag}", model_type="sersic galaxy model", target=target,
                                    psf_mode="full", psf=live,
                                    parameters={"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie})
    return live, gal


def run_auxpsf_case(ap, key, case):
    size, k = case["size"], case["psf_size"]
    psf_target = ap.image.PSF_Image(data=np.ones((k, k)) / k**2, pixelscale=1.0)
    blank = ap.image.Target_Image(data=np.zeros((size, size)), pixelscale=1.0)
    kind = case.get("psf_kind", "moffat")
    live_t, gal_t = build_auxpsf(ap, blank, psf_target, case["truth"], f"truth {key}", kind)
    truth_img = gal_t().data.detach().cpu().numpy()
    truth_psf = live_t().data.detach().cpu().numpy()
    data, weight = synthetic.add_noise(truth_img, case["seed"])
    target = ap.image.Target_Image(data=data, pixelscale=1.0, variance=1.0 / weight)
    live, gal = build_auxpsf(ap, target, psf_target, case["init"], f"fit {key}", kind)
    names = [str(v) for v in gal.parameters.vector_names()]
    psf0 = live().data.detach().cpu().numpy()
    model0 = gal().data.detach().cpu().numpy()
    J_rep = gal.jacobian(as_representation=True).data.detach().cpu().numpy()
    J_val = gal.jacobian(as_representation=False).data.detach().cpu().numpy()
    rep0 = gal.parameters.vector_representation().detach().cpu().numpy().copy()
    val0 = gal.parameters.vector_values().detach().cpu().numpy().copy()
    res = ap.fit.LM(gal, initial_state=rep0).fit()
    return dict(
        names=np.array(names), truth_model=truth_img, truth_psf=truth_psf, data=data, weight=weight,
        psf0=psf0, model0=model0, jac_rep=J_rep, jac_val=J_val, rep0=rep0, val0=val0,
        loss_history=np.array(res.loss_history), lambda_history=np.array(res.lambda_history),
        L_history=np.array(res.L_history), res=np.array(res.res()),
        final_values=gal.parameters.vector_values().detach().cpu().numpy(), message=np.array(res.message),
        spec=json.dumps(case),
    )


INIT_CASES = {
    "init_sersic_64": dict(kind="sersic", nx=64, ny=64, scale=1.0, sky=1.0, noise=0.05, seed=11,
                           params={"center": [31.7, 32.4], "q": 0.55, "PA": 0.9, "n": 2.5, "Re": 8.0, "Ie": 0.2}),
    "init_sersic_offcentre": dict(kind="sersic", nx=64, ny=64, scale=1.0, sky=1.0, noise=0.05, seed=12,
                                  params={"center": [24.3, 38.9], "q": 0.35, "PA": 2.6, "n": 1.2, "Re": 5.0, "Ie": 0.4}),
    "init_sersic_rect": dict(kind="sersic", nx=64, ny=48, scale=1.0, sky=1.0, noise=0.03, seed=13,
                             params={"center": [33.1, 23.6], "q": 0.8, "PA": 0.3, "n": 4.0, "Re": 6.0, "Ie": -0.3}),
    "init_sersic_mask": dict(kind="sersic", nx=64, ny=64, scale=1.0, sky=1.0, noise=0.05, seed=14, mask="rows",
                             params={"center": [30.6, 33.2], "q": 0.65, "PA": 1.9, "n": 1.8, "Re": 9.0, "Ie": 0.0}),
    "init_exp_64": dict(kind="exponential", nx=64, ny=64, scale=1.0, sky=1.0, noise=0.05, seed=15,
                        params={"center": [32.4, 31.1], "q": 0.5, "PA": 1.7, "Re": 7.0, "Ie": 0.3}),
    "init_sersic_scale08": dict(kind="sersic", nx=56, ny=56, scale=0.8, sky=1.0, noise=0.05, seed=16,
                                params={"center": [22.5, 21.9], "q": 0.7, "PA": 0.6, "n": 3.0, "Re": 5.0, "Ie": 0.1}),
    "init_sersic_big": dict(kind="sersic", nx=96, ny=96, scale=1.0, sky=1.0, noise=0.02, seed=17,
                            params={"center": [47.8, 48.3], "q": 0.6, "PA": 2.2, "n": 3.5, "Re": 16.0, "Ie": -0.2}),
    "init_sersic_compact": dict(kind="sersic", nx=48, ny=48, scale=1.0, sky=1.0, noise=0.1, seed=18,
                                params={"center": [23.9, 24.6], "q": 0.9, "PA": 0.1, "n": 1.0, "Re": 2.0, "Ie": 0.8}),
    # parameters with values are inputs: no centre of light, no PA, the fit starts from n
    "init_sersic_given": dict(kind="sersic", nx=64, ny=64, scale=1.0, sky=1.0, noise=0.05, seed=19,
                              params={"center": [29.4, 35.2], "q": 0.45, "PA": 2.3, "n": 3.0, "Re": 7.0, "Ie": 0.1},
                              given={"center": [29.5, 35.0], "PA": 2.25, "n": 2.8}),
}


def init_mask(kind, ny, nx, rng):
    if kind is None:
        return None
    m = np.zeros((ny, nx), dtype=bool)
    m[40:44, 10:50] = True
    m[rng.integers(0, ny, 60), rng.integers(0, nx, 60)] = True
    return m


def run_init_case(ap, key, case):
    """``model.initialize()`` of a Sérsic / exponential galaxy with no parameter values: the
    centre-of-light, angular-centre PA, isophote q and binned-profile Nelder-Mead heuristics."""
    from astrophot.models._shared_methods import _sample_image

    rng = np.random.default_rng(case["seed"])
    nx, ny, scale = case["nx"], case["ny"], case["scale"]
    psf = psf_array(("moffat", 3.5, 3.0, 13), scale)
    model_type = {"sersic": "sersic galaxy model", "exponential": "exponential galaxy model"}[case["kind"]]
    blank = ap.image.Target_Image(data=np.zeros((ny, nx)), pixelscale=scale, psf=psf)
    truth = ap.models.AstroPhot_Model(name=f"init truth {key}", model_type=model_type, target=blank,
                                      parameters=dict(case["params"]), psf_mode="full")
    img = truth().data.detach().cpu().numpy() + case["sky"] * scale**2
    data = (img + case["noise"] * rng.normal(size=img.shape)).astype(np.float32).astype(np.float64)
    mask = init_mask(case.get("mask"), ny, nx, rng)
    kw = {} if mask is None else {"mask": mask}
    target = ap.image.Target_Image(data=data, pixelscale=scale, psf=psf,
                                   variance=np.full(data.shape, case["noise"] ** 2), **kw)
    model = ap.models.AstroPhot_Model(name=f"init {key}", model_type=model_type, target=target, psf_mode="full",
                                      parameters={k: (list(v) if isinstance(v, list) else v)
                                                  for k, v in case.get("given", {}).items()})
    model.initialize()
    names = ["center", "q", "PA", "n", "Re", "Ie"] if case["kind"] == "sersic" else ["center", "q", "PA", "Re", "Ie"]
    vals = {k: model[k].value.detach().cpu().numpy() for k in names}
    R, I, S = _sample_image(target[model.window], model.transform_coordinates, model.radius_metric, model.parameters)
    out = dict(data=data, mask=np.zeros((0, 0), bool) if mask is None else mask, profile_R=R, profile_I=I,
               spec=json.dumps(case))
    for k, v in vals.items():
        out[f"value_{k}"] = v
    return out


def run_auxpsf_group_case(ap, key, case):
    """A group of the live-PSF galaxy and a locked flat sky (10^0 per pixel), psf_mode "full"."""
    size, k = case["size"], case["psf_size"]
    psf_target = ap.image.PSF_Image(data=np.ones((k, k)) / k**2, pixelscale=1.0)

    def group_of(target, vals, tag):
        live, gal = build_auxpsf(ap, target, psf_target, vals, tag)
        sky = ap.models.AstroPhot_Model(name=f"sky {tag}", model_type="flat sky model", target=target,
                                        parameters={"F": {"value": 0.0, "locked": True}})
        sky.initialize()
        grp = ap.models.AstroPhot_Model(name=f"group {tag}", model_type="group model", target=target,
                                        models=[gal, sky], psf_mode="full")
        return live, grp

    blank = ap.image.Target_Image(data=np.zeros((size, size)), pixelscale=1.0)
    _, grp_t = group_of(blank, case["truth"], f"truth {key}")
    truth_img = grp_t().data.detach().cpu().numpy()
    data, weight = synthetic.add_noise(truth_img, case["seed"])
    target = ap.image.Target_Image(data=data, pixelscale=1.0, variance=1.0 / weight)
    live, grp = group_of(target, case["init"], f"fit {key}")
    names = [str(v) for v in grp.parameters.vector_names()]
    model0 = grp().data.detach().cpu().numpy()
    J_rep = grp.jacobian(as_representation=True).data.detach().cpu().numpy()
    rep0 = grp.parameters.vector_representation().detach().cpu().numpy().copy()
    res = ap.fit.LM(grp, initial_state=rep0).fit()
    return dict(names=np.array(names), truth_model=truth_img, data=data, weight=weight, model0=model0,
                jac_rep=J_rep, rep0=rep0, loss_history=np.array(res.loss_history), res=np.array(res.res()),
                final_values=grp.parameters.vector_values().detach().cpu().numpy(), message=np.array(res.message),
                spec=json.dumps(case))


# the reference's PSF stamp builders (utils/initialize/construct_psf.py): Moffat (n, Rd, width,
# pixel scale) and Gaussian (sigma, width, pixel scale), 4 x 4 super-sampled and normalised
PSF_STAMP_CASES = {
    "moffat": [(3.5, 1.2, 9, 1.0), (3.5, 2.6, 21, 1.0), (2.5, 1.7, 25, 0.8), (4.8, 3.1, 15, 1.3)],
    "gaussian": [(1.0, 9, 1.0), (2.0, 51, 1.0), (1.4, 15, 0.8)],
}


def run_psf_stamps(ap):
    from astrophot.utils.initialize.construct_psf import gaussian_psf, moffat_psf

    out = {}
    for k, (n, rd, w, sc) in enumerate(PSF_STAMP_CASES["moffat"]):
        out[f"moffat_{k}_args"] = np.array([n, rd, w, sc])
        out[f"moffat_{k}"] = np.asarray(moffat_psf(n, rd, w, sc), dtype=np.float64)
    for k, (sig, w, sc) in enumerate(PSF_STAMP_CASES["gaussian"]):
        out[f"gaussian_{k}_args"] = np.array([sig, w, sc])
        out[f"gaussian_{k}"] = np.asarray(gaussian_psf(sig, w, sc), dtype=np.float64)
    return out


UPSCALE_CASES = {
    # one Sersic galaxy on a 40 x 40 image of 1"-pixels whose PSF image has 0.5"-pixels (a
    # 25 x 25 Moffat, FWHM 3"): the reference samples, integrates and convolves on the 2x finer
    # grid and sums 2 x 2 blocks back (models/model_object.py:308-350).  Model, representation
    # Jacobian and an LM fit from a perturbed start.
    "upscale_sersic_40": dict(kind="sersic", nx=40, ny=40, scale=1.0, upscale=2, psf=("moffat", 3.5, 3.0, 25),
                              truth={"center": [19.6, 20.3], "q": 0.65, "PA": 1.1, "n": 2.2, "Re": 5.5, "Ie": 1.6},
                              init={"center": [20.1, 19.9], "q": 0.72, "PA": 1.2, "n": 1.9, "Re": 6.3, "Ie": 1.5},
                              seed=29, max_iter=20),
}


def run_upscale_case(ap, key, case):
    import torch

    u, scale = case["upscale"], case["scale"]
    _, beta, fwhm, width = case["psf"]
    psf = synthetic.moffat_stamp(beta, synthetic.moffat_rd(fwhm, beta), width, scale / u)
    model_type = {"sersic": "sersic galaxy model", "exponential": "exponential galaxy model"}[case["kind"]]

    def target_of(data, variance=None):
        kw = {} if variance is None else {"variance": variance}
        return ap.image.Target_Image(data=data, pixelscale=scale, psf=ap.image.PSF_Image(data=psf, pixelscale=scale / u),
                                     **kw)

    shape = (case["ny"], case["nx"])
    truth = ap.models.AstroPhot_Model(name=f"{key} truth", model_type=model_type, target=target_of(np.zeros(shape)),
                                      parameters=dict(case["truth"]), psf_mode="full")
    truth_img = truth().data.detach().cpu().numpy()
    data, weight = synthetic.add_noise(truth_img, case["seed"])
    model = ap.models.AstroPhot_Model(name=f"{key} fit", model_type=model_type, target=target_of(data, 1.0 / weight),
                                      parameters=dict(case["init"]), psf_mode="full")
    init_img = model().data.detach().cpu().numpy()
    jac = model.jacobian(as_representation=True).data.detach().cpu().numpy()
    names = [str(n) for n in model.parameters.vector_names()]
    rep0 = model.parameters.vector_representation().detach().cpu().numpy().copy()
    # negative_log_likelihood and its reverse-mode autograd gradient at the initial point
    rep = model.parameters.vector_representation().detach().clone().requires_grad_(True)
    nll = model.negative_log_likelihood(parameters=rep, as_representation=True)
    nll.backward()
    nll_grad = rep.grad.detach().cpu().numpy().copy()
    model.parameters.vector_set_representation(torch.tensor(rep0))
    res = ap.fit.LM(model, initial_state=rep0, max_iter=case["max_iter"]).fit()
    return dict(psf=psf, data=data, weight=weight, truth_model=truth_img, init_model=init_img, jac_rep=jac,
                nll=np.array(float(nll.detach())), nll_grad=nll_grad,
                names=np.array(names), rep0=rep0, loss_history=np.array(res.loss_history),
                L_history=np.array(res.L_history), res=np.array(res.res()), message=np.array(res.message),
                spec=json.dumps(case))


def main():
    ap = import_reference()
    only = sys.argv[1] if len(sys.argv) > 1 else None
    if only == "upscale":
        for key, case in UPSCALE_CASES.items():
            out = run_upscale_case(ap, key, case)
            np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
            print("upscale", key, out["names"], out["jac_rep"].shape, out["loss_history"], str(out["message"]))
        return
    if only in ("freesky", "knobs", "groupupscale"):
        key = {"freesky": "group_freesky_96", "knobs": "group_knobs_96", "groupupscale": "group_upscale_96"}[only]
        out = run_group_case(ap, key, GROUP_CASES[key])
        np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
        print("group", key, out["names"], out["jac_rep"].shape, out["loss_history"], str(out["message"]))
        return
    if only == "psfstamps":
        out = run_psf_stamps(ap)
        np.savez_compressed(os.path.join(HERE, "psf_stamps.npz"), **out)
        print("psf stamps", sorted(k for k in out if not k.endswith("_args")))
        return
    if only == "lanczos":
        for key in ("sersic_psf_lanczos3", "exp_psf_lanczos2"):
            out = run_render_case(ap, key, RENDER_CASES[key])
            np.savez_compressed(os.path.join(HERE, f"render_{key}.npz"), **out)
            print("render", key, out["model"].shape, float(out["model"].sum()))
        return
    if only == "center":
        for key in ("sersic_psf_center", "sersic_nopsf_center"):
            out = run_render_case(ap, key, RENDER_CASES[key])
            np.savez_compressed(os.path.join(HERE, f"render_{key}.npz"), **out)
            print("render", key, out["model"].shape, float(out["model"].sum()))
        for key in ("lm_c0center_seed2",):
            out = run_lm_case(ap, key, LM_CASES[key])
            np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
            print("lm", key, len(out["loss_history"]), out["loss_history"], str(out["message"]))
        return
    if only == "auxpsf":
        for key, case in AUXPSF_CASES.items():
            out = run_auxpsf_case(ap, key, case)
            np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
            print("auxpsf", key, out["names"], out["loss_history"], str(out["message"]), out["final_values"])
        key = "auxpsf_group_48"
        out = run_auxpsf_group_case(ap, key, dict(AUXPSF_CASES["auxpsf_48"], seed=23))
        np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
        print("auxpsf group", key, out["names"], out["loss_history"], str(out["message"]), out["final_values"])
        return
    for key, case in (INIT_CASES if only != "segmap" else {}).items():
        out = run_init_case(ap, key, case)
        np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
        print("init", key, {k: out[k] for k in out if k.startswith("value_")})
    if only == "init":
        return
    for key, case in (ITER_CASES if only != "segmap" else {}).items():
        out = run_iter_case(ap, key, case)
        np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
        print("iter", key, out["loss_history"], str(out["message"]))
    if only == "iter":
        return
    for key, case in SEGMAP_CASES.items():
        out = run_segmap_case(ap, key, case)
        np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
        print("segmap", key, out["ids"], out["filtered_ids"])
    if only == "segmap":
        return
    for key, case in ADJOINT_CASES.items():
        out = run_adjoint_case(ap, key, case)
        np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
        print("adjoint", key, out["nll"], out["grad"])
    for key, case in GROUP_CASES.items():
        out = run_group_case(ap, key, case)
        np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
        print("group", key, out["jac_rep"].shape, out["loss_history"], str(out["message"]))
    for key, case in VJP_CASES.items():
        out = run_vjp_case(ap, key, case)
        np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
        print("vjp", key, out["nll"], out["grad"], out["grad_fwd"])
    for key, case in RENDER_CASES.items():
        out = run_render_case(ap, key, case)
        np.savez_compressed(os.path.join(HERE, f"render_{key}.npz"), **out)
        print("render", key, out["model"].shape, float(out["model"].sum()))
    for key, case in LM_CASES.items():
        out = run_lm_case(ap, key, case)
        np.savez_compressed(os.path.join(HERE, f"{key}.npz"), **out)
        print("lm", key, len(out["loss_history"]), out["loss_history"][-1], str(out["message"]))


if __name__ == "__main__":
    main()
