"""The live-PSF oracle (``oracle/psfmodel.py``) pinned to the reference's own outputs in
``tests/golden/auxpsf_48.npz`` and ``auxpsf_gauss_48.npz``: a Moffat or Gaussian PSF model
sampled on a 15 x 15 PSF image, a Sersic
galaxy convolved with it, the Jacobian over [PSF n, PSF Rd, galaxy parameters] and the LM fit of
all of them (``set_aux_psf``, models/model_object.py:133-149).  Also the host-side parameter
order of the drop-in API for the same construction."""

import json
import os

import numpy as np
import pytest

from oracle.lm import LMOracle
from oracle.psfmodel import LivePSFProblem, render_psf
from oracle.render import Component, Window

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = ["auxpsf_48", "auxpsf_gauss_48"]
LOCKED = {"moffat": {"I0": 0.0}, "gaussian": {"flux": 0.0}}


@pytest.fixture(scope="module", params=CASES)
def case(request):
    d = np.load(os.path.join(GOLDEN, f"{request.param}.npz"))
    return d, json.loads(str(d["spec"]))


def kind_of(spec):
    return spec.get("psf_kind", "moffat")


def psf_params(spec, which):
    return dict(spec[which]["psf"], **LOCKED[kind_of(spec)])


def problem(d, spec):
    ini = spec["init"]
    cx, cy, q, PA, n, Re, Ie = ini["gal"]
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
    size, k = spec["size"], spec["psf_size"]
    return LivePSFProblem(gal, Window.from_scale(size, size), psf_params(spec, "init"), (k, k), d["data"],
                          d["weight"], psf_kind=kind_of(spec))


def test_oracle_psf_image_matches_reference(case):
    d, spec = case
    K, _ = render_psf(psf_params(spec, "init"), d["psf0"].shape, kind=kind_of(spec))
    assert np.max(np.abs(K - d["psf0"])) <= 1e-12 * np.max(d["psf0"])
    Kt, _ = render_psf(psf_params(spec, "truth"), d["truth_psf"].shape, kind=kind_of(spec))
    assert np.max(np.abs(Kt - d["truth_psf"])) <= 1e-12 * np.max(d["truth_psf"])


def test_oracle_live_psf_model_and_jacobian_match_reference(case):
    d, spec = case
    pr = problem(d, spec)
    assert np.allclose(pr.representation(), d["rep0"], rtol=0, atol=1e-12)
    m = pr.forward(d["rep0"]).reshape(d["model0"].shape)
    assert np.max(np.abs(m - d["model0"])) <= 1e-12 * np.max(d["model0"])
    J = pr.jacobian(d["rep0"]).reshape(d["jac_rep"].shape)
    for k in range(J.shape[-1]):
        ref = d["jac_rep"][..., k]
        assert np.max(np.abs(J[..., k] - ref)) <= 1e-10 * np.max(np.abs(ref)), (k, str(d["names"][k]))


def test_oracle_lm_with_live_psf_matches_reference(case):
    d, spec = case
    pr = problem(d, spec)
    lm = LMOracle(pr, initial_state=d["rep0"].copy())
    lm.fit()
    assert lm.message == str(d["message"])
    assert np.allclose(lm.loss_history, d["loss_history"], rtol=1e-10, atol=0)
    assert np.allclose(pr.values(), d["final_values"], rtol=1e-8, atol=1e-10)


def test_api_vector_order_puts_the_live_psf_first(case):
    """Host logic only: a galaxy built with a Moffat PSF model as its ``psf`` links the PSF's
    parameters ahead of its own, as the reference's vector_names show."""
    torch = pytest.importorskip("torch")
    import astrophot_gb300 as ap

    d, spec = case
    ini = spec["init"]
    k = spec["psf_size"]
    psf_t = ap.image.PSF_Image(data=np.ones((k, k)) / k**2, pixelscale=1.0)
    live = ap.models.AstroPhot_Model(name="order psf", model_type=f"{kind_of(spec)} psf model", target=psf_t,
                                     parameters=dict(ini["psf"]))
    cx, cy, q, PA, n, Re, Ie = ini["gal"]
    tgt = ap.image.Target_Image(data=d["data"], pixelscale=1.0, variance=1.0 / d["weight"])
    gal = ap.models.AstroPhot_Model(name="order gal", model_type="sersic galaxy model", target=tgt, psf_mode="full",
                                    psf=live, parameters={"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re,
                                                          "Ie": Ie})
    assert [str(x) for x in gal.parameters.vector_names()] == [str(x) for x in d["names"]]
    assert np.allclose(gal.parameters.vector_values().numpy(), d["val0"])
    assert np.allclose(gal.parameters.vector_representation().numpy(), d["rep0"], atol=1e-12)
    first = "n" if kind_of(spec) == "moffat" else "sigma"
    assert isinstance(gal.psf, ap.models.PSF_Model) and torch.is_tensor(gal["order psf"][first].value)


def test_oracle_group_with_live_psf_and_sky_matches_reference():
    """``auxpsf_group_48``: a Group_Model of the live-PSF galaxy and a locked flat sky (1 count
    per pixel): the PSF parameters still lead the group's vector; model, Jacobian and LM."""
    d = np.load(os.path.join(GOLDEN, "auxpsf_group_48.npz"))
    spec = json.loads(str(d["spec"]))
    ini = spec["init"]
    cx, cy, q, PA, n, Re, Ie = ini["gal"]
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
    size, k = spec["size"], spec["psf_size"]
    pr = LivePSFProblem(gal, Window.from_scale(size, size), psf_params(spec, "init"), (k, k), d["data"],
                        d["weight"], sky=1.0)
    assert [str(x) for x in d["names"]] == ["n", "Rd", "center:0", "center:1", "q", "PA", "n", "Re", "Ie"]
    assert np.allclose(pr.representation(), d["rep0"], rtol=0, atol=1e-12)
    m = pr.forward(d["rep0"]).reshape(d["model0"].shape)
    assert np.max(np.abs(m - d["model0"])) <= 1e-12 * np.max(d["model0"])
    J = pr.jacobian(d["rep0"]).reshape(d["jac_rep"].shape)
    assert np.max(np.abs(J - d["jac_rep"])) <= 1e-10 * np.max(np.abs(d["jac_rep"]))
    lm = LMOracle(pr, initial_state=d["rep0"].copy())
    lm.fit()
    assert lm.message == str(d["message"])
    assert np.allclose(lm.loss_history, d["loss_history"], rtol=1e-10, atol=0)
    assert np.allclose(pr.values(), d["final_values"], rtol=1e-8, atol=1e-10)


def test_live_psf_limits_and_maps_equal_the_oracle():
    """Host logic: the live PSF's limits and value <-> representation maps (scene.py) are the
    oracle's for each PSF kind (Moffat n in (0.1, 10), Rd and sigma in (0, inf))."""
    pytest.importorskip("torch")
    from astrophot_gb300 import scene
    from astrophot_gb300.transforms import drep_dvalue, to_rep, to_value
    from oracle import render as R

    vals = {"n": [0.15, 1.0, 2.5, 9.5], "Rd": [0.3, 2.0, 11.0], "I0": [-1.0, 0.0, 2.0], "sigma": [0.4, 1.6, 7.0],
            "flux": [-0.5, 0.0, 1.5]}
    for kind, limits in scene.PSF_MODEL_LIMITS.items():
        for name, (lim, cyc) in limits.items():
            assert (lim, cyc) == R._spec(name, kind), (kind, name)
            for v in vals[name]:
                r = to_rep(lim, cyc, v)
                assert np.isclose(r, R.value_to_rep(name, v, kind), rtol=1e-14, atol=1e-14)
                assert np.isclose(to_value(lim, cyc, r), v, rtol=1e-13, atol=1e-13)
                assert np.isclose(drep_dvalue(lim, cyc, r), R.drep_dvalue(name, r, kind), rtol=1e-14, atol=1e-14)
