"""The CPU oracle against golden vectors recorded from the reference itself
(``tests/golden/make_golden.py``) and against the reference's own known-answer
tests (``tests/test_utils.py:16-38`` FFT convolution vs scipy, ``:344-435`` Sersic
closed forms, ``tests/test_model.py:49-74`` representation round trip)."""

import math
import os

import numpy as np
import pytest
import scipy.signal

import cases
from oracle.lm import GroupProblem, LMOracle
from oracle.render import (
    PSF,
    Component,
    Window,
    convolve_direct_semantics,
    convolve_fft_semantics,
    drep_dvalue,
    rep_to_value,
    sample_component,
    sample_group,
    sersic_total_flux,
    value_to_rep,
)


def component_from_spec(spec, **extra):
    p = dict(spec["params"])
    p["center"] = np.array(p["center"], dtype=float)
    knobs = dict(spec["knobs"])
    knobs.update(extra)
    return Component(spec["kind"], p, **knobs)


def window_from_spec(spec):
    return Window.from_scale(spec["nx"], spec["ny"], spec["scale"])


def psf_from_case(d):
    return PSF(d["psf"], d["spec"]["scale"]) if d["psf"].size else None


@pytest.mark.parametrize("name", cases.render_case_names())
def test_render_and_jacobian_match_reference(name):
    d = cases.load_render(name)
    spec = d["spec"]
    comp = component_from_spec(spec)
    r = sample_component(comp, window_from_spec(spec), psf_from_case(d), grad=True)
    scale = np.max(np.abs(d["model"]))
    assert np.max(np.abs(r.model - d["model"])) <= 1e-12 * scale
    J = np.stack([r.jac[s] for s in comp.free_slots()], -1)
    assert J.shape == d["jac_val"].shape
    for k in range(J.shape[-1]):
        colscale = np.max(np.abs(d["jac_val"][..., k]))
        assert np.max(np.abs(J[..., k] - d["jac_val"][..., k])) <= 1e-11 * colscale
    # representation-space Jacobian = value-space columns x d value / d rep
    names = [s[0] for s in comp.free_slots()]
    drep = np.array([drep_dvalue(nm, r_) for nm, r_ in zip(names, d["rep"])])
    Jr = J * drep
    for k in range(Jr.shape[-1]):
        colscale = np.max(np.abs(d["jac_rep"][..., k]))
        assert np.max(np.abs(Jr[..., k] - d["jac_rep"][..., k])) <= 1e-11 * colscale


@pytest.mark.parametrize("name", cases.upscale_case_names())
def test_psf_finer_than_image_matches_reference(name):
    """A PSF image of pixels ``upscale`` times finer than the image's: the oracle samples on the
    rescaled working window and sums the blocks back; model, Jacobian and the LM trajectory
    against the reference's."""
    d = cases.load_upscale(name)
    spec = d["spec"]
    p = dict(spec["init"])
    p["center"] = np.array(p["center"], dtype=float)
    comp = Component(spec["kind"], p, psf_mode="full")
    prob = GroupProblem([comp], Window.from_scale(spec["nx"], spec["ny"], spec["scale"]),
                        PSF(d["psf"], spec["scale"] / spec["upscale"]), d["data"], d["weight"])
    rep0 = prob.representation()
    assert np.allclose(rep0, d["rep0"], rtol=0, atol=1e-13)
    m = prob.forward(rep0).reshape(d["init_model"].shape)
    assert np.max(np.abs(m - d["init_model"])) <= 1e-12 * np.max(np.abs(d["init_model"]))
    J = prob.jacobian(rep0).reshape(d["jac_rep"].shape)
    for k in range(J.shape[-1]):
        ref = d["jac_rep"][..., k]
        assert np.max(np.abs(J[..., k] - ref)) <= 1e-11 * np.max(np.abs(ref)), k
    lm = LMOracle(prob, rep0, max_iter=spec["max_iter"]).fit()
    assert lm.message == d["message"]
    assert np.allclose(lm.loss_history, d["loss_history"], rtol=1e-10, atol=0)
    assert np.allclose(lm.res(), d["res"], rtol=1e-8, atol=1e-10)


@pytest.mark.parametrize("tag", ["locked", "free", "quirk"])
def test_group_with_sky_matches_reference(tag):
    d = cases.load_render("sersic_psf_64")
    spec = d["spec"]
    gal = component_from_spec(spec, psf_mode="none" if tag == "quirk" else "full")
    F = 0.3 if tag == "free" else 0.0
    sky = Component("flat_sky", {"F": F}, locked=() if tag == "free" else ("F",))
    model, J = sample_group([gal, sky], window_from_spec(spec), psf_from_case(d), grad=True)
    ref = d[f"group_{tag}_model"]
    assert np.max(np.abs(model - ref)) <= 1e-12 * np.max(np.abs(ref))
    slots = [s for c in (gal, sky) for s in c.free_slots()]
    names = [s[0] for s in slots]
    rep = np.concatenate([d["rep"], [F]] if tag == "free" else [d["rep"]])
    Jr = J * np.array([drep_dvalue(nm, r_) for nm, r_ in zip(names, rep)])
    refJ = d[f"group_{tag}_jac_rep"]
    assert Jr.shape == refJ.shape
    for k in range(Jr.shape[-1]):
        assert np.max(np.abs(Jr[..., k] - refJ[..., k])) <= 1e-11 * np.max(np.abs(refJ[..., k]))


def lm_problem(d):
    size = d["spec"]["size"]
    cx, cy, q, PA, n, Re, Ie = d["init"]
    knobs = {}
    if d["spec"].get("sampling_mode") == "midpoint_center":
        knobs = dict(sampling_mode="midpoint_center", integrate_mode="none")
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full",
                    **knobs)
    sky = Component("flat_sky", {"F": 0.0}, locked=("F",))
    return GroupProblem([gal, sky], Window.from_scale(size, size), PSF(d["psf"]), d["data"], d["weight"])


@pytest.mark.parametrize("name", [n for n in cases.lm_case_names() if n in ("lm_64", "lm_c0center_seed2")])
def test_lm_trajectory_matches_reference(name):
    d = cases.load_lm(name)
    prob = lm_problem(d)
    rep0 = prob.representation()
    assert np.allclose(rep0, d["rep0"], rtol=0, atol=1e-13)
    lm = LMOracle(prob, rep0).fit()
    assert lm.message == d["message"]
    assert len(lm.loss_history) == len(d["loss_history"])
    assert np.allclose(lm.loss_history, d["loss_history"], rtol=1e-12, atol=0)
    assert np.allclose(lm.L_history, d["L_history"], rtol=1e-12, atol=0)
    assert np.allclose(lm.res(), d["res"], rtol=1e-10, atol=1e-12)


def test_truth_model_matches_reference():
    d = cases.load_lm("lm_c0_seed0")
    size = d["spec"]["size"]
    cx, cy, q, PA, n, Re, Ie = d["truth"]
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
    sky = Component("flat_sky", {"F": 0.0}, locked=("F",))
    model, _ = sample_group([gal, sky], Window.from_scale(size, size), PSF(d["psf"]))
    assert np.max(np.abs(model - d["truth_model"])) <= 1e-12 * np.max(d["truth_model"])


# ---- the reference's own known-answer tests, restated ------------------------------


def test_fft_convolution_equals_scipy_same():
    """tests/test_utils.py:16-38: fft_convolve_torch == scipy.signal.fftconvolve(mode="same")
    on a zero-bordered image; both of the oracle's convolution forms must agree with it."""
    rng = np.random.default_rng(3)
    img = np.zeros((60, 70))
    img[15:-15, 15:-15] = rng.uniform(size=(30, 40))
    kern = rng.uniform(size=(11, 13))
    want = scipy.signal.fftconvolve(img, kern, mode="same")
    assert np.allclose(convolve_fft_semantics(img, kern), want, atol=1e-12)
    assert np.allclose(convolve_direct_semantics(img, kern), want, atol=1e-12)


def test_sersic_flux_closed_form():
    """tests/test_utils.py:344-435 pins sersic_Ie_to_flux against numerical integration."""
    from scipy.integrate import quad
    from oracle.render import sersic_b

    for n, Re, q in ((1.0, 5.0, 0.6), (4.0, 3.0, 0.9), (0.7, 12.0, 0.3)):
        b = sersic_b(n)
        num = quad(lambda r: 2 * math.pi * q * r * math.exp(-b * ((r / Re) ** (1 / n) - 1)), 0, np.inf, limit=500)[0]
        assert sersic_total_flux(1.0, n, Re, q) == pytest.approx(num, rel=1e-6)


@pytest.mark.parametrize("name,vals", [("q", [0.01, 0.5, 0.99]), ("n", [0.4, 2.0, 7.9]), ("Re", [0.1, 5.0, 400.0]),
                                       ("PA", [0.2, 1.0, 3.1]), ("center", [-3.0, 64.5]), ("Ie", [-1.0, 2.0])])
def test_representation_round_trip(name, vals):
    """tests/test_model.py:49-74: value -> representation -> value is the identity."""
    v = np.array(vals)
    assert np.allclose(rep_to_value(name, value_to_rep(name, v)), v, rtol=1e-12, atol=1e-12)
    # derivative of rep -> value against a central difference
    r = value_to_rep(name, v)
    h = 1e-6 * np.maximum(1.0, np.abs(r))
    fd = (rep_to_value(name, r + h) - rep_to_value(name, r - h)) / (2 * h)
    assert np.allclose(drep_dvalue(name, r), fd, rtol=1e-6, atol=1e-9)


# ---- adjoint: the gradient of the reference's negative log-likelihood -------------------


def vjp_problem(d):
    spec = d["spec"]
    size = spec["size"]
    cx, cy, q, PA, n, Re, Ie = d["init"]
    params = {"center": [cx, cy], "q": q, "PA": PA, "Re": Re, "Ie": Ie}
    if spec["model"] == "sersic":
        params["n"] = n
    psf = PSF(d["psf"]) if d["psf"].size else None
    gal = Component(spec["model"], params, psf_mode="full" if psf is not None else "none")
    mask = d["mask"] if d["mask"].any() else None
    return GroupProblem([gal], Window.from_scale(size, size), psf, d["data"], d["weight"], mask)


def oracle_nll(prob, rep):
    """``negative_log_likelihood`` (models/core_model.py:220-256): sum(W (model - data)^2) / 2
    over the unmasked pixels."""
    m = prob.forward(rep)
    keep = np.ones(m.shape, bool) if prob.mask is None else ~prob.mask.reshape(-1)
    return 0.5 * float(np.sum((prob.W.reshape(-1) * (m - prob.Y.reshape(-1)) ** 2)[keep]))


def oracle_nll_grad(prob, rep):
    """J_rep^T W (model - data) over the unmasked pixels."""
    J = prob.jacobian(rep)
    m = prob.forward(rep)
    keep = np.ones(m.shape, bool) if prob.mask is None else ~prob.mask.reshape(-1)
    return J[keep].T @ (prob.W.reshape(-1)[keep] * (m - prob.Y.reshape(-1))[keep])


@pytest.mark.parametrize("name", cases.vjp_case_names())
def test_nll_gradient_matches_reference(name):
    """The oracle's adjoint J_rep^T W (model - data) equals the reference's forward-mode
    jacobian() contracted with the residual (``grad_fwd``) and the FP64 central difference of
    the oracle's nll; it equals the reference's reverse-mode autograd gradient (``grad``) except
    for the center under PSF shift, where reverse mode adds the sampling-coordinate path."""
    d = cases.load_vjp(name)
    prob = vjp_problem(d)
    rep = prob.representation()
    assert np.allclose(rep, d["rep"], rtol=0, atol=1e-13)
    assert oracle_nll(prob, rep) == pytest.approx(float(d["nll"]), rel=1e-12)
    g = oracle_nll_grad(prob, rep)
    scale = np.max(np.abs(d["grad_fwd"]))
    assert np.max(np.abs(g - d["grad_fwd"])) <= 1e-9 * scale, (g, d["grad_fwd"])
    shifted = d["psf"].size > 0
    rest = slice(2, None) if shifted else slice(None)
    assert np.max(np.abs(g[rest] - d["grad"][rest])) <= 1e-9 * scale
    fd = np.zeros_like(rep)
    for k in range(len(rep)):
        h = 1e-6 * max(1.0, abs(rep[k]))
        rp, rm = rep.copy(), rep.copy()
        rp[k] += h
        rm[k] -= h
        fd[k] = (oracle_nll(prob, rp) - oracle_nll(prob, rm)) / (2 * h)
    assert np.max(np.abs(fd - d["grad_fwd"])) <= 1e-5 * scale, (fd, d["grad_fwd"])


def test_reverse_mode_center_gradient_is_shift_plus_coordinate_path():
    """Under PSF shift the reference's reverse-mode center gradient equals the derivative through
    the sub-pixel PSF shift plus the sampling-coordinate path -d profile / d(x, y) (convolved with
    the shifted PSF): the pixel_shift of the working window (models/model_object.py:319-323)
    that cancels the coordinate path in the forward function is not seen by backward."""
    import oracle.render as R

    d = cases.load_vjp("vjp_sersic_96")
    prob = vjp_problem(d)
    prob.set_representation(prob.representation())
    comp = prob.components[0]
    captured = {}
    orig = R._component_partials

    def with_coords(comp_, deep, finish, from_coords, win):
        jc = orig(comp_, deep, finish, True, win)
        captured["coords"] = (jc[("center", 0)], jc[("center", 1)])
        return orig(comp_, deep, finish, from_coords, win)

    R._component_partials = with_coords
    try:
        r = R.sample_component(comp, prob.window, prob.psf, grad=True)
    finally:
        R._component_partials = orig
    res = prob.W * (r.model - prob.Y)
    gc = [np.sum(res * (r.jac[("center", k)] + captured["coords"][k])) for k in range(2)]
    assert np.allclose(gc, d["grad"][:2], rtol=1e-11, atol=0)


# ---- Group_Model with per-component windows and a linked centre ------------------------------


def group_problem(d, values=None, truth=False):
    """The group of ``tests/golden/make_golden.py`` GROUP_SOURCES on the oracle (its flat sky
    locked at F = 0, or free from the case's initial / truth F)."""
    sources = (
        ("sersic", ((8, 72), (10, 74)), None),
        ("exponential", ((8, 72), (10, 74)), 0),
        ("sersic", ((50, 96), (36, 90)), None),
        ("sersic", ((0, 44), (52, 96)), None),
    )
    values = d["init_values"] if values is None else values
    knobs = d["spec"].get("knobs") or [{}] * len(sources)
    comps, links = [], {}
    for ci, ((kind, win, link), v) in enumerate(zip(sources, values)):
        cx, cy, q, PA, n, Re, Ie = v
        p = {"center": [cx, cy], "q": q, "PA": PA, "Re": Re, "Ie": Ie}
        if kind == "sersic":
            p["n"] = n
        comps.append(Component(kind, p, psf_mode="full", window=win, **knobs[ci]))
        if link is not None:
            links[(ci, "center")] = (link, "center")
    spec = d["spec"]
    if spec.get("sky_free"):
        comps.append(Component("flat_sky", {"F": spec["sky_F_truth" if truth else "sky_F_init"]}))
    else:
        comps.append(Component("flat_sky", {"F": 0.0}, locked=("F",)))
    N = spec["size"]
    psf = PSF(d["psf"], scale=1.0 / spec.get("psf_upscale", 1))  # a finer PSF grid: psf_upscale
    return GroupProblem(comps, Window.from_scale(N, N), psf, d["data"], d["weight"], links=links)


@pytest.mark.parametrize("name", cases.group_case_names())
def test_group_windows_links_match_reference(name):
    d = cases.load_group(name)
    prob = group_problem(d)
    rep0 = prob.representation()
    assert len(rep0) == len(d["names"]) == 25 + bool(d["spec"].get("sky_free"))
    assert np.allclose(rep0, d["rep0"], rtol=0, atol=1e-13)
    m = prob.forward(rep0).reshape(d["init_model"].shape)
    assert np.max(np.abs(m - d["init_model"])) <= 1e-12 * np.max(np.abs(d["init_model"]))
    truth = group_problem(d, d["truth_values"], truth=True)
    mt = truth.forward(truth.representation()).reshape(d["truth_model"].shape)
    assert np.max(np.abs(mt - d["truth_model"])) <= 1e-12 * np.max(np.abs(d["truth_model"]))
    J = prob.jacobian(rep0).reshape(d["jac_rep"].shape)
    for k in range(J.shape[-1]):
        ref = d["jac_rep"][..., k]
        assert np.max(np.abs(J[..., k] - ref)) <= 1e-11 * np.max(np.abs(ref)), k


@pytest.mark.parametrize("name", cases.group_case_names())
def test_group_lm_trajectory_matches_reference(name):
    d = cases.load_group(name)
    prob = group_problem(d)
    lm = LMOracle(prob, prob.representation(), max_iter=d["spec"]["max_iter"]).fit()
    assert lm.message == d["message"]
    assert np.allclose(lm.loss_history, d["loss_history"], rtol=1e-10, atol=0)
    assert np.allclose(lm.res(), d["res"], rtol=1e-8, atol=1e-10)


# ---- adjoint of a bulge + disk group (shared centres, windows, 65 x 65 PSF) -----------------


def adjoint_problem(d):
    comps, links = [], {}
    for k, (c, w, b, dk) in enumerate(zip(d["centers"], d["windows"], d["bulges"], d["disks"])):
        win = tuple(tuple(int(v) for v in r) for r in w)
        q, PA, n, Re, Ie = b
        comps.append(Component("sersic", {"center": list(c), "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie},
                               psf_mode="full", window=win))
        q, PA, Re, Ie = dk
        comps.append(Component("exponential", {"center": list(c), "q": q, "PA": PA, "Re": Re, "Ie": Ie},
                               psf_mode="full", window=win))
        links[(2 * k + 1, "center")] = (2 * k, "center")
    comps.append(Component("flat_sky", {"F": 0.0}, locked=("F",)))
    N = d["spec"]["size"]
    return GroupProblem(comps, Window.from_scale(N, N), PSF(d["psf"]), d["data"], d["weight"], links=links)


@pytest.mark.parametrize("name", cases.adjoint_case_names())
def test_group_adjoint_golden_pins_the_oracle(name):
    """nll of the group, the own-window Jacobian contracted with the residual (grad_fwd) and the
    FP64 central differences (step 1e-6 relative) of the group-window forward, which the
    reference's reverse-mode gradient equals away from the centres."""
    d = cases.load_adjoint(name)
    prob = adjoint_problem(d)
    rep = prob.representation()
    assert np.allclose(rep, d["rep"], rtol=0, atol=1e-12)
    m = prob.forward(rep)
    assert np.max(np.abs(m - d["model"].reshape(-1))) <= 1e-12 * np.max(d["model"])
    W, Y = prob.W.reshape(-1), prob.Y.reshape(-1)
    nll = 0.5 * float(np.sum(W * (m - Y) ** 2))
    assert nll == pytest.approx(float(d["nll"]), rel=1e-12)
    J = prob.jacobian(rep)
    g = J.T @ (W * (prob.forward(rep) - Y))
    scale = np.max(np.abs(d["grad_fwd"]))
    assert np.max(np.abs(g - d["grad_fwd"])) <= 1e-9 * scale
    # finite differences on two entries (a bulge axis ratio, a centre)
    names = list(d["names"])
    for k in (2, 0):
        h = 1e-6 * max(1.0, abs(rep[k]))
        rp, rm = rep.copy(), rep.copy()
        rp[k] += h
        rm[k] -= h
        fp = 0.5 * float(np.sum(W * (prob.forward(rp) - Y) ** 2))
        fm = 0.5 * float(np.sum(W * (prob.forward(rm) - Y) ** 2))
        fd = (fp - fm) / (2 * h)
        if names[k].startswith("center"):
            # the reverse-mode centre adds the sampling-coordinate path: not the derivative
            assert abs(fd - d["grad"][k]) > 1e-3 * abs(fd)
        else:
            assert abs(fd - d["grad"][k]) <= 1e-5 * scale, (k, names[k], fd, d["grad"][k])


# ---- Iter_LM: LM on chunks of the joint vector ----------------------------------------------


@pytest.mark.parametrize("name", cases.iter_case_names())
def test_iter_lm_first_sweep_matches_reference(name):
    """The first sweep of ``Iter_LM`` (four chunk LMs over the 25-entry vector of the linked
    group) against the reference's: the sweep loss and the state after it.  (The full five-sweep
    run, 2 minutes on the oracle, agrees to 1e-10 in loss and 3e-10 in state; the GPU test runs
    it through the library.)"""
    from oracle.lm import IterLMOracle

    d = cases.load_iter(name)
    g = cases.load_group(d["spec"]["group"])
    prob = group_problem(g)
    it = IterLMOracle(prob, d["rep0"], chunks=d["spec"]["chunks"], method=d["spec"]["method"], max_iter=1).fit()
    assert it.ndf == int(d["ndf"])
    assert np.isclose(it.loss_history[0], d["loss_history"][0], rtol=1e-10, atol=0)
    assert np.allclose(it.lambda_history[0], d["lambda_history"][0], rtol=1e-8, atol=1e-10)


def test_psf_stamps_match_reference_builders():
    """The Moffat and Gaussian PSF stamps this library builds for its fixtures and synthetic
    workloads equal the reference's own builders (utils/initialize/construct_psf.py:8-65, recorded
    by tests/golden/make_golden.py psfstamps): same 4 x 4 super-sampling grid and normalisation."""
    from astrophot_gb300 import synthetic

    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "psf_stamps.npz"))
    k = 0
    while f"moffat_{k}" in d:
        n, rd, w, sc = d[f"moffat_{k}_args"]
        got = synthetic.moffat_stamp(float(n), float(rd), int(w), float(sc))
        np.testing.assert_allclose(got, d[f"moffat_{k}"], rtol=1e-12, atol=1e-15)
        k += 1
    assert k == 4
    k = 0
    while f"gaussian_{k}" in d:
        sig, w, sc = d[f"gaussian_{k}_args"]
        got = synthetic.gaussian_stamp(float(sig), int(w), float(sc))
        np.testing.assert_allclose(got, d[f"gaussian_{k}"], rtol=1e-12, atol=1e-15)
        k += 1
    assert k == 3
