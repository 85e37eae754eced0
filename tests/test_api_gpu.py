"""The drop-in API on the GPU, written like the reference's own tests: models built with
``AstroPhot_Model(model_type=...)`` on a ``Target_Image``, sampled, differentiated and fitted
with ``fit.LM``; compared with the golden vectors recorded from the reference."""

import math

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import cases  # noqa: E402


@pytest.fixture(scope="module")
def ap():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import astrophot_gb300

    return astrophot_gb300


def close(got, ref, rel=1e-5):
    return np.max(np.abs(np.asarray(got) - ref)) <= rel * np.max(np.abs(ref))


def model_from_case(ap, name, tag):
    d = cases.load_render(name)
    spec = d["spec"]
    psf = d["psf"] if d["psf"].size else None
    tar = ap.image.Target_Image(data=np.zeros((spec["ny"], spec["nx"])), pixelscale=spec["scale"], psf=psf)
    kind = {"sersic": "sersic galaxy model", "exponential": "exponential galaxy model"}[spec["kind"]]
    m = ap.models.AstroPhot_Model(name=f"api {name} {tag}", model_type=kind, target=tar, parameters=dict(spec["params"]),
                                  **spec["knobs"])
    return d, tar, m


@pytest.mark.parametrize("name", cases.render_case_names())
def test_model_call_and_jacobian_match_reference(ap, name):
    d, tar, m = model_from_case(ap, name, "a")
    img = m()
    assert close(img.data.numpy(), d["model"])
    J = m.jacobian(as_representation=True)
    assert J.data.shape == d["jac_rep"].shape
    for k in range(J.data.shape[-1]):
        assert close(J.data[..., k].numpy(), d["jac_rep"][..., k], rel=2e-4)


def test_group_with_sky_and_psf_mode_quirk(ap):
    for tag, gmode, lock, F in (("locked", "full", True, 0.0), ("free", "full", False, 0.3), ("quirk", None, True, 0.0)):
        d, tar, gal = model_from_case(ap, "sersic_psf_64", f"g {tag}")
        sky = ap.models.AstroPhot_Model(name=f"api sky {tag}", model_type="flat sky model", target=tar,
                                        parameters={"F": {"value": F, "locked": lock}})
        sky.initialize()
        kw = {} if gmode is None else {"psf_mode": gmode}
        grp = ap.models.AstroPhot_Model(name=f"api grp {tag}", model_type="group model", target=tar, models=[gal, sky], **kw)
        assert close(grp().data.numpy(), d[f"group_{tag}_model"])
        J = grp.jacobian(as_representation=True).data.numpy()
        ref = d[f"group_{tag}_jac_rep"]
        assert J.shape == ref.shape
        for k in range(ref.shape[-1]):
            assert close(J[..., k], ref[..., k], rel=2e-4)


def test_sky_first_group_keeps_vector_order(ap):
    d, tar, gal = model_from_case(ap, "sersic_psf_64", "order")
    sky = ap.models.AstroPhot_Model(name="api sky order", model_type="flat sky model", target=tar, parameters={"F": 0.3})
    sky.initialize()
    grp = ap.models.AstroPhot_Model(name="api grp order", model_type="group model", target=tar, models=[sky, gal],
                                    psf_mode="full")
    assert grp.parameters.vector_names()[0] == "F"
    J = grp.jacobian(as_representation=True).data.numpy()
    ref = d["group_free_jac_rep"]  # reference order: galaxy then sky
    assert close(J[..., 0], ref[..., -1], rel=2e-4)
    for k in range(7):
        assert close(J[..., 1 + k], ref[..., k], rel=2e-4)


def lm_target(ap, d, tag):
    tar = ap.image.Target_Image(data=d["data"], pixelscale=1.0, psf=d["psf"], variance=1.0 / d["weight"])
    cx, cy, q, PA, n, Re, Ie = d["init"]
    kw = {}
    if d["spec"].get("sampling_mode") == "midpoint_center":
        kw = dict(sampling_mode="midpoint_center", integrate_mode="none")
    gal = ap.models.AstroPhot_Model(name=f"lm gal {tag}", model_type="sersic galaxy model", target=tar, psf_mode="full",
                                    parameters={"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, **kw)
    sky = ap.models.AstroPhot_Model(name=f"lm sky {tag}", model_type="flat sky model", target=tar,
                                    parameters={"F": {"value": 0.0, "locked": True}})
    sky.initialize()
    return ap.models.AstroPhot_Model(name=f"lm grp {tag}", model_type="group model", target=tar, models=[gal, sky],
                                     psf_mode="full"), gal


@pytest.mark.parametrize("name", cases.lm_case_names())
def test_fit_lm_matches_reference(ap, name):
    d = cases.load_lm(name)
    grp, gal = lm_target(ap, d, name)
    rep0 = grp.parameters.vector_representation().numpy()
    assert np.allclose(rep0, d["rep0"], atol=1e-13)
    res = ap.fit.LM(grp, initial_state=rep0).fit()
    assert abs(min(res.loss_history) / d["loss_history"].min() - 1) <= 1e-4
    assert np.allclose(res.loss_history[:3], d["loss_history"][:3], rtol=1e-6)
    assert res.message in ("success", "success by immobility. Convergence not guaranteed",
                           "fail. Could not find step to improve Chi^2")
    # the model now holds res(); its vector agrees with the reference's fitted vector
    got = grp.parameters.vector_representation().numpy()
    assert np.allclose(got, res.res(), rtol=1e-12, atol=1e-12)
    cov = res.covariance_matrix
    sig = np.sqrt(np.diag(cov.numpy()))
    vals = grp.parameters.vector_values().numpy()
    ref_vals = d["final_values"]
    assert np.all(np.abs(vals - ref_vals) <= 0.25 * sig)
    res.update_uncertainty()
    assert np.allclose(grp.parameters.vector_uncertainty().numpy(), sig)


def test_fit_recovers_truth_like_the_reference_test(ap):
    """tests/test_fit.py:71-161 style: noisy Sersic, LM from a nearby start recovers it."""
    d = cases.load_lm("lm_c0_seed0")
    grp, gal = lm_target(ap, d, "truth")
    ap.fit.LM(grp).fit()
    truth = d["truth"]
    assert gal["center"].value[0].item() / truth[0] == pytest.approx(1, abs=1e-2)
    assert gal["center"].value[1].item() / truth[1] == pytest.approx(1, abs=1e-2)
    assert gal["n"].value.item() == pytest.approx(truth[4], abs=0.3)
    assert gal["q"].value.item() == pytest.approx(truth[2], abs=0.05)
    assert gal["Ie"].value.item() == pytest.approx(truth[6], abs=0.1)


def test_batch_lm_equals_single_lm(ap):
    names = cases.lm_case_names()
    singles, batch_models = [], []
    for name in names:
        d = cases.load_lm(name)
        g1, _ = lm_target(ap, d, f"s {name}")
        singles.append(ap.fit.LM(g1, initial_state=d["rep0"]).fit())
        g2, _ = lm_target(ap, d, f"b {name}")
        batch_models.append(g2)
    b = ap.fit.BatchLM(batch_models, initial_states=[cases.load_lm(n)["rep0"] for n in names]).fit()
    for s, f in zip(singles, b.fits):
        assert s.loss_history == f.loss_history
        assert np.array_equal(np.asarray(s.res()), f.res_state.numpy())


def test_bad_modes_raise(ap):
    from astrophot_gb300.errors import SpecificationConflict

    d, tar, m = model_from_case(ap, "sersic_nopsf", "bad")
    m.sampling_mode = "bogus"
    with pytest.raises(SpecificationConflict):
        m()
    m.sampling_mode = "midpoint"
    m.integrate_mode = "full"
    with pytest.raises(SpecificationConflict):
        m()


def test_model_window_inside_target(ap):
    """A model on a sub-window of its target renders like the oracle on that window."""
    from oracle.render import PSF, Component, Window, sample_component

    d = cases.load_render("sersic_psf_64")
    spec = d["spec"]
    tar = ap.image.Target_Image(data=np.zeros((64, 64)), pixelscale=1.0, psf=d["psf"])
    p = spec["params"]
    m = ap.models.AstroPhot_Model(name="api win", model_type="sersic galaxy model", target=tar, psf_mode="full",
                                  window=[[10, 50], [5, 58]], parameters=dict(p))
    img = m().data.numpy()
    assert img.shape == (53, 40)
    comp = Component("sersic", {"center": np.array(p["center"]), "q": p["q"], "PA": p["PA"], "n": p["n"], "Re": p["Re"],
                                "Ie": p["Ie"]}, psf_mode="full")
    ref = sample_component(comp, Window(40, 53, np.eye(2), np.array([-10.5, -5.5]), np.zeros(2)), PSF(d["psf"])).model
    assert close(img, ref)


# the GROUP_SOURCES of tests/golden/make_golden.py, built as the reference's user code does
GROUP_SOURCES = (
    ("bulge", "sersic", [[8, 72], [10, 74]], None),
    ("disk", "exponential", [[8, 72], [10, 74]], "bulge"),
    ("east", "sersic", [[50, 96], [36, 90]], None),
    ("south", "sersic", [[0, 44], [52, 96]], None),
)


def build_group(ap, target, values, tag, spec=None):
    spec = spec or {}
    knobs = spec.get("knobs") or [{}] * len(GROUP_SOURCES)
    models = {}
    for (name, kind, window, link), v, kw in zip(GROUP_SOURCES, values, knobs):
        cx, cy, q, PA, n, Re, Ie = [float(x) for x in v]
        p = {"q": q, "PA": PA, "Re": Re, "Ie": Ie}
        if link is None:
            p["center"] = [cx, cy]
        if kind == "sersic":
            p["n"] = n
        m = ap.models.AstroPhot_Model(name=f"{tag} {name}", model_type=f"{kind} galaxy model", target=target,
                                      window=window, parameters=p, **kw)
        if link is not None:
            m.parameters["center"].value = models[link].parameters["center"]
        models[name] = m
    free = bool(spec.get("sky_free", False))
    sky = ap.models.AstroPhot_Model(name=f"{tag} sky", model_type="flat sky model", target=target,
                                    parameters={"F": {"value": spec.get("sky_F_init", 0.0), "locked": not free}})
    sky.initialize()
    return ap.models.AstroPhot_Model(name=f"{tag} group", model_type="group model", target=target,
                                     models=list(models.values()) + [sky], psf_mode="full")


@pytest.mark.parametrize("name", cases.group_case_names())
def test_multi_galaxy_group_matches_reference(ap, name):
    """Windows per galaxy, a linked centre, PSF: model, representation Jacobian and LM."""
    d = cases.load_group(name)
    u = d["spec"].get("psf_upscale", 1)
    psf = d["psf"] if u == 1 else ap.image.PSF_Image(data=d["psf"], pixelscale=1.0 / u)
    target = ap.image.Target_Image(data=d["data"], pixelscale=1.0, psf=psf, variance=1.0 / d["weight"])
    grp = build_group(ap, target, d["init_values"], f"api {name}", d["spec"])
    assert list(grp.parameters.vector_names()) == [str(n) for n in d["names"]]
    assert np.allclose(grp.parameters.vector_representation().numpy(), d["rep0"], atol=1e-12)
    assert close(grp().data.numpy(), d["init_model"])
    J = grp.jacobian(as_representation=True).data.numpy()
    for k in range(J.shape[-1]):
        assert close(J[..., k], d["jac_rep"][..., k], rel=2e-4), k
    res = ap.fit.LM(grp, max_iter=d["spec"]["max_iter"]).fit()
    assert res.message == d["message"]
    assert abs(min(res.loss_history) / d["loss_history"].min() - 1) <= 1e-4


@pytest.mark.parametrize("name", cases.init_case_names())
def test_initialize_matches_reference(ap, name):
    """``model.initialize()`` with no (or some) parameter values, as the reference's
    ``tests/golden/init_*`` recorded it: centre of light, PA, isophote q, profile fit."""
    d = cases.load_init(name)
    spec = d["spec"]
    kw = {} if d["mask"] is None else {"mask": d["mask"]}
    tar = ap.image.Target_Image(data=d["data"], pixelscale=spec["scale"], variance=np.full(d["data"].shape, 0.0025), **kw)
    kind = {"sersic": "sersic galaxy model", "exponential": "exponential galaxy model"}[spec["kind"]]
    given = {k: (list(v) if isinstance(v, list) else v) for k, v in spec.get("given", {}).items()}
    m = ap.models.AstroPhot_Model(name=f"api init {name}", model_type=kind, target=tar, parameters=given)
    m.initialize()
    names = ["center", "q", "PA", "n", "Re", "Ie"] if spec["kind"] == "sersic" else ["center", "q", "PA", "Re", "Ie"]
    for k in names:
        got = m[k].value.detach().cpu().numpy()
        ref = d[f"value_{k}"]
        tol = 1e-9 if k in ("center", "PA", "q") else 1e-3
        assert np.max(np.abs(got - ref) / np.maximum(1.0, np.abs(ref))) <= tol, (k, got, ref)


@pytest.mark.parametrize("name", cases.upscale_case_names())
def test_psf_finer_than_image_matches_reference(ap, name):
    """A PSF image with pixels twice finer than the image's (``PSF_Image(pixelscale=0.5)`` on a
    1"-pixel target): sampled, integrated and convolved on the finer grid and summed back in
    2 x 2 blocks, as the reference does; model, Jacobian and LM against its golden."""
    d = cases.load_upscale(name)
    spec = d["spec"]
    u, scale = spec["upscale"], spec["scale"]
    kind = {"sersic": "sersic galaxy model", "exponential": "exponential galaxy model"}[spec["kind"]]
    tar = ap.image.Target_Image(data=d["data"], pixelscale=scale, variance=1.0 / d["weight"],
                                psf=ap.image.PSF_Image(data=d["psf"], pixelscale=scale / u))
    m = ap.models.AstroPhot_Model(name=f"api {name}", model_type=kind, target=tar, parameters=dict(spec["init"]),
                                  psf_mode="full")
    assert list(m.parameters.vector_names()) == [str(n) for n in d["names"]]
    assert np.allclose(m.parameters.vector_representation().numpy(), d["rep0"], atol=1e-12)
    assert close(m().data.numpy(), d["init_model"])
    J = m.jacobian(as_representation=True).data.numpy()
    for k in range(J.shape[-1]):
        assert close(J[..., k], d["jac_rep"][..., k], rel=2e-4), k
    # the adjoint through the finer grid and the block sums: negative_log_likelihood().backward()
    # against the reference's autograd gradient, and, for the render's own derivative (without
    # the sampling-coordinate path reverse-mode autograd adds to the centre under a PSF shift),
    # against J^T W (model - data) of the reference's Jacobian
    vec = torch.tensor(d["rep0"], dtype=torch.float64, requires_grad=True)
    nll = m.negative_log_likelihood(parameters=vec, as_representation=True)
    assert abs(float(nll.detach()) / float(d["nll"]) - 1) <= 1e-5
    nll.backward()
    want = d["nll_grad"]
    assert np.allclose(vec.grad.numpy(), want, rtol=1e-3, atol=1e-3 * np.max(np.abs(want)))
    m.reference_center_gradient = False
    vec = torch.tensor(d["rep0"], dtype=torch.float64, requires_grad=True)
    m.negative_log_likelihood(parameters=vec, as_representation=True).backward()
    want = np.einsum("yxk,yx->k", d["jac_rep"], d["weight"] * (d["init_model"] - d["data"]))
    assert np.allclose(vec.grad.numpy(), want, rtol=1e-3, atol=1e-3 * np.max(np.abs(want)))
    res = ap.fit.LM(m, max_iter=spec["max_iter"]).fit()
    print(name, res.loss_history, d["loss_history"], res.message)
    assert res.message == d["message"]
    assert abs(min(res.loss_history) / d["loss_history"].min() - 1) <= 1e-5
    assert np.allclose(res.loss_history[:3], d["loss_history"][:3], rtol=1e-5)
    assert np.allclose(res.res(), d["res"], rtol=1e-4, atol=1e-6)


def test_lanczos_shift_adjoint_and_fit_match_oracle(ap):
    """psf_subpixel_shift "lanczos:3": the adjoint (the render's own derivative) against
    J^T W (model - data) of the reference's Jacobian, and LM(model).fit() from a perturbed start
    against the oracle's LM from the same start (a Lanczos stamp's trials render in full)."""
    from oracle.lm import GroupProblem, LMOracle
    from oracle.render import PSF, Component, Window

    d = cases.load_render("sersic_psf_lanczos3")
    spec = d["spec"]
    rng = np.random.default_rng(41)
    var = d["model"] + 10.0
    data = d["model"] + rng.normal(size=d["model"].shape) * np.sqrt(var)
    tar = ap.image.Target_Image(data=data, pixelscale=spec["scale"], psf=d["psf"], variance=var)
    m = ap.models.AstroPhot_Model(name="api lanczos fit", model_type="sersic galaxy model", target=tar,
                                  parameters=dict(spec["params"]), **spec["knobs"])
    m.reference_center_gradient = False
    rep0 = torch.tensor(d["rep"], dtype=torch.float64, requires_grad=True)
    m.negative_log_likelihood(parameters=rep0, as_representation=True).backward()
    want = np.einsum("yxk,yx->k", d["jac_rep"], (d["model"] - data) / var)
    assert np.allclose(rep0.grad.numpy(), want, rtol=1e-3, atol=1e-3 * np.max(np.abs(want)))

    start = dict(spec["params"])
    start.update(center=[spec["params"]["center"][0] + 0.4, spec["params"]["center"][1] - 0.3],
                 q=0.6, PA=1.0, n=2.2, Re=8.8, Ie=1.1)
    m2 = ap.models.AstroPhot_Model(name="api lanczos fit 2", model_type="sersic galaxy model", target=tar,
                                   parameters=start, **spec["knobs"])
    x0 = m2.parameters.vector_representation().numpy().copy()
    res = ap.fit.LM(m2, max_iter=30).fit()
    p = {k: (np.array(v, dtype=float) if k == "center" else v) for k, v in start.items()}
    comp = Component("sersic", p, **spec["knobs"])
    prob = GroupProblem([comp], Window.from_scale(spec["nx"], spec["ny"], spec["scale"]),
                        PSF(d["psf"], spec["scale"]), data, 1.0 / var)
    lm = LMOracle(prob, x0, max_iter=30).fit()
    print(res.loss_history, lm.loss_history, res.message, lm.message)
    assert abs(min(res.loss_history) / min(lm.loss_history) - 1) <= 1e-5
    assert np.allclose(res.res(), lm.res(), rtol=1e-3, atol=1e-4)
