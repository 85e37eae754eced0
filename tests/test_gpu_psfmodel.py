"""Fitted parametric PSFs on the GPU against the reference's own outputs
(``tests/golden/auxpsf_48.npz``, Moffat; ``auxpsf_gauss_48.npz``, Gaussian): the PSF model sampled
and normalised on the device, a Sersic galaxy convolved with it (model and Jacobian, the PSF's
parameters leading the vector), the scene LM fitting PSF and galaxy together, and the same
through the drop-in model API."""

import json
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
LOCKED = {"moffat": {"I0": 0.0}, "gaussian": {"flux": 0.0}}


@pytest.fixture(scope="module", params=["auxpsf_48", "auxpsf_gauss_48"])
def case(request):
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    d = np.load(os.path.join(GOLDEN, f"{request.param}.npz"))
    return d, json.loads(str(d["spec"]))


def kind_of(spec):
    return spec.get("psf_kind", "moffat")


def psf_params(spec, which):
    return dict(spec[which]["psf"], **LOCKED[kind_of(spec)])


def make_scene(d, spec, mode="direct"):
    from astrophot_gb300.scene import LivePSF, Scene, SceneSource

    ini = spec["init"]
    k, size = spec["psf_size"], spec["size"]
    live = LivePSF(psf_params(spec, "init"), (k, k), kind=kind_of(spec))
    src = SceneSource("sersic", list(ini["gal"]))
    return Scene(size, size, [src], None, d["data"], d["weight"], psf_model=live,
                 options=dict(psf_convolve_mode=mode))


def test_live_psf_image_matches_reference(case):
    from astrophot_gb300.scene import LivePSF

    d, spec = case
    kind = kind_of(spec)
    for key, img in (("init", d["psf0"]), ("truth", d["truth_psf"])):
        live = LivePSF(psf_params(spec, key), img.shape, kind=kind)
        K = live.image()
        assert np.max(np.abs(K - img)) <= 2e-6 * np.max(img), key
    # d(normalised image) / d(free parameters) against central differences of the float64 oracle
    from oracle.psfmodel import render_psf

    p = psf_params(spec, "init")
    live = LivePSF(p, d["psf0"].shape, kind=kind)
    _, dK = live.render(True)
    dK = dK.cpu().numpy().reshape(len(live.free), *d["psf0"].shape)
    for j, name in enumerate(live.free):
        h = 1e-5 * p[name]
        pp, pm = dict(p), dict(p)
        pp[name] += h
        pm[name] -= h
        fd = (render_psf(pp, d["psf0"].shape, kind=kind)[0] - render_psf(pm, d["psf0"].shape, kind=kind)[0]) / (2 * h)
        assert np.max(np.abs(dK[j] - fd)) <= 2e-4 * np.max(np.abs(fd)), name


@pytest.mark.parametrize("mode", ["direct", "fft"])
def test_scene_with_live_psf_matches_reference(case, mode):
    d, spec = case
    sc = make_scene(d, spec, mode)
    rep0 = d["rep0"]
    assert np.allclose(sc.representation(), rep0, atol=1e-12)
    m = sc.forward(rep0).cpu().numpy().reshape(d["model0"].shape)
    assert np.max(np.abs(m - d["model0"])) <= 1e-5 * np.max(d["model0"])
    J = sc.jacobian_image(rep0)
    for k in range(J.shape[-1]):
        ref = d["jac_rep"][..., k]
        err = np.max(np.abs(J[..., k] - ref)) / np.max(np.abs(ref))
        assert err <= 2e-4, (k, str(d["names"][k]), err)


def test_scene_lm_with_live_psf_matches_reference(case):
    from astrophot_gb300.scene import SceneLM

    d, spec = case
    sc = make_scene(d, spec)
    lm = SceneLM(sc, initial_state=d["rep0"].copy()).fit()
    ref_loss = float(np.min(d["loss_history"]))
    got = float(np.min(lm.loss_history))
    assert abs(got / ref_loss - 1) <= 1e-4, (got, ref_loss)
    assert lm.message == str(d["message"])
    vals = np.concatenate([[sc.live_psf.params[f] for f in sc.live_psf.free], np.asarray(sc.sources[0].params)])
    assert np.allclose(vals, d["final_values"], rtol=2e-3, atol=2e-3), (vals, d["final_values"])


def test_api_galaxy_with_psf_model_fits_like_reference(case):
    """The reference's construction: ``psf=`` a "moffat psf model" / "gaussian psf model" on a
    PSF_Image, ``LM().fit()``."""
    import astrophot_gb300 as ap

    d, spec = case
    ini = spec["init"]
    k = spec["psf_size"]
    psf_t = ap.image.PSF_Image(data=np.ones((k, k)) / k**2, pixelscale=1.0)
    live = ap.models.AstroPhot_Model(name="api psf", model_type=f"{kind_of(spec)} psf model", target=psf_t,
                                     parameters=dict(ini["psf"]))
    assert np.max(np.abs(live().data.numpy() - d["psf0"])) <= 2e-6 * np.max(d["psf0"])
    cx, cy, q, PA, n, Re, Ie = ini["gal"]
    tgt = ap.image.Target_Image(data=d["data"], pixelscale=1.0, variance=1.0 / d["weight"])
    gal = ap.models.AstroPhot_Model(name="api gal", model_type="sersic galaxy model", target=tgt, psf_mode="full",
                                    psf=live, parameters={"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re,
                                                          "Ie": Ie})
    img = gal().data.numpy()
    assert np.max(np.abs(img - d["model0"])) <= 1e-5 * np.max(d["model0"])
    J = gal.jacobian(as_representation=True).data.numpy()
    assert J.shape == d["jac_rep"].shape
    assert np.max(np.abs(J - d["jac_rep"])) <= 2e-4 * np.max(np.abs(d["jac_rep"]))
    res = ap.fit.LM(gal).fit()
    assert res.message == str(d["message"])
    assert np.allclose(gal.parameters.vector_values().numpy(), d["final_values"], rtol=2e-3, atol=2e-3)
    first = "n" if kind_of(spec) == "moffat" else "sigma"
    assert abs(live[first].value.item() - d["final_values"][0]) <= 2e-3 * d["final_values"][0]


def test_live_psf_columns_add_over_sources_and_feed_the_normal_equations(case):
    """Two overlapping galaxies sharing one live PSF: the PSF columns of the pair are the sums of
    each galaxy's own (the model is a sum), and the device J^T W J, J^T v and J h over the joint
    vector (PSF entries first) equal the dense products of the assembled Jacobian."""
    from astrophot_gb300.scene import LivePSF, Scene, SceneSource

    d, spec = case
    rng = np.random.default_rng(3)
    size = 64
    gals = [[24.3, 27.6, 0.7, 1.0, 1.5, 2.5, 2.2], [37.1, 33.4, 0.5, 2.2, 2.5, 3.5, 1.8]]
    wins = [((8, 44), (10, 46)), ((20, 60), (14, 54))]
    data = rng.normal(size=(size, size)) + 1.0
    weight = rng.uniform(0.5, 1.5, size=(size, size))
    kind = kind_of(spec)
    psf = dict(n=2.7, Rd=2.1, I0=0.0) if kind == "moffat" else dict(sigma=1.8, flux=0.0)

    def scene(idx):
        return Scene(size, size, [SceneSource("sersic", gals[i], wins[i]) for i in idx], None, data, weight,
                     psf_model=LivePSF(psf, (15, 15), kind=kind))

    both, one, two = scene([0, 1]), scene([0]), scene([1])
    Jb = both.jacobian_image(both.representation())
    J1 = one.jacobian_image(one.representation())
    J2 = two.jacobian_image(two.representation())
    m = both.n_psf
    for c in range(m):
        ref = J1[..., c] + J2[..., c]
        assert np.max(np.abs(Jb[..., c] - ref)) <= 1e-5 * np.max(np.abs(ref)), c
    assert np.allclose(Jb[..., m : m + 7], J1[..., m:], rtol=0, atol=1e-6 * np.abs(J1).max())
    assert np.allclose(Jb[..., m + 7 :], J2[..., m:], rtol=0, atol=1e-6 * np.abs(J2).max())
    # normal equations on the device against the dense Jacobian
    both.jacobian(both.representation())
    H = both.hess().cpu().numpy()
    Jf = Jb.reshape(-1, both.P).astype(np.float64)
    w = weight.reshape(-1)
    Href = Jf.T @ (Jf * w[:, None])
    assert np.max(np.abs(H - Href)) <= 1e-4 * np.max(np.abs(Href))
    v = torch.tensor(rng.normal(size=size * size), dtype=torch.float32, device="cuda")
    g = both.jt(v).cpu().numpy()
    gref = Jf.T @ v.cpu().numpy().astype(np.float64)
    assert np.max(np.abs(g - gref)) <= 1e-4 * np.max(np.abs(gref))
    h = torch.tensor(rng.normal(size=both.P), dtype=torch.float64, device="cuda")
    jh = both.jvp(h).cpu().numpy()
    jhref = Jf @ h.cpu().numpy()
    assert np.max(np.abs(jh - jhref)) <= 1e-4 * np.max(np.abs(jhref))


def test_concurrent_scene_fits_equal_sequential_ones(case):
    """fit_scenes: independent live-PSF fits on worker streams end exactly where the same fits
    run one after another end."""
    from astrophot_gb300.scene import SceneLM, fit_scenes

    d, spec = case
    scenes = [make_scene(d, spec) for _ in range(4)]
    x0 = d["rep0"].copy()
    for k, sc in enumerate(scenes):  # four different starting points
        x0k = x0.copy()
        x0k[2] += 0.1 * k
        scenes[k]._x0 = x0k
    seq = [SceneLM(sc, initial_state=sc._x0.copy()).fit() for sc in scenes]
    con = fit_scenes(scenes, [sc._x0 for sc in scenes], workers=4)
    for a, b in zip(seq, con):
        assert a.message == b.message
        assert np.array_equal(np.asarray(a.loss_history), np.asarray(b.loss_history))
        assert np.array_equal(a.res(), b.res())


def test_adjoint_with_live_psf_matches_reference_jacobian(case):
    """The scene adjoint with a live PSF (PSF entries included) equals J^T g of the reference's
    Jacobian, and the drop-in nll().backward() gives the reference's gradient sum W (M - D) dM."""
    import astrophot_gb300 as ap

    d, spec = case
    sc = make_scene(d, spec)
    rng = np.random.default_rng(9)
    g = rng.normal(size=d["model0"].shape)
    got = sc.vjp(d["rep0"], torch.tensor(g, dtype=torch.float32)).numpy()
    ref = np.einsum("yxk,yx->k", d["jac_rep"], g)
    assert np.max(np.abs(got - ref)) <= 1e-4 * np.max(np.abs(ref)), (got, ref)

    ini = spec["init"]
    k = spec["psf_size"]
    psf_t = ap.image.PSF_Image(data=np.ones((k, k)) / k**2, pixelscale=1.0)
    live = ap.models.AstroPhot_Model(name="nll psf", model_type=f"{kind_of(spec)} psf model", target=psf_t,
                                     parameters=dict(ini["psf"]))
    cx, cy, q, PA, n, Re, Ie = ini["gal"]
    tgt = ap.image.Target_Image(data=d["data"], pixelscale=1.0, variance=1.0 / d["weight"])
    gal = ap.models.AstroPhot_Model(name="nll gal", model_type="sersic galaxy model", target=tgt, psf_mode="full",
                                    psf=live, parameters={"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re,
                                                          "Ie": Ie})
    gal.reference_center_gradient = False  # the render's derivative, which the Jacobian holds
    vec = torch.tensor(d["rep0"], dtype=torch.float64, requires_grad=True)
    nll = gal.negative_log_likelihood(parameters=vec, as_representation=True)
    nll.backward()
    gref = np.einsum("yxk,yx->k", d["jac_rep"], d["weight"] * (d["model0"] - d["data"]))
    assert np.max(np.abs(vec.grad.numpy() - gref)) <= 1e-3 * np.max(np.abs(gref)), (vec.grad.numpy(), gref)


def test_api_group_with_live_psf_and_sky_fits_like_reference():
    """``auxpsf_group_48``: Group_Model([galaxy with psf= a moffat psf model, locked flat sky],
    psf_mode="full") through the drop-in API: model, Jacobian (the PSF's n and Rd first) and
    ``LM(group).fit()`` against the reference's own."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import astrophot_gb300 as ap

    d = np.load(os.path.join(GOLDEN, "auxpsf_group_48.npz"))
    spec = json.loads(str(d["spec"]))
    ini = spec["init"]
    k = spec["psf_size"]
    psf_t = ap.image.PSF_Image(data=np.ones((k, k)) / k**2, pixelscale=1.0)
    tgt = ap.image.Target_Image(data=d["data"], pixelscale=1.0, variance=1.0 / d["weight"])
    live = ap.models.AstroPhot_Model(name="grp psf", model_type="moffat psf model", target=psf_t,
                                     parameters=dict(ini["psf"]))
    cx, cy, q, PA, n, Re, Ie = ini["gal"]
    gal = ap.models.AstroPhot_Model(name="grp gal", model_type="sersic galaxy model", target=tgt, psf_mode="full",
                                    psf=live, parameters={"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re,
                                                          "Ie": Ie})
    sky = ap.models.AstroPhot_Model(name="grp sky", model_type="flat sky model", target=tgt,
                                    parameters={"F": {"value": 0.0, "locked": True}})
    sky.initialize()
    grp = ap.models.AstroPhot_Model(name="grp", model_type="group model", target=tgt, models=[gal, sky],
                                    psf_mode="full")
    assert [str(x) for x in grp.parameters.vector_names()] == [str(x) for x in d["names"]]
    img = grp().data.numpy()
    assert np.max(np.abs(img - d["model0"])) <= 1e-5 * np.max(d["model0"])
    J = grp.jacobian(as_representation=True).data.numpy()
    assert np.max(np.abs(J - d["jac_rep"])) <= 2e-4 * np.max(np.abs(d["jac_rep"]))
    res = ap.fit.LM(grp).fit()
    assert res.message == str(d["message"])
    assert np.allclose(grp.parameters.vector_values().numpy(), d["final_values"], rtol=2e-3, atol=2e-3)
