"""The adjoint of the render (``ap_render_vjp``) on the GPU: against the gradient of the
reference's negative log-likelihood recorded from the reference itself (reverse-mode autograd
``grad`` and forward-mode ``jacobian()`` contracted with the residual ``grad_fwd``), against the
library's own Jacobian, through ``torch.autograd`` and through the drop-in ``Model``
``negative_log_likelihood().backward()``."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import cases  # noqa: E402


@pytest.fixture(scope="module")
def N():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from astrophot_gb300 import _native

    return _native


def full_init(d):
    v = np.r_[d["init"], 0.0]
    if d["spec"]["model"] != "sersic":
        v[4] = 1.0
    return v


def vjp_batch(N, d):
    spec = d["spec"]
    size = spec["size"]
    psf = d["psf"] if d["psf"].size else None
    free = 0x7F if spec["model"] == "sersic" else (0x7F & ~(1 << 4))
    opts = N.make_options(profile=spec["model"], psf_mode="full" if psf is not None else "none", free_mask=free,
                          has_sky=False)
    b = N.StampBatch([(size, size)], None if psf is None else [psf.shape[::-1]], N.scale_geometry(1), opts)
    return b, (None if psf is None else b.pack_psf([psf]))


def residual_weights(b, d, model):
    """W (model - data) on unmasked pixels, zero on masked ones (float64, output layout)."""
    m = model.to(torch.float64)
    r = b.pack([d["weight"]], torch.float64) * (m - b.pack([d["data"]], torch.float64))
    keep = torch.logical_not(b.pack([d["mask"].astype(np.uint8)], torch.uint8).bool())
    return torch.where(keep, r, torch.zeros_like(r))


# FP32 render and FP32 per-thread partial sums: the gradient agrees with the FP64 reference
# to this fraction of its largest entry
VJP_REL = 1e-5


@pytest.mark.parametrize("name", cases.vjp_case_names())
def test_vjp_matches_reference_gradient(N, name):
    d = cases.load_vjp(name)
    b, psf = vjp_batch(N, d)
    params = torch.tensor(full_init(d)[None, :])
    model = b.render(params, psf)
    g = residual_weights(b, d, model)
    scale = np.max(np.abs(d["grad_fwd"]))
    exact = b.vjp(params, psf, g, as_representation=True).cpu().numpy()[0]
    print(name, "render derivative", exact, "reference forward mode", d["grad_fwd"])
    assert np.max(np.abs(exact - d["grad_fwd"])) <= VJP_REL * scale
    quirk = b.vjp(params, psf, g, as_representation=True, reference_center=True).cpu().numpy()[0]
    print(name, "reference-center", quirk, "reference reverse mode", d["grad"])
    assert np.max(np.abs(quirk - d["grad"])) <= VJP_REL * np.max(np.abs(d["grad"]))
    if d["psf"].size == 0:
        # no PSF shift: both flags give the same sums
        assert np.array_equal(exact, quirk)


@pytest.mark.parametrize("name", cases.vjp_case_names())
def test_vjp_is_jacobian_transpose(N, name):
    """vjp(g) == J^T g for a random g, J from ap_jacobian, value and representation space."""
    d = cases.load_vjp(name)
    b, psf = vjp_batch(N, d)
    params = torch.tensor(full_init(d)[None, :])
    rng = np.random.default_rng(11)
    g = torch.tensor(rng.normal(size=b.out_pixels), dtype=torch.float32, device=b.device)
    for rep in (False, True):
        _, jac = b.jacobian(params, psf, as_representation=rep)
        J = jac.to(torch.float64).reshape(b.n_free, -1)
        want = (J @ g.to(torch.float64)).cpu().numpy()
        got = b.vjp(params, psf, g, as_representation=rep).cpu().numpy()[0]
        assert np.max(np.abs(got - want)) <= 1e-5 * np.max(np.abs(want)), (got, want)


def test_vjp_batched_equals_single(N):
    """Stamps of one batch are independent: each stamp's VJP equals the VJP of that stamp alone."""
    from astrophot_gb300 import synthetic

    specs = synthetic.cutout_stamps(4, seed=21, lo=24, hi=80)
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0xFF, has_sky=True)
    shapes = [(s.nx, s.ny) for s in specs]
    kshapes = [(s.psf.shape[1], s.psf.shape[0]) for s in specs]
    big = N.StampBatch(shapes, kshapes, N.scale_geometry(len(specs)), opts)
    params = torch.tensor(np.array([np.r_[s.init, 0.2] for s in specs]))
    psf = big.pack_psf([s.psf for s in specs])
    rng = np.random.default_rng(4)
    gs = [rng.normal(size=(s.ny, s.nx)).astype(np.float32) for s in specs]
    out = big.vjp(params, psf, big.pack(gs), as_representation=True).cpu().numpy()
    for i, s in enumerate(specs):
        one = N.StampBatch([shapes[i]], [kshapes[i]], N.scale_geometry(1), opts)
        o1 = one.vjp(params[i : i + 1], one.pack_psf([s.psf]), one.pack([gs[i]]), as_representation=True).cpu().numpy()
        assert np.array_equal(o1[0], out[i])


def test_autograd_render(N):
    """``astrophot_gb300.autograd.render``: loss = sum(c * model) backpropagates J^T c to the
    fitted slots and zero to the locked ones."""
    from astrophot_gb300.autograd import render

    d = cases.load_vjp("vjp_sersic_96")
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0x7F & ~(1 << 3), has_sky=False)
    b = N.StampBatch([(96, 96)], [(25, 25)], N.scale_geometry(1), opts)
    psf = b.pack_psf([d["psf"]])
    params = torch.tensor(full_init(d)[None, :], device=b.device, requires_grad=True)
    c = torch.tensor(np.random.default_rng(2).normal(size=b.out_pixels), dtype=torch.float32, device=b.device)
    loss = torch.sum(c * render(b, params, psf))
    loss.backward()
    _, jac = b.jacobian(params.detach(), psf, as_representation=False)
    want = (jac.to(torch.float64).reshape(b.n_free, -1) @ c.to(torch.float64)).cpu().numpy()
    got = params.grad.cpu().numpy()[0]
    assert got[3] == 0.0 and got[7] == 0.0
    assert np.max(np.abs(got[[0, 1, 2, 4, 5, 6]] - want)) <= 1e-5 * np.max(np.abs(want))


@pytest.mark.parametrize("name", cases.vjp_case_names())
def test_model_nll_backward_matches_reference(name):
    """The drop-in: ``model.negative_log_likelihood(parameters=rep, as_representation=True)``
    then ``.backward()``, as a user of the reference writes it."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import astrophot_gb300 as ap

    d = cases.load_vjp(name)
    spec = d["spec"]
    psf = d["psf"] if d["psf"].size else None
    kw = dict(pixelscale=1.0) if psf is None else dict(pixelscale=1.0, psf=psf)
    target = ap.image.Target_Image(data=d["data"], variance=1.0 / d["weight"], mask=d["mask"], **kw)
    cx, cy, q, PA, n, Re, Ie = [float(v) for v in d["init"]]
    params = {"center": [cx, cy], "q": q, "PA": PA, "Re": Re, "Ie": Ie}
    if spec["model"] == "sersic":
        params["n"] = n
    model = ap.models.AstroPhot_Model(name=f"vjp api {name}", model_type=f"{spec['model']} galaxy model", target=target,
                                      psf_mode="full" if psf is not None else "none", parameters=params)
    for reference_center, key in ((True, "grad"), (False, "grad_fwd")):
        model.reference_center_gradient = reference_center
        rep = model.parameters.vector_representation().detach().clone().requires_grad_(True)
        nll = model.negative_log_likelihood(parameters=rep, as_representation=True)
        assert nll.item() == pytest.approx(float(d["nll"]), rel=1e-5)
        nll.backward()
        ref = d[key]
        assert np.max(np.abs(rep.grad.numpy() - ref)) <= VJP_REL * np.max(np.abs(ref)), (rep.grad, ref)


# ---- the adjoint of a scene: bulge + disk pairs sharing centres, windows, 65 x 65 PSF ---------


def adjoint_scene(d):
    from astrophot_gb300 import scene as SC

    srcs = []
    for k, (c, w, b, dk) in enumerate(zip(d["centers"], d["windows"], d["bulges"], d["disks"])):
        win = tuple(tuple(int(v) for v in r) for r in w)
        q, PA, n, Re, Ie = b
        srcs.append(SC.SceneSource("sersic", [c[0], c[1], q, PA, n, Re, Ie], win))
        q, PA, Re, Ie = dk
        srcs.append(SC.SceneSource("exponential", [c[0], c[1], q, PA, 1.0, Re, Ie], win, link_center=2 * k))
    N = d["spec"]["size"]
    return SC.Scene(N, N, srcs, d["psf"], d["data"], d["weight"], sky=1.0)


@pytest.mark.parametrize("name", cases.adjoint_case_names())
def test_scene_adjoint_matches_reference_autograd(N, name):
    """The scene's adjoint (render VJPs, PSF-convolved tiles recomputed) against the reference's
    negative_log_likelihood().backward() on a 256 x 256 crop of bulge + disk pairs."""
    d = cases.load_adjoint(name)
    sc = adjoint_scene(d)
    rep = sc.representation()
    assert np.allclose(rep, d["rep"], atol=1e-12)
    model = sc.forward(rep)
    assert np.max(np.abs(model.cpu().numpy() - d["model"].reshape(-1))) <= 1e-5 * np.max(d["model"])
    g = sc.weight.double() * (model.double() - sc.data.double())
    quirk = sc.vjp(rep, g.float(), reference_center=True).numpy()
    scale = np.max(np.abs(d["grad"]))
    print(name, "reverse-mode", np.max(np.abs(quirk - d["grad"])) / scale)
    # FP32 renders and 65 x 65-tap FP32 convolution sums over ~10^5 pixels per source: measured
    # 3.8e-5 of the largest entry
    assert np.max(np.abs(quirk - d["grad"])) <= 1e-4 * scale
    exact = sc.vjp(rep, g.float()).numpy()
    centre = np.array([str(n).startswith("center") for n in d["names"]])
    assert np.array_equal(exact[~centre], quirk[~centre])
    # centre entries: the derivative through the PSF shift, as the Jacobian-based gradient
    sc.jacobian(rep)
    jt = sc.jt((-g).float().contiguous()).cpu().numpy() * -1.0
    assert np.max(np.abs(exact[centre] - jt[centre])) <= 1e-4 * scale


@pytest.mark.parametrize("name", cases.adjoint_case_names())
def test_group_nll_backward_matches_reference(name):
    """The drop-in: a Group_Model of linked bulge + disk pairs, nll.backward()."""
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    import astrophot_gb300 as ap

    d = cases.load_adjoint(name)
    target = ap.image.Target_Image(data=d["data"], pixelscale=1.0, psf=d["psf"], variance=1.0 / d["weight"])
    models = []
    for k, (c, w, b, dk) in enumerate(zip(d["centers"], d["windows"], d["bulges"], d["disks"])):
        win = [[int(w[0][0]), int(w[0][1])], [int(w[1][0]), int(w[1][1])]]
        q, PA, n, Re, Ie = [float(v) for v in b]
        bulge = ap.models.AstroPhot_Model(name=f"bulge {k}", model_type="sersic galaxy model", target=target,
                                          window=win, parameters={"center": [float(c[0]), float(c[1])], "q": q,
                                                                  "PA": PA, "n": n, "Re": Re, "Ie": Ie})
        q, PA, Re, Ie = [float(v) for v in dk]
        disk = ap.models.AstroPhot_Model(name=f"disk {k}", model_type="exponential galaxy model", target=target,
                                         window=win, parameters={"q": q, "PA": PA, "Re": Re, "Ie": Ie})
        disk.parameters["center"].value = bulge.parameters["center"]
        models += [bulge, disk]
    sky = ap.models.AstroPhot_Model(name="sky", model_type="flat sky model", target=target,
                                    parameters={"F": {"value": 0.0, "locked": True}})
    sky.initialize()
    grp = ap.models.AstroPhot_Model(name="bulge disk group", model_type="group model", target=target,
                                    models=models + [sky], psf_mode="full")
    assert [str(n) for n in grp.parameters.vector_names()] == [str(n) for n in d["names"]]
    rep = grp.parameters.vector_representation().detach().clone().requires_grad_(True)
    nll = grp.negative_log_likelihood(parameters=rep, as_representation=True)
    assert nll.item() == pytest.approx(float(d["nll"]), rel=1e-5)
    nll.backward()
    assert np.max(np.abs(rep.grad.numpy() - d["grad"])) <= 1e-4 * np.max(np.abs(d["grad"]))
