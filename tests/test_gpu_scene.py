"""Scenes on the GPU (many galaxies on one image, joint LM): against the reference's
``Group_Model`` golden (per-component pixel windows, a bulge and a disk sharing one centre
node, PSF convolution) recorded from the reference, and the scene primitives against numpy."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import cases  # noqa: E402


@pytest.fixture(scope="module")
def S():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from astrophot_gb300 import scene

    return scene


# the GROUP_SOURCES of tests/golden/make_golden.py
WINDOWS = (((8, 72), (10, 74)), ((8, 72), (10, 74)), ((50, 96), (36, 90)), ((0, 44), (52, 96)))
KINDS = ("sersic", "exponential", "sersic", "sersic")
LINKS = (None, 0, None, None)


def golden_scene(S, d, values=None):
    """The golden group as a scene: a locked sky of 10^0 = 1 per pixel, or a free flat sky
    (F last in the joint vector, after the galaxies); per-galaxy sampling settings as the
    sources' options."""
    values = d["init_values"] if values is None else values
    spec = d["spec"]
    knobs = spec.get("knobs") or [None] * len(KINDS)
    srcs = [S.SceneSource(k, list(v), w, l, options=o or None)
            for k, v, w, l, o in zip(KINDS, values, WINDOWS, LINKS, knobs)]
    N = spec["size"]
    sky = dict(sky_F=spec["sky_F_init"]) if spec.get("sky_free") else dict(sky=1.0)
    return S.Scene(N, N, srcs, d["psf"], d["data"], d["weight"], psf_upscale=spec.get("psf_upscale", 1), **sky)


@pytest.mark.parametrize("name", cases.group_case_names())
def test_scene_model_and_jacobian_match_reference(S, name):
    d = cases.load_group(name)
    sc = golden_scene(S, d)
    rep0 = sc.representation()
    assert sc.P == len(d["names"])
    assert np.allclose(rep0, d["rep0"], rtol=0, atol=1e-12)
    m = sc.forward(rep0).cpu().numpy().reshape(d["init_model"].shape)
    ref = d["init_model"]
    assert np.max(np.abs(m - ref)) <= 1e-5 * np.max(np.abs(ref)), np.max(np.abs(m - ref)) / np.max(np.abs(ref))
    J = sc.jacobian_image(rep0)
    for k in range(J.shape[-1]):
        rk = d["jac_rep"][..., k]
        err = np.max(np.abs(J[..., k] - rk)) / np.max(np.abs(rk))
        assert err <= 2e-4, (k, err)


@pytest.mark.parametrize("name", cases.group_case_names())
def test_scene_primitives_match_numpy(S, name):
    d = cases.load_group(name)
    sc = golden_scene(S, d)
    rep0 = sc.representation()
    J = sc.jacobian_image(rep0).reshape(-1, sc.P)
    W = d["weight"].astype(np.float32).astype(np.float64).reshape(-1)
    Ht = sc.hess()
    H = Ht.cpu().numpy()
    Hn = J.T @ (W[:, None] * J)
    assert np.max(np.abs(H - Hn)) <= 1e-5 * np.max(np.abs(Hn))
    # the linked centre's entries gather several blocks: in a fixed order, so the same bits
    # every time (and symmetric, each transpose entry being the same sum)
    for _ in range(3):
        assert torch.equal(sc.hess(), Ht)
    assert np.array_equal(H, H.T)
    rng = np.random.default_rng(3)
    v = rng.normal(size=J.shape[0]).astype(np.float32)
    vt = torch.tensor(v, device="cuda")
    jt_t = sc.jt(vt)
    jt = jt_t.cpu().numpy()
    want = J.T @ v.astype(np.float64)
    assert np.max(np.abs(jt - want)) <= 1e-5 * np.max(np.abs(want))
    assert all(torch.equal(sc.jt(vt), jt_t) for _ in range(3))
    h = rng.normal(size=sc.P)
    jv = sc.jvp(torch.tensor(h, device="cuda")).cpu().numpy()
    want = J @ h
    assert np.max(np.abs(jv - want)) <= 1e-5 * np.max(np.abs(want))


@pytest.mark.parametrize("mixed", [True, False])
@pytest.mark.parametrize("n", [7, 32, 100, 257, 1400])
def test_dense_damped_solve_matches_numpy(S, n, mixed):
    """The damped solve (float32 Cholesky + float64 refinement, or the float64 Cholesky) against
    numpy's float64 solve of the reference's damped matrix."""
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, 2 * n))
    H = A @ A.T
    g = rng.normal(size=n)
    L = 0.37
    I = np.eye(n)
    D = np.ones_like(H) - I
    M = H * (I + D / (1 + L)) + L * I * (1 + np.diag(H))
    want = np.linalg.solve(M, g)
    d = cases.load_group(cases.group_case_names()[0])
    sc = golden_scene(S, d)
    sc.P = n
    sc._solve_ws = torch.empty(int(sc.lib.ap_dense_solve_workspace_bytes(n)), dtype=torch.uint8, device="cuda")
    h = sc.solve(torch.tensor(H, device="cuda"), torch.tensor(g, device="cuda"), L, mixed=mixed).cpu().numpy()
    assert sc._last_mixed == mixed  # the mixed solve converged without the float64 fallback
    assert np.allclose(h, want, rtol=1e-9, atol=1e-12 * np.max(np.abs(want)))
    # another right-hand side on the same factor (the geodesic term's solve)
    g2 = rng.normal(size=n)
    h2 = sc.solve(torch.tensor(H, device="cuda"), torch.tensor(g2, device="cuda"), L, reuse=True,
                  mixed=mixed).cpu().numpy()
    want2 = np.linalg.solve(M, g2)
    assert np.allclose(h2, want2, rtol=1e-9, atol=1e-12 * np.max(np.abs(want2)))
    # not positive definite: reported, not solved
    assert sc.solve(torch.tensor(-H, device="cuda"), torch.tensor(g, device="cuda"), 0.0, mixed=mixed) is None


def test_mixed_solve_hands_ill_conditioned_systems_to_float64(S):
    """A system beyond float32's reach (condition 1e12, no damping): the mixed solve reports -1
    with h = 0 through the C ABI, and Scene.solve then returns the float64 factorisation's h."""
    from astrophot_gb300 import _native as N

    n = 200
    rng = np.random.default_rng(11)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    H = (Q * np.logspace(0, -12, n)) @ Q.T
    H = (H + H.T) / 2
    g = rng.normal(size=n)
    d = cases.load_group(cases.group_case_names()[0])
    sc = golden_scene(S, d)
    sc.P = n
    sc._solve_ws = torch.empty(int(sc.lib.ap_dense_solve_workspace_bytes(n)), dtype=torch.uint8, device="cuda")
    Ht, gt = torch.tensor(H, device="cuda"), torch.tensor(g, device="cuda")
    h = torch.full((n,), 7.0, dtype=torch.float64, device="cuda")
    info = torch.zeros(1, dtype=torch.int32, device="cuda")
    N.check(sc.lib.ap_dense_damped_solve_mixed(n, N._ptr(Ht), N._ptr(gt), 0.0, N._ptr(h), N._ptr(sc._solve_ws),
                                               sc._solve_ws.numel(), N._ptr(info), N._stream()), "mixed")
    assert int(info.item()) == -1
    assert torch.all(h == 0)
    got = sc.solve(Ht, gt, 0.0)
    want = sc.solve(Ht, gt, 0.0, mixed=False)
    assert got is not None and not sc._last_mixed
    assert torch.equal(got, want)


@pytest.mark.parametrize("name", cases.group_case_names())
def test_scene_lm_matches_reference(S, name):
    d = cases.load_group(name)
    sc = golden_scene(S, d)
    lm = S.SceneLM(sc, max_iter=d["spec"]["max_iter"]).fit()
    print(name, lm.loss_history, d["loss_history"], lm.message)
    assert lm.message == d["message"]
    assert abs(min(lm.loss_history) / d["loss_history"].min() - 1) <= 1e-4
    # the first steps follow the reference's trajectory
    assert np.allclose(lm.loss_history[:3], d["loss_history"][:3], rtol=1e-5)


@pytest.mark.parametrize("name", cases.group_case_names())
def test_device_staging_equals_host_staging(S, name):
    """Parameter rows staged on the device from a device vector x + alpha v equal the host
    staging of the same vector (values beyond the PA period and far into the limits included)."""
    d = cases.load_group(name)
    sc = golden_scene(S, d)
    rep0 = sc.representation()
    rng = np.random.default_rng(5)
    v = rng.normal(size=sc.P) * 3.0
    alpha = 0.7
    x = rep0 + alpha * v
    sc._stage(x)
    host = sc._stage_d.clone()
    sc.set_stage_base(rep0)
    sc._stage_dev(torch.tensor(rep0, device="cuda"), torch.tensor(v, device="cuda"), alpha)
    dev = sc._stage_d.clone()
    used = sc._stage_rows() >= 0
    if sc.sky_free:
        used[sc._sky_row] = True  # the free sky's F in cell 0 of its row
    assert torch.allclose(dev[used], host[used], rtol=4e-16, atol=0)
    # without the direction vector
    sc._stage_dev(torch.tensor(x, device="cuda"))
    assert torch.allclose(sc._stage_d[used], host[used], rtol=4e-16, atol=0)


@pytest.mark.parametrize("name", cases.group_case_names())
def test_scene_lm_device_loop_equals_host_loop(S, name):
    """The LM with its vectors on the device (one status read per damping trial) takes the host
    loop's steps: the same message, iterations, loss history and fitted vector."""
    d = cases.load_group(name)
    a = S.SceneLM(golden_scene(S, d), max_iter=d["spec"]["max_iter"], device_loop=False).fit()
    b = S.SceneLM(golden_scene(S, d), max_iter=d["spec"]["max_iter"], device_loop=True,
                  precise_trials=False).fit()
    assert b.device_loop and not a.device_loop
    assert a.message == b.message and a.iterations == b.iterations
    np.testing.assert_allclose(b.loss_history, a.loss_history, rtol=1e-9)
    np.testing.assert_allclose(b.L_history, a.L_history, rtol=0)
    np.testing.assert_allclose(b.res(), a.res(), rtol=1e-9, atol=1e-12)


@pytest.mark.parametrize("name", cases.group_case_names())
def test_difference_render_is_precise(S, name):
    """A trial rendered as its difference to the recorded base render against the float64
    oracle's difference, for a change far below float32's resolution of the model (a free sky's
    term included): the plain float32 renders' difference misses it by orders of magnitude more.
    The base point moves every centre off the golden's whole and half pixels: a centre on a
    half pixel rounds to the other pixel under the smallest step (the model jumps there, in the
    reference too), and one on a pixel centre has a zero sub-pixel shift, whose kernel change is
    formed by subtraction."""
    from test_oracle_golden import group_problem

    d = cases.load_group(name)
    sc = golden_scene(S, d)
    rep0 = sc.representation()
    centre = np.array([str(n).startswith("center") for n in d["names"]])
    rep0 = rep0 + np.where(centre, 0.137, 0.0)
    rng = np.random.default_rng(7)
    v = rng.normal(size=sc.P)
    v /= np.linalg.norm(v)
    alpha = 1e-6
    sc.set_stage_base(rep0)
    x, vd = torch.tensor(rep0, device="cuda"), torch.tensor(v, device="cuda")
    Y0 = sc.forward_base_device(x).clone()
    assert torch.equal(Y0, sc.forward_device(x))  # the base render is the plain render
    dY = sc.forward_diff_device(x, vd, alpha).double().cpu().numpy()
    Y1 = sc.forward_device(x, vd, alpha).double().cpu().numpy()
    prob = group_problem(d)
    assert np.allclose(prob.representation() + np.where(centre, 0.137, 0.0), rep0, rtol=0, atol=1e-12)
    want = prob.forward(rep0 + alpha * v) - prob.forward(rep0)
    scale = np.max(np.abs(want))
    err = np.max(np.abs(dY - want)) / scale
    err_plain = np.max(np.abs(Y1 - Y0.double().cpu().numpy() - want)) / scale
    print(name, err, err_plain)
    assert err <= 1e-3 and err <= err_plain / 10, (err, err_plain)
    # chi^2's change W dm (dm - 2 (data - base)) summed in float64 from the float32 images
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    sc.chi2_change_into(sc.forward_diff_device(x, vd, alpha), Y0, out)
    W = d["weight"].reshape(-1).astype(np.float32).astype(np.float64)
    D = d["data"].reshape(-1).astype(np.float32).astype(np.float64)
    y0 = Y0.double().cpu().numpy()
    dchi2 = np.sum(W * dY * (dY - 2 * (D - y0)))
    assert abs(float(out.item()) - dchi2) <= 1e-9 * np.sum(np.abs(W * dY * (dY - 2 * (D - y0))))


def test_scene_with_mask_and_no_psf_matches_oracle(S):
    """Masked pixels and no PSF: model, Jacobian and the joint LM against the oracle."""
    from oracle.lm import GroupProblem, LMOracle
    from oracle.render import Component, Window

    rng = np.random.default_rng(17)
    N = 72
    wins = (((0, 48), (4, 60)), ((20, 72), (10, 72)), ((10, 70), (30, 72)))
    truth = ((22.3, 30.8, 0.6, 0.9, 2.2, 6.0, 1.9), (47.1, 40.2, 0.45, 2.3, 1.0, 9.0, 1.6),
             (39.6, 55.4, 0.8, 0.4, 3.1, 4.0, 2.1))
    kinds = ("sersic", "exponential", "sersic")

    def comps(values):
        out = []
        for k, v, w in zip(kinds, values, wins):
            p = {"center": [v[0], v[1]], "q": v[2], "PA": v[3], "Re": v[5], "Ie": v[6]}
            if k == "sersic":
                p["n"] = v[4]
            out.append(Component(k, p, window=w))
        out.append(Component("flat_sky", {"F": 0.0}, locked=("F",)))
        return out

    prob_t = GroupProblem(comps(truth), Window.from_scale(N, N), None, np.zeros((N, N)))
    img = prob_t.forward(prob_t.representation()).reshape(N, N)
    var = img + 10.0
    data = img + np.sqrt(var) * rng.normal(size=img.shape)
    weight = 1.0 / var
    mask = np.zeros((N, N), bool)
    mask[30:38, 5:30] = True
    mask[::9, ::7] = True
    init = [tuple(np.array(v) * np.array([1, 1, 1.08, 1, 0.9, 1.1, 1]) + np.array([0.5, -0.4, 0, 0.05, 0, 0, -0.05]))
            for v in truth]
    prob = GroupProblem(comps(init), Window.from_scale(N, N), None, data, weight, mask)
    srcs = [S.SceneSource(k, list(v), w) for k, v, w in zip(kinds, init, wins)]
    sc = S.Scene(N, N, srcs, None, data, weight, mask=mask, sky=1.0)
    rep = sc.representation()
    assert np.allclose(rep, prob.representation(), atol=1e-12)
    m = sc.forward(rep).cpu().numpy()
    ref = prob.forward(rep)
    assert np.max(np.abs(m - ref)) <= 1e-5 * np.max(np.abs(ref))
    J = sc.jacobian_image(rep).reshape(-1, sc.P)
    Jr = prob.jacobian(rep)
    for k in range(sc.P):
        assert np.max(np.abs(J[:, k] - Jr[:, k])) <= 2e-4 * np.max(np.abs(Jr[:, k])), k
    lm = S.SceneLM(sc, max_iter=15).fit()
    lmo = LMOracle(prob, rep, max_iter=15).fit()
    print(lm.loss_history, lmo.loss_history)
    assert abs(min(lm.loss_history) / min(lmo.loss_history) - 1) <= 1e-4


@pytest.mark.parametrize("name", cases.iter_case_names())
def test_scene_iter_lm_matches_reference(S, name):
    """``Iter_LM`` (sequential chunks of 7 over the linked group's 25 entries, 5 sweeps) on the
    scene: the reference's sweep losses, message and final state."""
    d = cases.load_iter(name)
    g = cases.load_group(d["spec"]["group"])
    sc = golden_scene(S, g)
    assert np.allclose(sc.representation(), d["rep0"], atol=1e-12)
    it = S.SceneIterLM(sc, chunks=d["spec"]["chunks"], method=d["spec"]["method"], max_iter=d["spec"]["max_iter"]).fit()
    print(it.loss_history, d["loss_history"])
    assert it.ndf == int(d["ndf"])
    assert it.message == d["message"]
    assert np.allclose(it.loss_history, d["loss_history"], rtol=1e-5, atol=0)
    assert np.max(np.abs(it.res() - d["res"])) <= 1e-3


def test_iter_lm_drop_in_api(S):
    """``fit.Iter_LM`` on a drop-in group model built like the reference's tests."""
    import astrophot_gb300 as ap

    d = cases.load_iter(cases.iter_case_names()[0])
    g = cases.load_group(d["spec"]["group"])
    N = g["spec"]["size"]
    tar = ap.image.Target_Image(data=g["data"], pixelscale=1.0, psf=g["psf"], variance=1.0 / g["weight"])
    models = []
    for i, (k, v, w, l) in enumerate(zip(KINDS, g["init_values"], WINDOWS, LINKS)):
        cx, cy, q, PA, n, Re, Ie = v
        p = {"q": q, "PA": PA, "Re": Re, "Ie": Ie}
        if l is None:
            p["center"] = [cx, cy]
        if k == "sersic":
            p["n"] = n
        m = ap.models.AstroPhot_Model(name=f"iterlm {i}", model_type=f"{k} galaxy model", target=tar,
                                      window=[list(w[0]), list(w[1])], parameters=p)
        if l is not None:
            m.parameters["center"].value = models[l].parameters["center"]
        models.append(m)
    sky = ap.models.AstroPhot_Model(name="iterlm sky", model_type="flat sky model", target=tar,
                                    parameters={"F": {"value": 0.0, "locked": True}})
    sky.initialize()
    grp = ap.models.AstroPhot_Model(name="iterlm group", model_type="group model", target=tar,
                                    models=models + [sky], psf_mode="full")
    res = ap.fit.Iter_LM(grp, chunks=7, method="sequential", max_iter=2).fit()
    assert np.allclose(res.loss_history, d["loss_history"][:2], rtol=1e-5)
    assert res.message == "fail max iterations reached: 2"
