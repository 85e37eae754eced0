"""CUDA path (through the C ABI) against the reference's golden vectors and the oracle.

Tolerances (FP32 rendering against float64):
  model images : max |gpu - ref| <= 1e-5 * max |ref|, and per pixel <= 1e-5 relative where
                 |ref| > 1e-3 max |ref|
  Jacobians    : per column max |gpu - ref| <= 2e-4 * max |ref column|
  LM           : the reference's message and iteration count, final chi2/ndf and fitted
                 value-space parameters within 1e-4 relative, loss history within 1e-6
"""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu

import cases  # noqa: E402
from oracle.lm import GroupProblem, LMOracle  # noqa: E402
from oracle.render import (  # noqa: E402
    PSF,
    Component,
    Window,
    sample_component,
    sample_group,
    shift_psf_bilinear,
)


@pytest.fixture(scope="module")
def N():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from astrophot_gb300 import _native

    return _native


def assert_image_close(got, ref, rel=1e-5, pix=1e-5):
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) <= rel * scale, np.max(np.abs(got - ref)) / scale
    bright = np.abs(ref) > 1e-3 * scale
    r = np.abs(got - ref)[bright] / np.abs(ref)[bright]
    assert r.max() <= pix, r.max()


def full_params(spec):
    p = spec["params"]
    return np.array([p["center"][0], p["center"][1], p["q"], p["PA"], p.get("n", 1.0), p["Re"], p["Ie"], 0.0])


def batch_for_case(N, d, free_mask=None, has_sky=False):
    spec = d["spec"]
    knobs = spec["knobs"]
    kind = spec["kind"]
    if free_mask is None:
        free_mask = 0x7F if kind == "sersic" else (0x7F & ~(1 << 4))
    opts = N.make_options(
        profile=kind,
        sampling_mode=knobs.get("sampling_mode", "midpoint"),
        integrate_mode=knobs.get("integrate_mode", "threshold"),
        psf_mode=knobs.get("psf_mode", "none"),
        psf_subpixel_shift=knobs.get("psf_subpixel_shift", "bilinear"),
        free_mask=free_mask,
        has_sky=has_sky,
    )
    psf = d["psf"] if d["psf"].size else None
    b = N.StampBatch(
        [(spec["nx"], spec["ny"])],
        [(psf.shape[1], psf.shape[0])] if psf is not None else None,
        N.scale_geometry(1, spec["scale"]),
        opts,
    )
    return b, (b.pack_psf([psf]) if psf is not None else None)


@pytest.mark.parametrize("name", cases.render_case_names())
def test_render_and_jacobian_match_reference(N, name):
    d = cases.load_render(name)
    spec = d["spec"]
    b, psf = batch_for_case(N, d)
    params = torch.tensor(full_params(spec)[None, :])
    model = b.unpack(b.render(params, psf))[0]
    assert_image_close(model, d["model"])
    m2, jac = b.jacobian(params, psf, as_representation=True)
    assert_image_close(b.unpack(m2)[0], d["model"])
    J = jac.cpu().numpy().reshape(b.n_free, spec["ny"], spec["nx"])
    for k in range(b.n_free):
        ref = d["jac_rep"][..., k]
        assert np.max(np.abs(J[k] - ref)) <= 2e-4 * np.max(np.abs(ref)), (k, np.max(np.abs(J[k] - ref)) / np.max(np.abs(ref)))
    _, jv = b.jacobian(params, psf, as_representation=False)
    Jv = jv.cpu().numpy().reshape(b.n_free, spec["ny"], spec["nx"])
    for k in range(b.n_free):
        ref = d["jac_val"][..., k]
        assert np.max(np.abs(Jv[k] - ref)) <= 2e-4 * np.max(np.abs(ref))


@pytest.mark.parametrize("tag", ["locked", "free"])
def test_galaxy_plus_sky_matches_reference(N, tag):
    d = cases.load_render("sersic_psf_64")
    spec = d["spec"]
    F = 0.3 if tag == "free" else 0.0
    free = 0xFF if tag == "free" else 0x7F
    b, psf = batch_for_case(N, d, free_mask=free, has_sky=True)
    p = full_params(spec)
    p[7] = F
    params = torch.tensor(p[None, :])
    model, jac = b.jacobian(params, psf, as_representation=True)
    assert_image_close(b.unpack(model)[0], d[f"group_{tag}_model"])
    J = jac.cpu().numpy().reshape(b.n_free, spec["ny"], spec["nx"])
    refJ = d[f"group_{tag}_jac_rep"]
    assert refJ.shape[-1] == b.n_free
    for k in range(b.n_free):
        assert np.max(np.abs(J[k] - refJ[..., k])) <= 2e-4 * np.max(np.abs(refJ[..., k]))


def test_psf_shift_matches_oracle(N):
    d = cases.load_render("sersic_psf_n4")
    spec = d["spec"]
    b, psf = batch_for_case(N, d)
    params = torch.tensor(full_params(spec)[None, :])
    k, dk = b.psf_shift(params, psf)
    ky, kx = d["psf"].shape
    kp = (ky + 2) * (kx + 2)
    got = k[0, :kp].cpu().numpy().reshape(ky + 2, kx + 2)
    # centre (20.2, 23.9) in pixels of the window padded by the PSF border (reference pixel
    # (-0.5, -0.5) + border, scale 1): shift = pc - round(pc)
    bx, by = (kx + 1) // 2, (ky + 1) // 2
    pc = np.array([20.2 - 0.5 + bx, 23.9 - 0.5 + by])
    shift = pc - np.round(pc)
    s, dsx, dsy = shift_psf_bilinear(d["psf"], shift, True)
    S = s.sum()
    ref = s / S
    assert np.max(np.abs(got - ref)) <= 1e-6 * np.max(ref)
    gx = dk[0, 0, :kp].cpu().numpy().reshape(ky + 2, kx + 2)
    refx = dsx / S - s * dsx.sum() / S**2
    assert np.max(np.abs(gx - refx)) <= 1e-5 * np.max(np.abs(refx))


def test_damped_solve_matches_numpy(N):
    rng = np.random.default_rng(0)
    m, p = 64, 7
    A = rng.normal(size=(m, 40, p))
    H = np.einsum("mki,mkj->mij", A, A)
    g = rng.normal(size=(m, p))
    L = 10.0 ** rng.uniform(-6, 6, size=m)
    h = N.damped_solve(torch.tensor(H).cuda(), torch.tensor(g).cuda(), torch.tensor(L).cuda()).cpu().numpy()
    for i in range(m):
        I = np.eye(p)
        D = np.ones((p, p)) - I
        M = H[i] * (I + D / (1 + L[i])) + L[i] * I * (1 + np.diag(H[i]))
        assert np.allclose(h[i], np.linalg.solve(M, g[i]), rtol=1e-9, atol=1e-12)


def test_chi2_matches_numpy(N):
    d = cases.load_render("sersic_psf_64")
    b, psf = batch_for_case(N, d)
    params = torch.tensor(full_params(d["spec"])[None, :])
    model = b.render(params, psf)
    rng = np.random.default_rng(5)
    m = b.unpack(model)[0].astype(np.float64)
    data = (m + rng.normal(size=m.shape)).astype(np.float32)
    w = rng.uniform(0.5, 2, size=m.shape).astype(np.float32)
    mask = np.zeros(m.shape, dtype=np.uint8)
    mask[3, 4] = 1
    c = b.chi2(b.pack([data]), b.pack([w]), b.pack([mask], torch.uint8), model).item()
    mf = b.unpack(model)[0].astype(np.float32)
    ref = np.sum(((data.astype(np.float64) - mf) ** 2 * w)[mask == 0])
    assert c == pytest.approx(ref, rel=1e-6)


def lm_case_problem(d):
    size = d["spec"]["size"]
    cx, cy, q, PA, n, Re, Ie = d["init"]
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
    sky = Component("flat_sky", {"F": 0.0}, locked=("F",))
    return GroupProblem([gal, sky], Window.from_scale(size, size), PSF(d["psf"]), d["data"], d["weight"])


@pytest.mark.parametrize("name", cases.lm_case_names())
@pytest.mark.parametrize("graph", [False, True])
def test_lm_matches_reference(N, name, graph):
    """The reference's own fit, reproduced: same message and iteration count, final chi2/ndf
    within 1e-4 relative, fitted value-space parameters within 1e-4 relative, and the loss
    history within 1e-6 relative at every iteration.  The damping trials are rendered as
    differences to the step's base point (precise_trials), so the damping search takes the
    float64 reference's decisions down to chi^2 changes of 1e-10."""
    from astrophot_gb300.transforms import rep_to_slots

    d = cases.load_lm(name)
    size = d["spec"]["size"]
    sampling = d["spec"].get("sampling_mode", "midpoint")
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0x7F, has_sky=True, sampling_mode=sampling,
                          integrate_mode="none" if sampling == "midpoint_center" else "threshold")
    b = N.StampBatch([(size, size)], [(25, 25)], N.scale_geometry(1), opts)
    fixed = torch.tensor(np.r_[d["init"], 0.0][None, :])
    state, chi2, iters, status = b.lm_fit(
        b.pack([d["data"]]),
        b.pack([d["weight"]]),
        None,
        b.pack_psf([d["psf"]]),
        fixed,
        torch.tensor(d["rep0"][None, :]),
        N.make_lm_options(use_graph=graph),
    )
    ref_chi2 = d["loss_history"].min()
    assert abs(chi2.item() / ref_chi2 - 1) <= 1e-4
    assert N.LM_MESSAGES[status.item()] == d["message"]
    assert iters.item() == len(d["loss_history"]) - 1
    vals = rep_to_slots(state.cpu().numpy(), fixed.numpy(), 0x7F)[0][:7]
    rel = np.abs(vals - d["final_values"]) / np.abs(d["final_values"])
    print(name, "fitted value-space parameters, relative offset", rel)
    assert np.all(rel <= 1e-4), rel
    loss, L, xs = b.lm_history()
    np.testing.assert_allclose(loss[0, : iters.item() + 1].cpu().numpy(), d["loss_history"], rtol=1e-6)
    # the damping values too, up to the last step: there the competing trials' chi^2 values differ
    # by ~1e-14 relative (steps at L and L / 9 of a change of ~1e-8), the reference's own float64
    # rounding, so which of them it keeps is decided by that rounding
    n = iters.item()
    np.testing.assert_allclose(L[0, :n].cpu().numpy(), d["L_history"][:n], rtol=1e-9)


def test_lm_plain_trials_option(N):
    """precise_trials=False keeps the plain FP32 trial renders: the same fit ends at the same
    chi2 within 1e-4 (its decisions near convergence follow FP32 rounding instead)."""
    d = cases.load_lm("lm_64")
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0x7F, has_sky=True)
    b = N.StampBatch([(64, 64)], [(25, 25)], N.scale_geometry(1), opts)
    args = (b.pack([d["data"]]), b.pack([d["weight"]]), None, b.pack_psf([d["psf"]]),
            torch.tensor(np.r_[d["init"], 0.0][None, :]), torch.tensor(d["rep0"][None, :]))
    _, c_plain, _, s_plain = b.lm_fit(*args, N.make_lm_options(precise_trials=False))
    _, c_prec, _, s_prec = b.lm_fit(*args, N.make_lm_options())
    assert abs(c_plain.item() / d["loss_history"].min() - 1) <= 1e-4
    assert abs(c_prec.item() / d["loss_history"].min() - 1) <= 1e-4


def test_batched_equals_single(N):
    """Stamps are independent: one batch of uneven stamps reproduces each stamp fitted alone,
    bit for bit (fixed per-stamp reduction order)."""
    from astrophot_gb300 import synthetic
    from astrophot_gb300.transforms import slots_to_rep

    specs = synthetic.cutout_stamps(5, seed=3, lo=24, hi=72)
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0x7F, has_sky=True)
    shapes = [(s.nx, s.ny) for s in specs]
    kshapes = [(s.psf.shape[1], s.psf.shape[0]) for s in specs]
    big = N.StampBatch(shapes, kshapes, N.scale_geometry(len(specs)), opts)
    truth = np.array([np.r_[s.truth, 0.0] for s in specs])
    init = np.array([np.r_[s.init, 0.0] for s in specs])
    psf = big.pack_psf([s.psf for s in specs])
    models = big.unpack(big.render(torch.tensor(truth), psf))
    datas, ws = [], []
    for s, m in zip(specs, models):
        dd, ww = synthetic.add_noise(m.astype(np.float64), s.seed)
        datas.append(dd.astype(np.float32))
        ws.append(ww.astype(np.float32))
    lmo = N.make_lm_options()
    st, c2, it, stt = big.lm_fit(big.pack(datas), big.pack(ws), None, psf, torch.tensor(init),
                                 torch.tensor(slots_to_rep(init, 0x7F)), lmo)
    for i, s in enumerate(specs):
        one = N.StampBatch([shapes[i]], [kshapes[i]], N.scale_geometry(1), opts)
        st1, c21, it1, stt1 = one.lm_fit(one.pack([datas[i]]), one.pack([ws[i]]), None, one.pack_psf([s.psf]),
                                         torch.tensor(init[i : i + 1]), torch.tensor(slots_to_rep(init[i : i + 1], 0x7F)), lmo)
        assert c21.item() == c2[i].item()
        assert it1.item() == it[i].item()
        assert np.array_equal(st1.cpu().numpy()[0], st.cpu().numpy()[i])


def test_uneven_batch_render_matches_oracle(N):
    """Many stamps of different sizes / PSFs in one launch, each checked against the oracle."""
    from astrophot_gb300 import synthetic

    specs = synthetic.cutout_stamps(6, seed=9, lo=20, hi=90)
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0x7F, has_sky=True)
    b = N.StampBatch([(s.nx, s.ny) for s in specs], [(s.psf.shape[1], s.psf.shape[0]) for s in specs],
                     N.scale_geometry(len(specs)), opts)
    truth = np.array([np.r_[s.truth, 0.0] for s in specs])
    got = b.unpack(b.render(torch.tensor(truth), b.pack_psf([s.psf for s in specs])))
    for s, g in zip(specs, got):
        cx, cy, q, PA, n, Re, Ie = s.truth
        gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
        sky = Component("flat_sky", {"F": 0.0}, locked=("F",))
        ref, _ = sample_group([gal, sky], Window.from_scale(s.nx, s.ny), PSF(s.psf.astype(np.float32).astype(np.float64)))
        assert_image_close(g, ref)


@pytest.mark.parametrize("shape,psf_w", [((3, 3), 5), ((5, 4), 11), ((1, 1), 3), ((17, 2), 7)])
def test_tiny_stamps_and_psf_larger_than_stamp(N, shape, psf_w):
    nx, ny = shape
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0x7F)
    psf = np.outer(np.hanning(psf_w + 2)[1:-1], np.hanning(psf_w + 2)[1:-1])
    psf /= psf.sum()
    b = N.StampBatch([(nx, ny)], [(psf_w, psf_w)], N.scale_geometry(1), opts)
    p = np.array([nx / 2 + 0.2, ny / 2 - 0.3, 0.6, 0.4, 1.5, 2.0, 1.0, 0.0])
    got = b.unpack(b.render(torch.tensor(p[None, :]), b.pack_psf([psf])))[0]
    comp = Component("sersic", {"center": p[:2], "q": p[2], "PA": p[3], "n": p[4], "Re": p[5], "Ie": p[6]}, psf_mode="full")
    ref = sample_component(comp, Window.from_scale(nx, ny), PSF(psf.astype(np.float32).astype(np.float64))).model
    assert_image_close(got, ref)


def test_masked_and_zero_weight_pixels(N):
    d = cases.load_lm("lm_64")
    size = d["spec"]["size"]
    mask = np.zeros((size, size), dtype=np.uint8)
    mask[10:20, 30:40] = 1
    data = d["data"].copy()
    data[mask.astype(bool)] = np.nan  # masked pixels are never read into the sums
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0x7F, has_sky=True)
    b = N.StampBatch([(size, size)], [(25, 25)], N.scale_geometry(1), opts)
    state, chi2, iters, status = b.lm_fit(
        b.pack([data]), b.pack([d["weight"]]), b.pack([mask], torch.uint8), b.pack_psf([d["psf"]]),
        torch.tensor(np.r_[d["init"], 0.0][None, :]), torch.tensor(d["rep0"][None, :]), N.make_lm_options())
    assert np.isfinite(chi2.item())
    prob = lm_case_problem(d)
    prob.Y = data
    prob.mask = mask.astype(bool)
    lm = LMOracle(prob, d["rep0"]).fit()
    assert abs(chi2.item() / lm.res_loss() - 1) <= 1e-4


def test_option_errors(N):
    from astrophot_gb300.errors import SpecificationConflict

    with pytest.raises(SpecificationConflict):
        N.make_options(sampling_mode="bogus")
    with pytest.raises(SpecificationConflict):
        N.make_options(integrate_mode="full")
    with pytest.raises(SpecificationConflict):  # the centre supersampling replaces the integration
        N.make_options(sampling_mode="midpoint_center", integrate_mode="threshold")
    with pytest.raises(RuntimeError):
        N.StampBatch([(10, 10)], [(4, 4)], N.scale_geometry(1), N.make_options(psf_mode="full"))


def test_profiler_outside_and_inside_capture(N):
    """Kernel timing works for plain calls (ap_render) and for captured LM rounds alike."""
    d = cases.load_render("sersic_psf_64")
    b, psf = batch_for_case(N, d)
    params = torch.tensor(full_params(d["spec"])[None, :])
    b.profile(True)
    b.render(params, psf)
    torch.cuda.synchronize()
    kt = b.kernel_times()
    b.profile(False)
    assert kt["conv"][1] >= 1 and kt["conv"][0] > 0


def test_autotuned_grid_gives_identical_renders(N):
    """The render-pass autotuner changes only persistent-grid sizes: the renders, Jacobians and
    LM results stay bit for bit the same (every reduction has a fixed order)."""
    from astrophot_gb300 import synthetic

    specs = synthetic.cutout_stamps(12, seed=5, lo=24, hi=96)
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0x7F, has_sky=True)
    b = N.StampBatch([(s.nx, s.ny) for s in specs], [(s.psf.shape[1], s.psf.shape[0]) for s in specs],
                     N.scale_geometry(len(specs)), opts)
    psf = b.pack_psf([s.psf for s in specs])
    params = torch.tensor(np.array([np.r_[s.init, 0.0] for s in specs]))
    m0, j0 = b.jacobian(params, psf)
    m0, j0 = m0.clone(), j0.clone()
    res = b.autotune(params, psf, jacobian=True)
    assert set(res["blocks_per_sm"]) == {"sample", "integrate", "conv", "psf"}
    assert all(1 <= v <= 64 for v in res["blocks_per_sm"].values()) and res["render_pass_ms"] > 0
    m1, j1 = b.jacobian(params, psf)
    assert torch.equal(m0, m1) and torch.equal(j0, j1)
    b.set_grid({"sample": 3, "integrate": 2, "conv": 5, "psf": 1})
    m2, j2 = b.jacobian(params, psf)
    assert torch.equal(m0, m2) and torch.equal(j0, j2)


LM_VARIANTS = {
    # profile, psf, sampling, free sky, mask
    "exponential_no_psf": ("exponential", False, "midpoint", False, False),
    "sersic_simpsons_psf": ("sersic", True, "simpsons", False, False),
    "sersic_free_sky_mask": ("sersic", True, "midpoint", True, True),
    "exponential_psf_trapezoid": ("exponential", True, "trapezoid", False, False),
}


@pytest.mark.parametrize("name", sorted(LM_VARIANTS))
def test_lm_variants_match_oracle(N, name):
    """Batched LM with other options (profile, PSF, sampling mode, free sky, masked pixels):
    final chi2/ndf against the float64 oracle LM from the same data and initial vector."""
    from astrophot_gb300 import synthetic
    from astrophot_gb300.transforms import slots_to_rep

    kind, with_psf, sampling, free_sky, with_mask = LM_VARIANTS[name]
    size = 48
    rng = np.random.default_rng(sum(map(ord, name)))
    truth = synthetic.draw_sersic(rng, size, size)
    truth[5] = min(truth[5], 9.0)
    if kind == "exponential":
        truth[4] = 1.0
    init = synthetic.perturb_sersic(rng, truth)
    if kind == "exponential":
        init[4] = 1.0
    F_true, F_init = (0.2, 0.15) if free_sky else (0.0, 0.0)
    psf = synthetic.moffat_stamp(3.5, synthetic.moffat_rd(3.0, 3.5), 15) if with_psf else None
    slots = [0, 1, 2, 3, 4, 5, 6] if kind == "sersic" else [0, 1, 2, 3, 5, 6]
    if free_sky:
        slots.append(7)
    fmask = sum(1 << s for s in slots)
    opts = N.make_options(profile=kind, psf_mode="full" if with_psf else "none", sampling_mode=sampling,
                          free_mask=fmask, has_sky=True)
    b = N.StampBatch([(size, size)], [(15, 15)] if with_psf else None, N.scale_geometry(1), opts)
    psf_d = b.pack_psf([psf]) if with_psf else None
    t8 = np.r_[truth, F_true]
    model = b.unpack(b.render(torch.tensor(t8[None, :]), psf_d))[0].astype(np.float64)
    data, weight = synthetic.add_noise(model, 11)
    mask = np.zeros((size, size), dtype=np.uint8)
    if with_mask:
        mask[5:14, 20:31] = 1
        mask[::6, ::5] = 1
    i8 = np.r_[init, F_init]
    state, chi2, iters, status = b.lm_fit(
        b.pack([data]), b.pack([weight]), b.pack([mask], torch.uint8) if with_mask else None, psf_d,
        torch.tensor(i8[None, :]), torch.tensor(slots_to_rep(i8[None, :], fmask)), N.make_lm_options())
    p = {"center": [init[0], init[1]], "q": init[2], "PA": init[3], "Re": init[5], "Ie": init[6]}
    if kind == "sersic":
        p["n"] = init[4]
    gal = Component(kind, p, psf_mode="full" if with_psf else "none", sampling_mode=sampling)
    sky = Component("flat_sky", {"F": F_init}, locked=() if free_sky else ("F",))
    psf32 = None if psf is None else PSF(psf.astype(np.float32).astype(np.float64))
    prob = GroupProblem([gal, sky], Window.from_scale(size, size), psf32,
                        data.astype(np.float32).astype(np.float64), weight.astype(np.float32).astype(np.float64),
                        mask.astype(bool) if with_mask else None)
    lm = LMOracle(prob, prob.representation()).fit()
    print(name, chi2.item(), lm.res_loss(), iters.item(), lm.iterations, N.LM_MESSAGES[status.item()], lm.message)
    assert abs(chi2.item() / lm.res_loss() - 1) <= 1e-4


def test_values_to_rep_matches_host_transforms(N):
    from astrophot_gb300.transforms import slots_to_rep
    from astrophot_gb300 import synthetic

    rng = np.random.default_rng(12)
    rows = np.array([np.r_[synthetic.draw_sersic(rng, 64, 64), 0.1] for _ in range(50)])
    rows[:, 3] += np.pi * rng.integers(-2, 3, 50)  # PA outside [0, pi): the cyclic map wraps it
    for mask in (0x7F, 0xFF, 0x6F):
        got = N.values_to_rep(torch.tensor(rows, device="cuda"), mask).cpu().numpy()
        want = slots_to_rep(rows, mask)
        assert np.allclose(got, want, rtol=1e-12, atol=1e-12)
