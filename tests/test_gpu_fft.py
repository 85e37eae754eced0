"""PSF convolution by FFT (``fft_min_kernel``): against the reference's golden renders (which
the reference itself convolved by FFT) and against the direct convolution of the same batch,
for the model, the Jacobian, the adjoint and the batched LM."""

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


def close(got, ref, rel=1e-5, bright_rel=1e-4):
    """within rel of the image maximum everywhere, and within bright_rel pixel by pixel where
    the image is above 1 % of its maximum (FP32 FFT error is relative to the maximum)"""
    scale = np.max(np.abs(ref))
    err = np.max(np.abs(got - ref)) / scale
    bright = np.abs(ref) > 1e-2 * scale
    prel = np.max(np.abs(got - ref)[bright] / np.abs(ref)[bright])
    return err <= rel and prel <= bright_rel, (err, prel)


def params_of(spec):
    p = spec["params"]
    return np.array([p["center"][0], p["center"][1], p["q"], p["PA"], p.get("n", 1.0), p["Re"], p["Ie"], 0.0])


PSF_CASES = [n for n in cases.render_case_names() if cases.load_render(n)["psf"].size]


@pytest.mark.parametrize("name", PSF_CASES)
def test_fft_convolution_matches_reference_goldens(N, name):
    """Every stamp convolved by FFT (threshold 1): the reference's model and Jacobian."""
    d = cases.load_render(name)
    spec = d["spec"]
    kind = spec["kind"]
    opts = N.make_options(profile=kind, sampling_mode=spec["knobs"].get("sampling_mode", "midpoint"),
                          integrate_mode=spec["knobs"].get("integrate_mode", "threshold"), psf_mode="full",
                          psf_subpixel_shift=spec["knobs"].get("psf_subpixel_shift", "bilinear"),
                          free_mask=0x7F if kind == "sersic" else 0x6F, fft_min_kernel=1)
    psf = d["psf"]
    b = N.StampBatch([(spec["nx"], spec["ny"])], [(psf.shape[1], psf.shape[0])], N.scale_geometry(1, spec["scale"]), opts)
    kp = b.pack_psf([psf])
    params = torch.tensor(params_of(spec)[None, :])
    model = b.unpack(b.render(params, kp))[0]
    ok, err = close(model, d["model"])
    assert ok, err
    _, jac = b.jacobian(params, kp, as_representation=True)
    J = jac.cpu().numpy().reshape(b.n_free, spec["ny"], spec["nx"])
    for k in range(b.n_free):
        ref = d["jac_rep"][..., k]
        assert np.max(np.abs(J[k] - ref)) <= 2e-4 * np.max(np.abs(ref)), (k, np.max(np.abs(J[k] - ref)) / np.max(np.abs(ref)))


def _large_psf_batch(N, fft, kinds=("sersic",)):
    from astrophot_gb300 import synthetic

    shapes = [(128, 96), (80, 112), (150, 150)]
    psfs = [synthetic.gaussian_stamp(2.0, 51, 1.0), synthetic.moffat_stamp(3.5, synthetic.moffat_rd(4.0, 3.5), 65, 1.0),
            synthetic.moffat_stamp(3.5, synthetic.moffat_rd(3.0, 3.5), 41, 1.0)]
    opts = N.make_options(profile=kinds[0], psf_mode="full", free_mask=0x7F if kinds[0] == "sersic" else 0x6F,
                          has_sky=True, fft_min_kernel=1 if fft else 0)
    b = N.StampBatch(shapes, [p.shape[::-1] for p in psfs], N.scale_geometry(len(shapes)), opts)
    params = np.array([[64.3, 47.6, 0.6, 0.8, 2.2, 14.0, 0.9, 0.0],
                       [40.1, 57.2, 0.45, 2.1, 1.3, 9.0, 1.2, 0.0],
                       [75.4, 74.8, 0.8, 1.4, 3.5, 22.0, 0.5, 0.0]])
    return b, b.pack_psf(psfs), torch.tensor(params), shapes


def test_fft_matches_direct_on_large_psfs(N):
    """51², 65² and 41² PSFs on uneven stamps: FFT against direct convolution."""
    bd, kd, params, shapes = _large_psf_batch(N, fft=False)
    bf, kf, _, _ = _large_psf_batch(N, fft=True)
    md, jd = bd.jacobian(params, kd, as_representation=True)
    mf, jf = bf.jacobian(params, kf, as_representation=True)
    for a, c in zip(bd.unpack(md), bf.unpack(mf)):
        ok, err = close(c, a)  # measured 3.8e-6 of the maximum, 6e-6 per bright pixel
        assert ok, err
    Jd, Jf = jd.cpu().numpy(), jf.cpu().numpy()
    for k in range(bd.n_free):
        for s, (nx, ny) in enumerate(shapes):
            o = bd.out_offsets[s]
            a, c = Jd[k, o : o + nx * ny], Jf[k, o : o + nx * ny]
            assert np.max(np.abs(a - c)) <= 1e-4 * np.max(np.abs(a)), (k, s)
    # the adjoint of the render through the FFT path
    g = torch.randn(bd.out_pixels, generator=torch.Generator().manual_seed(3)).float().cuda()
    vd = bd.vjp(params, kd, g).cpu().numpy()
    vf = bf.vjp(params, kf, g).cpu().numpy()
    assert np.max(np.abs(vd - vf) / np.maximum(np.abs(vd), 1e-3 * np.max(np.abs(vd)))) <= 1e-3


def test_fft_lm_matches_direct(N):
    """The batched LM on the three large-PSF stamps ends at the same chi^2 either way."""
    bd, kd, truth, shapes = _large_psf_batch(N, fft=False)
    bf, kf, _, _ = _large_psf_batch(N, fft=True)
    model = bd.render(truth, kd)
    rng = np.random.default_rng(11)
    sig = 0.05
    data = (model + torch.tensor(rng.normal(size=model.numel()) * sig, dtype=torch.float32, device=model.device))
    weight = torch.full_like(data, 1.0 / sig**2)
    init = truth.clone()
    init[:, 0] += 0.4
    init[:, 5] *= 1.1
    init[:, 4] *= 0.9
    rep = N.values_to_rep(init.cuda(), 0x7F)
    lmo = N.make_lm_options()
    sd, cd, itd, std = bd.lm_fit(data, weight, None, kd, init, rep, lmo)
    sf, cf, itf, stf = bf.lm_fit(data, weight, None, kf, init, rep, lmo)
    cd, cf = cd.cpu().numpy(), cf.cpu().numpy()
    assert np.all(np.abs(cf / cd - 1) <= 1e-5), (cd, cf)
    assert np.allclose(sf.cpu().numpy(), sd.cpu().numpy(), rtol=1e-3, atol=1e-3)
