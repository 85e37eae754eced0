"""ap_render_noalloc: the render entry point for callers that cannot allocate device memory.

Such callers (a host that reserves all device memory for its own pool, a plugin without
access to that pool's allocator, a pipeline that must not stall on an allocation) pass only
their inputs and outputs; the entry point's scratch is a fixed array inside the library.
These tests call it through the C ABI and compare its images with the regular batch entry
point ap_render and with the reference's golden images, within the same tolerance as the other
image tests, on two calls in a row (the second call must not see stale state from the first),
including a large stamp followed by a small one."""

import ctypes

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


def assert_image_close(got, ref, rel=1e-5, pix=1e-5):
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) <= rel * scale, np.max(np.abs(got - ref)) / scale
    bright = np.abs(ref) > 1e-3 * scale
    r = (np.abs(got - ref)[bright] / np.abs(ref)[bright]).max()
    assert r <= pix, r


def noalloc_render(N, nx, ny, psf, psf_shape, geometry, opts, params):
    assert params.dtype == torch.float64 and params.is_contiguous()  # the C ABI reads double[8]
    model = torch.full((ny * nx,), float("nan"), dtype=torch.float32, device="cuda")
    g = np.ascontiguousarray(geometry, dtype=np.float64)
    kx, ky = psf_shape
    rc = N.lib().ap_render_noalloc(
        nx, ny, kx, ky, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(opts),
        ctypes.c_void_p(params.data_ptr()),
        ctypes.c_void_p(psf.data_ptr()) if psf is not None else None,
        ctypes.c_void_p(model.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.AP_OK, rc
    torch.cuda.synchronize()
    return model.cpu().numpy().reshape(ny, nx)


@pytest.mark.parametrize("name", ["sersic_psf_64", "sersic_psf_n4", "sersic_nopsf", "exp_psf",
                                  "sersic_nopsf_simpsons", "sersic_nopsf_quad3"])
def test_noalloc_matches_batch_render_twice(N, name):
    d = cases.load_render(name)
    spec = d["spec"]
    knobs = spec["knobs"]
    opts = N.make_options(profile=spec["kind"], sampling_mode=knobs.get("sampling_mode", "midpoint"),
                          psf_mode=knobs.get("psf_mode", "none"),
                          free_mask=0x7F if spec["kind"] == "sersic" else 0x6F)
    psf_np = d["psf"] if d["psf"].size else None
    geom = N.scale_geometry(1, spec["scale"])
    batch = N.StampBatch([(spec["nx"], spec["ny"])], [(psf_np.shape[1], psf_np.shape[0])] if psf_np is not None else None,
                         geom, opts)
    psf = batch.pack_psf([psf_np]) if psf_np is not None else None
    p = spec["params"]
    base = np.array([p["center"][0], p["center"][1], p["q"], p["PA"], p.get("n", 1.0), p["Re"], p["Ie"], 0.0])
    second = base.copy()
    second[0] += 1.37
    second[1] -= 0.61
    second[5] *= 0.8
    for k, vals in enumerate((base, second)):
        params = torch.tensor(vals[None, :], device="cuda")
        want = batch.unpack(batch.render(params, psf))[0]
        kshape = (psf_np.shape[1], psf_np.shape[0]) if psf_np is not None else (0, 0)
        got = noalloc_render(N, spec["nx"], spec["ny"], psf, kshape, geom[0], opts, params[0].contiguous())
        assert_image_close(got, want)
        if k == 0:
            # its own level-1 path (float64 split decisions inline) against the reference's image
            assert_image_close(got, d["model"])


def test_noalloc_small_stamp_after_a_large_one(N):
    """A 256 x 256 stamp, then a 40 x 48 one: the second image must equal the batch render (the
    shared scratch keeps the large stamp's contents)."""
    geom = N.scale_geometry(1)
    opts = N.make_options(psf_mode="full")
    big_psf = np.ones((21, 21)) / 441.0
    bb = N.StampBatch([(256, 256)], [(21, 21)], geom, opts)
    pb = bb.pack_psf([big_psf])
    params = torch.tensor([[128.3, 127.6, 0.5, 1.0, 2.0, 30.0, 1.0, 0.0]], dtype=torch.float64, device="cuda")
    noalloc_render(N, 256, 256, pb, (21, 21), geom[0], opts, params[0].contiguous())
    d = cases.load_render("sersic_psf_n4")
    spec = d["spec"]
    sb = N.StampBatch([(spec["nx"], spec["ny"])], [(d["psf"].shape[1], d["psf"].shape[0])], geom, opts)
    ps = sb.pack_psf([d["psf"]])
    p = spec["params"]
    small = torch.tensor([[p["center"][0], p["center"][1], p["q"], p["PA"], p["n"], p["Re"], p["Ie"], 0.0]],
                         dtype=torch.float64, device="cuda")
    want = sb.unpack(sb.render(small, ps))[0]
    got = noalloc_render(N, spec["nx"], spec["ny"], ps, (d["psf"].shape[1], d["psf"].shape[0]), geom[0], opts,
                         small[0].contiguous())
    assert_image_close(got, want)
    assert_image_close(got, d["model"])


def test_noalloc_rejects_oversized_sides(N):
    """Sides beyond the stated limits are refused before any arithmetic on them."""
    opts = N.make_options()
    params = torch.zeros(8, dtype=torch.float64, device="cuda")
    model = torch.zeros(4, dtype=torch.float32, device="cuda")
    g = np.ascontiguousarray(N.scale_geometry(1)[0])
    rc = N.lib().ap_render_noalloc(1 << 17, 2, 0, 0, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   ctypes.byref(opts), ctypes.c_void_p(params.data_ptr()), None,
                                   ctypes.c_void_p(model.data_ptr()),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.AP_ERR_ARG


def test_noalloc_rejects_windows_beyond_its_scratch(N):
    opts = N.make_options(psf_mode="full")
    psf = torch.ones(21 * 21, dtype=torch.float32, device="cuda") / 441
    params = torch.tensor([300.0, 300.0, 0.5, 1.0, 2.0, 10.0, 1.0, 0.0], dtype=torch.float64, device="cuda")
    model = torch.zeros(600 * 600, dtype=torch.float32, device="cuda")
    g = np.ascontiguousarray(N.scale_geometry(1)[0])
    rc = N.lib().ap_render_noalloc(600, 600, 21, 21, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                   ctypes.byref(opts), ctypes.c_void_p(params.data_ptr()),
                                   ctypes.c_void_p(psf.data_ptr()), ctypes.c_void_p(model.data_ptr()),
                                   ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == N.AP_ERR_WORKSPACE


def test_noalloc_handles_the_largest_cutout(N):
    """A 256 x 256 stamp with a 21 x 21 PSF (the largest of the cutout workload) fits."""
    opts = N.make_options(psf_mode="full")
    psf_np = np.ones((21, 21)) / 441.0
    geom = N.scale_geometry(1)
    batch = N.StampBatch([(256, 256)], [(21, 21)], geom, opts)
    psf = batch.pack_psf([psf_np])
    params = torch.tensor([[128.3, 127.6, 0.5, 1.0, 2.0, 12.0, 1.0, 0.0]], dtype=torch.float64, device="cuda")
    want = batch.unpack(batch.render(params, psf))[0]
    got = noalloc_render(N, 256, 256, psf, (21, 21), geom[0], opts, params[0].contiguous())
    assert_image_close(got, want)
