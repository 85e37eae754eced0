"""Host-side checks that need no GPU: the C-ABI library loads and exports every entry point
declared in include/astrophot_gb300.h; the host-only planning calls validate their inputs;
the product's parameter transforms agree with the oracle's."""

import ctypes
import os
import re

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "include", "astrophot_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ap_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def N():
    from astrophot_gb300 import _native

    if not os.path.exists(_native.LIB_PATH):
        from astrophot_gb300 import _build

        _build.build()
    return _native


def test_library_exports_every_declared_symbol(N):
    lib = ctypes.CDLL(N.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 15
    for name in syms:
        assert hasattr(lib, name), name
    # and the Python binding declares argtypes for each
    bound = {name for name, _ in N.EXPORTS}
    assert set(syms) <= bound, set(syms) - bound
    assert N.lib().ap_version().decode().startswith("astrophot_gb300")


def _create(N, shapes, psf_shapes, opts):
    n = len(shapes)
    nx = (ctypes.c_int32 * n)(*[s[0] for s in shapes])
    ny = (ctypes.c_int32 * n)(*[s[1] for s in shapes])
    kx = (ctypes.c_int32 * n)(*[s[0] for s in psf_shapes]) if psf_shapes else None
    ky = (ctypes.c_int32 * n)(*[s[1] for s in psf_shapes]) if psf_shapes else None
    g = np.ascontiguousarray(N.scale_geometry(n))
    h = ctypes.c_void_p()
    rc = N.lib().ap_batch_create(ctypes.byref(h), n, nx, ny, kx, ky, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(opts))
    return rc, h


def test_batch_plan_sizes_and_offsets(N):
    opts = N.make_options(psf_mode="full", has_sky=True)
    shapes = [(32, 40), (100, 77), (5, 5)]
    psfs = [(9, 9), (21, 15), (3, 3)]
    rc, h = _create(N, shapes, psfs, opts)
    assert rc == N.AP_OK
    L = N.lib()
    out_px, psf_px, ws = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    assert L.ap_batch_sizes(h, ctypes.byref(out_px), ctypes.byref(psf_px), ctypes.byref(ws)) == 0
    assert out_px.value == sum(a * b for a, b in shapes)
    assert psf_px.value == sum(a * b for a, b in psfs)
    assert ws.value > 0 and ws.value % 256 == 0
    oo, po = (ctypes.c_int64 * 3)(), (ctypes.c_int64 * 3)()
    assert L.ap_batch_offsets(h, oo, po) == 0
    assert list(oo) == [0, 32 * 40, 32 * 40 + 100 * 77]
    assert list(po) == [0, 81, 81 + 21 * 15]
    lmws = ctypes.c_int64()
    assert L.ap_lm_workspace_bytes(h, ctypes.byref(N.make_lm_options()), ctypes.byref(lmws)) == 0
    assert lmws.value > out_px.value * 4 * 8
    # a render before binding a workspace is refused, not attempted
    assert L.ap_render(h, None, None, None, None) == N.AP_ERR_ARG
    L.ap_batch_destroy(h)


@pytest.mark.parametrize(
    "shapes,psfs,kw,code",
    [
        ([(10, 10)], [(4, 5)], {"psf_mode": "full"}, 1),            # even PSF
        ([(0, 10)], None, {}, 1),                                  # empty stamp
        ([(10, 10)], None, {"integrate_max_depth": 4}, 2),         # deeper than supported
        ([(10, 10)], None, {"integrate_gridding": 6}, 2),
        ([(10, 10)], None, {"profile": "exponential", "free_mask": 0x7F}, 1),  # n is not fitted
        ([(10, 10)], None, {"free_mask": 0xFF}, 1),                # F fitted without a sky
        ([(2, 2)], None, {}, 1),                                   # curvature stencil needs 3x3
    ],
)
def test_batch_create_rejects_bad_input(N, shapes, psfs, kw, code):
    rc, h = _create(N, shapes, psfs, N.make_options(**kw))
    assert rc == code
    assert not h.value


def test_midpoint_center_options(N):
    """The centre-supersampling mode: planned with integrate_mode none, refused with the
    threshold integration (which it replaces) and with a negative radius."""
    opts = N.make_options(sampling_mode="midpoint_center", integrate_mode="none", psf_mode="full")
    rc, h = _create(N, [(64, 64)], [(25, 25)], opts)
    assert rc == 0
    N.lib().ap_batch_destroy(h)
    opts.integrate_mode = 1  # threshold
    assert _create(N, [(64, 64)], [(25, 25)], opts)[0] == N.AP_ERR_UNSUPPORTED
    opts = N.make_options(sampling_mode="midpoint_center", integrate_mode="none", center_radius=-1.0)
    assert _create(N, [(64, 64)], None, opts)[0] == N.AP_ERR_ARG


def test_sampling_modes_without_curvature_accept_tiny_windows(N):
    rc, h = _create(N, [(1, 1)], None, N.make_options(sampling_mode="quad:3"))
    assert rc == 0
    N.lib().ap_batch_destroy(h)


def test_transforms_match_oracle():
    from astrophot_gb300.transforms import rep_to_slots, slots_to_rep
    from oracle.render import rep_to_value, value_to_rep

    rng = np.random.default_rng(1)
    vals = np.stack(
        [rng.uniform(0, 100, 20), rng.uniform(0, 100, 20), rng.uniform(0.01, 0.99, 20), rng.uniform(0, np.pi, 20),
         rng.uniform(0.4, 7.9, 20), rng.uniform(0.1, 50, 20), rng.uniform(-1, 3, 20), rng.uniform(-1, 1, 20)], 1)
    rep = slots_to_rep(vals, 0xFF)
    names = ["center", "center", "q", "PA", "n", "Re", "Ie", "F"]
    for k, nm in enumerate(names):
        assert np.allclose(rep[:, k], value_to_rep(nm, vals[:, k]), rtol=1e-13, atol=1e-13)
    back = rep_to_slots(rep, vals * 0, 0xFF)
    assert np.allclose(back, vals, rtol=1e-12, atol=1e-12)


def test_synthetic_workload_is_seeded_and_in_range():
    from astrophot_gb300 import synthetic

    a = synthetic.cutout_stamps(50, seed=4)
    b = synthetic.cutout_stamps(50, seed=4)
    assert all(np.array_equal(x.truth, y.truth) and x.nx == y.nx for x, y in zip(a, b))
    for s in a:
        assert 32 <= s.nx <= 256 and s.nx == s.ny
        assert s.psf.shape[0] % 2 == 1 and 9 <= s.psf.shape[0] <= 21
        cx, cy, q, PA, n, Re, Ie = s.truth
        assert 0.3 <= q < 1 and 0.5 <= n <= 4 and 5 <= Re <= 20 and 0 <= PA < np.pi and 0 <= Ie <= 2
        assert abs(s.psf.sum() - 1) < 1e-12


def test_lanczos_shift_options(N):
    """psf_subpixel_shift "lanczos:k": parsed into ap_options.lanczos_order with the full PSF mode,
    planned by ap_batch_create; orders outside 1..8, or a Lanczos order without the shifted
    PSF mode, are refused."""
    from astrophot_gb300.errors import SpecificationConflict

    o = N.make_options(psf_mode="full", psf_subpixel_shift="lanczos:3")
    assert o.lanczos_order == 3 and o.psf_mode == N.PSF_FULL
    assert N.make_options(psf_mode="full").lanczos_order == 0
    rc, h = _create(N, [(32, 32)], [(9, 9)], o)
    assert rc == N.AP_OK
    N.lib().ap_batch_destroy(h)
    for bad in ("lanczos:9", "lanczos:0", "lanczos:x"):
        with pytest.raises(SpecificationConflict):
            N.make_options(psf_mode="full", psf_subpixel_shift=bad)
    o = N.make_options(psf_mode="full", psf_subpixel_shift="none")
    o.lanczos_order = 3
    rc, h = _create(N, [(32, 32)], [(9, 9)], o)
    assert rc == N.AP_ERR_UNSUPPORTED and not h.value
