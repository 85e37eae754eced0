"""The adjoint of a full-size bulge + disk field on the GPU: 500 Sersic bulge + exponential disk
pairs sharing their centres on a 2048 x 2048 image with a 65 x 65 Moffat PSF (the adjoint
configuration at its stated size; the PSF-convolved tiles are recomputed inside the adjoint,
never stored).  The scene's gradient of the chi^2 (its VJP with the upstream weighted residual)
is checked for three of the pairs against the oracle's Jacobian of those pairs contracted with
the same residual image, and against the scene's own Jacobian transpose for all parameters."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def field():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from astrophot_gb300 import scene as SC
    from astrophot_gb300 import synthetic

    truth, init, windows, psf = synthetic.bulge_disk_field(5)
    size = 2048
    zeros = np.zeros((size, size))
    sc_t = SC.Scene(size, size, synthetic.bulge_disk_sources(truth, windows), psf, zeros, zeros + 1, sky=1.0)
    model = sc_t.forward(sc_t.representation()).cpu().numpy().astype(np.float64).reshape(size, size)
    del sc_t
    data, weight = synthetic.add_noise(model, 5)
    sc = SC.Scene(size, size, synthetic.bulge_disk_sources(init, windows), psf, data, weight, sky=1.0)
    return sc, init, windows, psf


def test_full_field_adjoint_matches_oracle_jacobian(field):
    from oracle.render import PSF, Component, Window, drep_dvalue, sample_component, sub_window, value_to_rep

    sc, init, windows, psf = field
    assert sc.P == 500 * 11
    rep = sc.representation()
    model = sc.forward(rep)
    g = (sc.weight.double() * (model.double() - sc.data.double())).float()
    vjp = sc.vjp(rep, g).numpy()
    gimg = g.cpu().numpy().astype(np.float64).reshape(2048, 2048)
    win = Window.from_scale(2048, 2048)
    names = {0: ("center", 0), 1: ("center", 1), 2: ("q", 0), 3: ("PA", 0), 4: ("n", 0), 5: ("Re", 0), 6: ("Ie", 0)}
    checked = []
    for k in (0, 250, 499):
        cx, cy, bq, bpa, bn, bre, bie, dq, dpa, dre, die = init[k]
        (x0, x1), (y0, y1) = windows[k]
        sw = sub_window(win, windows[k])
        gw = gimg[y0:y1, x0:x1]
        bulge = Component("sersic", {"center": [cx, cy], "q": bq, "PA": bpa, "n": bn, "Re": bre, "Ie": bie},
                          psf_mode="full", window=windows[k])
        disk = Component("exponential", {"center": [cx, cy], "q": dq, "PA": dpa, "Re": dre, "Ie": die},
                         psf_mode="full", window=windows[k])
        for si, comp in ((2 * k, bulge), (2 * k + 1, disk)):
            jac = sample_component(comp, sw, PSF(psf), grad=True).jac
            for slot, j in sc.gidx[si].items():
                name = names[slot]
                val = np.atleast_1d(comp.params[name[0]])[name[1]]
                r = value_to_rep(name[0], val, comp.kind)
                grad = np.sum(jac[name] * gw) * drep_dvalue(name[0], r, comp.kind)
                checked.append((j, grad))
    want = {}
    for j, v in checked:  # the shared centre sums its bulge and disk columns
        want[j] = want.get(j, 0.0) + v
    idx = np.array(sorted(want))
    ref = np.array([want[j] for j in idx])
    scale = np.max(np.abs(ref))
    err = np.max(np.abs(vjp[idx] - ref)) / scale
    print("full-field adjoint vs oracle Jacobian^T g on three pairs:", err)
    assert err <= 1e-4


def test_full_field_adjoint_is_jacobian_transpose(field):
    sc, _, _, _ = field
    rep = sc.representation()
    model = sc.forward(rep)
    g = (sc.weight.double() * (model.double() - sc.data.double())).float()
    vjp = sc.vjp(rep, g).numpy()
    sc.jacobian(rep)
    jt = sc.jt(g.contiguous()).cpu().numpy()
    scale = np.max(np.abs(jt))
    assert np.max(np.abs(vjp - jt)) <= 1e-4 * scale
