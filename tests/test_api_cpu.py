"""Host-side behaviour of the drop-in API, restating the reference's own tests where they
pin it (tests/test_parameter.py:287-420 vector masks and representation, tests/test_model.py
:49-115 round trip and bad modes, tests/test_window.py window arithmetic).  No GPU needed:
building models and parameters never touches the device."""

import math

import numpy as np
import pytest
import torch

import astrophot_gb300 as ap
from astrophot_gb300.errors import InvalidParameter, NameNotAllowed, SpecificationConflict, UnrecognizedModel
from astrophot_gb300.param import Param_Mask, Param_SoftLimits, Param_Unlock, Parameter_Node


def test_parameter_vector_api_and_masks():
    P = Parameter_Node("group")
    a = Parameter_Node("a", value=[1.0, 2.0])
    b = Parameter_Node("b", value=0.5, limits=(0, 1))
    c = Parameter_Node("c", value=3.0, locked=True)
    d = Parameter_Node("d", value=1.0, limits=(0, math.pi), cyclic=True)
    P.link(a, b, c, d)
    assert P.vector_values().tolist() == [1.0, 2.0, 0.5, 1.0]  # locked c left out
    rep = P.vector_representation()
    assert rep[2].item() == pytest.approx(0.0, abs=1e-15)  # tan(0.5 pi - pi/2)
    P.vector_set_representation(rep)
    assert np.allclose(P.vector_values().numpy(), [1.0, 2.0, 0.5, 1.0])
    with Param_Mask(P, torch.tensor([True, False, True, False])):
        assert P.vector_values().tolist() == [1.0, 0.5]
        P.vector_set_values([7.0, 0.25])
    assert P.vector_values().tolist() == [7.0, 2.0, 0.25, 1.0]
    assert len(P.vector_identities()) == 4


def test_limits_raise_and_soft_limits_push_inside():
    q = Parameter_Node("q", value=0.5, limits=(0, 1))
    with pytest.raises(InvalidParameter):
        q.value = 1.0
    with Param_SoftLimits(q):
        q.value = 2.0
    assert q.value.item() == pytest.approx(0.999)
    pa = Parameter_Node("PA", value=0.1, limits=(0, math.pi), cyclic=True)
    pa.value = -0.1
    assert pa.value.item() == pytest.approx(math.pi - 0.1)


def test_locked_parameters_ignore_writes_unless_unlocked():
    p = Parameter_Node("F", value=1.0, locked=True)
    p.value = 2.0
    assert p.value.item() == 1.0
    with Param_Unlock(p):
        p.value = 2.0
    assert p.value.item() == 2.0 and p.locked


def test_model_factory_specs_and_representation_round_trip():
    tar = ap.image.Target_Image(data=np.zeros((30, 40)), pixelscale=0.8)
    m = ap.models.AstroPhot_Model(name="rt", model_type="sersic galaxy model", target=tar,
                                  parameters={"center": [10.0, 12.0], "q": 0.6, "PA": 2.0, "n": 3.0, "Re": 4.0, "Ie": 0.3})
    assert isinstance(m, ap.models.Sersic_Galaxy)
    assert m.parameters["q"].limits == (0.0, 1.0) and m.parameters["PA"].cyclic
    assert m.parameters["n"].limits == (0.36, 8.0) and m.parameters["Re"].limits == (0.0, None)
    v = m.parameters.vector_values().clone()
    m.parameters.vector_set_representation(m.parameters.vector_representation())
    assert torch.allclose(m.parameters.vector_values(), v, rtol=1e-12, atol=1e-12)
    e = ap.models.AstroPhot_Model(name="rt e", model_type="exponential galaxy model", target=tar,
                                  parameters={"center": [1.0, 2.0], "q": 0.6, "PA": 2.0, "Re": 4.0, "Ie": 0.3})
    assert list(e.parameters.vector_names()) == ["center:0", "center:1", "q", "PA", "Re", "Ie"]
    with pytest.raises(UnrecognizedModel):
        ap.models.AstroPhot_Model(name="x", model_type="spline galaxy model", target=tar)
    with pytest.raises(NameNotAllowed):
        ap.models.AstroPhot_Model(name="a:b", model_type="flat sky model", target=tar)


def test_group_pushes_psf_mode_and_sky_center_is_locked():
    tar = ap.image.Target_Image(data=np.zeros((30, 40)), pixelscale=1.0, psf=np.ones((5, 5)) / 25)
    g1 = ap.models.AstroPhot_Model(name="gp gal", model_type="sersic galaxy model", target=tar, psf_mode="full",
                                   parameters={"center": [10.0, 12.0], "q": 0.6, "PA": 2.0, "n": 3.0, "Re": 4.0, "Ie": 0.3})
    sky = ap.models.AstroPhot_Model(name="gp sky", model_type="flat sky model", target=tar, parameters={"F": 0.1})
    sky.initialize()
    grp = ap.models.AstroPhot_Model(name="gp", model_type="group model", target=tar, models=[g1, sky])
    assert g1.psf_mode == "none"  # the group's default psf_mode is pushed onto its models
    assert sky.parameters["center"].locked
    assert list(grp.parameters.vector_names()) == ["center:0", "center:1", "q", "PA", "n", "Re", "Ie", "F"]
    grp.psf_mode = "full"
    assert g1.psf_mode == "full" and sky.psf_mode == "none"


def test_windows_intersect_union_and_indices():
    tar = ap.image.Target_Image(data=np.arange(30 * 40, dtype=float).reshape(30, 40), pixelscale=1.0)
    w = tar.window.copy().crop_to_pixel([[5, 25], [3, 18]])
    assert list(w.pixel_shape) == [20, 15]
    sub = tar[w]
    assert torch.equal(sub.data, tar.data[3:18, 5:25])
    w2 = tar.window.copy().crop_to_pixel([[20, 35], [10, 29]])
    inter = w & w2
    assert list(inter.pixel_shape) == [5, 8]
    uni = w | w2
    assert list(uni.pixel_shape) == [30, 26]
    rows, cols = tar.window.get_self_indices(inter)
    assert (rows.start, rows.stop, cols.start, cols.stop) == (10, 18, 20, 25)


def test_psf_must_be_odd():
    with pytest.raises(SpecificationConflict):
        ap.image.PSF_Image(np.ones((4, 5)))
    tar = ap.image.Target_Image(data=np.zeros((10, 10)), psf=np.ones((5, 7)) / 35)
    assert list(tar.psf.psf_border_int) == [4, 3]


def test_target_weight_variance_and_nan_mask():
    data = np.ones((6, 6))
    data[2, 3] = np.nan
    tar = ap.image.Target_Image(data=data, variance=np.full((6, 6), 4.0))
    assert torch.allclose(tar.weight, torch.full((6, 6), 0.25, dtype=torch.float64))
    assert tar.has_mask and bool(tar.mask[2, 3]) and int(tar.mask.sum()) == 1
