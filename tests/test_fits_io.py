"""FITS image I/O (``fits_io``) and ``Target_Image.save`` / ``load`` with the reference's HDU
layout (image/image_object.py:400-428, image/target_image.py:503-532)."""

import numpy as np
import pytest

from astrophot_gb300 import fits_io


@pytest.mark.parametrize("dtype", [np.float64, np.float32, np.int64, np.int32, np.int16, np.uint8])
def test_fits_round_trip(tmp_path, dtype):
    rng = np.random.default_rng(0)
    a = (rng.normal(size=(7, 11)) * 100).astype(dtype)
    b = np.arange(15, dtype=np.float64).reshape(5, 3)
    long = "[" + ", ".join(str(v) for v in rng.normal(size=20)) + "]"  # needs CONTINUE cards
    f = str(tmp_path / "x.fits")
    fits_io.write_hdus(f, [(a, {"IMAGE": "PRIMARY", "PXLSCALE": "[[1.0, 0.0], [0.0, 1.0]]", "LONGSTR": long,
                                "QUOTE": "it's", "FLAG": True, "NUM": 2.5}), (b, {"IMAGE": "WEIGHT"})])
    raw = open(f, "rb").read()
    assert len(raw) % 2880 == 0
    assert raw[:30] == b"SIMPLE  =                    T"
    out = fits_io.read_hdus(f)
    assert len(out) == 2
    (da, ha), (db, hb) = out
    assert da.dtype == np.dtype(dtype) and np.array_equal(da, a)
    assert np.array_equal(db, b)
    assert ha["IMAGE"] == "PRIMARY" and ha["LONGSTR"] == long and ha["QUOTE"] == "it's"
    assert ha["FLAG"] is True and ha["NUM"] == 2.5 and ha["NAXIS1"] == 11 and ha["NAXIS2"] == 7
    assert hb["XTENSION"] == "IMAGE" and hb["IMAGE"] == "WEIGHT"


def test_target_image_save_load(tmp_path):
    import astrophot_gb300 as ap

    rng = np.random.default_rng(1)
    data = rng.normal(size=(20, 30))
    var = rng.uniform(0.5, 2.0, size=data.shape)
    mask = np.zeros(data.shape, bool)
    mask[3, 4] = True
    psf = ap.utils.initialize.moffat_psf(3.5, 2.0, 11, 0.8)
    tar = ap.image.Target_Image(data=data, pixelscale=0.8, psf=psf, variance=var, mask=mask, zeropoint=22.5,
                                origin=(3.0, -2.0))
    f = str(tmp_path / "t.fits")
    tar.save(f)
    back = ap.image.Target_Image(filename=f)
    assert np.allclose(back.data.numpy(), data)
    assert np.allclose(back.weight.numpy(), 1 / var)
    assert np.allclose(back.window.pixelscale, tar.window.pixelscale)
    assert np.allclose(back.window.reference_imagexy, tar.window.reference_imagexy)
    assert np.array_equal(back.window.pixel_shape, tar.window.pixel_shape)
    assert back.zeropoint == 22.5
    assert np.allclose(back.psf.data.numpy(), psf)
    # the reference writes the mask as "MASK" and looks for "mask" when loading: it does not come back
    assert not back.has_mask
    kinds = [h["IMAGE"] for _, h in fits_io.read_hdus(f)]
    assert kinds == ["PRIMARY", "WEIGHT", "MASK", "PSF"]
