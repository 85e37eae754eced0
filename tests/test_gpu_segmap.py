"""Segmentation-map helpers on the GPU (``ap_segmap_*``, ``ap_window_flux``) against the
reference's own outputs in ``tests/golden/segmap_*.npz`` and against the oracle."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

import cases  # noqa: E402


@pytest.fixture(scope="module")
def SM():
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA GPU")
    from astrophot_gb300 import segmap

    return segmap


@pytest.mark.parametrize("name", cases.segmap_case_names())
def test_segmap_helpers_match_reference(SM, name, tmp_path):
    d = cases.load_segmap(name)
    seg, image = d["seg"], d["image"]
    ids = list(d["ids"])
    cen = SM.centroids_from_segmentation_map(seg, image)
    pas = SM.PA_from_segmentation_map(seg, image, cen)
    qs = SM.q_from_segmentation_map(seg, image, cen, pas)
    wins = SM.windows_from_segmentation_map(seg)
    assert list(cen) == ids and list(wins) == ids
    for k, i in enumerate(ids):
        assert np.allclose(cen[i], d["centroids"][k], rtol=1e-10)
        assert abs(pas[i] - d["pas"][k]) <= 1e-10
        assert abs(qs[i] - d["qs"][k]) <= 1e-9
        assert wins[i] == d["windows"][k].tolist()
    scaled = SM.scale_windows(wins, image_shape=image.shape, expand_scale=1.5, expand_border=3)
    assert [scaled[i] for i in ids] == d["scaled"].tolist()
    kept = SM.filter_windows(scaled, min_size=30, max_area=3800, min_flux=700.0, image=image)
    assert sorted(kept) == list(d["filtered_ids"])
    # the same map read back from FITS and .npy files
    from astrophot_gb300 import fits_io

    f = str(tmp_path / "seg.fits")
    fits_io.write_hdus(f, [(seg.astype(np.int32), {})])
    np.save(str(tmp_path / "img.npy"), image)
    assert SM.windows_from_segmentation_map(f) == wins
    cen2 = SM.centroids_from_segmentation_map(f, str(tmp_path / "img.npy"))
    assert all(np.allclose(cen2[i], cen[i], rtol=1e-12) for i in ids)


def test_segment_statistics_match_oracle_on_a_large_map(SM):
    """A 1024 x 1024 map with 500 segments (random ellipses on noise): GPU against the oracle."""
    from oracle import segmap as O

    rng = np.random.default_rng(4)
    n = 1024
    yy, xx = np.mgrid[0:n, 0:n]
    seg = np.zeros((n, n), np.int32)
    img = rng.normal(scale=0.1, size=(n, n))
    for sid in range(1, 501):
        cx, cy = rng.uniform(0, n, 2)
        a, q, pa = rng.uniform(3, 20), rng.uniform(0.2, 1), rng.uniform(0, np.pi)
        dx, dy = xx - cx, yy - cy
        u = dx * np.cos(pa) + dy * np.sin(pa)
        v = (-dx * np.sin(pa) + dy * np.cos(pa)) / q
        r = np.hypot(u, v)
        m = r < a
        seg[m] = sid * 3  # ids with gaps
        img[m] += 10 * np.exp(-r[m] / (a / 3))
    img = img.astype(np.float32).astype(np.float64)
    st = SM.segment_statistics(seg, img)
    cen = O.centroids(seg, img)
    pas = O.position_angles(seg, img, cen)
    qs = O.axis_ratios(seg, img, cen, pas)
    wins = O.windows(seg)
    assert st["ids"] == list(cen)
    for k, i in enumerate(st["ids"]):
        assert np.allclose(st["centroid"][k], cen[i], rtol=1e-9)
        assert abs(st["pa"][k] - pas[i]) <= 1e-8
        assert abs(st["q"][k] - qs[i]) <= 1e-8
        assert st["bbox"][k].tolist() == [wins[i][0][0], wins[i][0][1], wins[i][1][0], wins[i][1][1]]
