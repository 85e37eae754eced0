"""The oracle of the reference's segmentation-map helpers against the reference's outputs
recorded in ``tests/golden/segmap_*.npz``."""

import numpy as np
import pytest

import cases
from oracle import segmap


@pytest.mark.parametrize("name", cases.segmap_case_names())
def test_segmap_oracle_matches_reference(name):
    d = cases.load_segmap(name)
    seg, image = d["seg"], d["image"]
    ids = segmap.segment_ids(seg)
    assert ids == list(d["ids"])
    cen = segmap.centroids(seg, image)
    pas = segmap.position_angles(seg, image, cen)
    qs = segmap.axis_ratios(seg, image, cen, pas)
    wins = segmap.windows(seg)
    for k, i in enumerate(ids):
        assert np.allclose(cen[i], d["centroids"][k], rtol=1e-12)
        assert np.isclose(pas[i], d["pas"][k], rtol=1e-12)
        assert np.isclose(qs[i], d["qs"][k], rtol=1e-11)
        assert wins[i] == d["windows"][k].tolist()
    scaled = segmap.scale_windows(wins, image_shape=image.shape, expand_scale=1.5, expand_border=3)
    assert [scaled[i] for i in ids] == d["scaled"].tolist()
    kept = segmap.filter_windows(scaled, min_size=30, max_area=3800, min_flux=700.0, image=image)
    assert sorted(kept) == list(d["filtered_ids"])
