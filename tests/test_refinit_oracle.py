"""The oracle of the reference's initial-value heuristics (``initialize()``) against the
reference's own outputs recorded in ``tests/golden/init_*.npz``, and its Nelder-Mead
restatement against scipy's."""

import numpy as np
import pytest

import cases
from oracle import refinit

NAMES = cases.init_case_names()


def _names(kind):
    return ["center", "q", "PA", "n", "Re", "Ie"] if kind == "sersic" else ["center", "q", "PA", "Re", "Ie"]


@pytest.mark.parametrize("name", NAMES)
def test_oracle_matches_reference_initialize(name):
    d = cases.load_init(name)
    spec = d["spec"]
    out = refinit.initialize(d["data"], spec["kind"], spec["scale"], mask=d["mask"], given=spec.get("given"))
    for k in _names(spec["kind"]):
        assert np.allclose(out[k], d[f"value_{k}"], rtol=1e-12, atol=1e-12), (k, out[k], d[f"value_{k}"])
    if "profile_R" in out:
        assert np.allclose(out["profile_R"], d["profile_R"], rtol=1e-12)
        assert np.allclose(out["profile_I"], d["profile_I"], rtol=1e-12, atol=1e-12)


def test_golden_cases_cover_the_quirks():
    names = set(NAMES)
    assert {"init_exp_64", "init_sersic_mask", "init_sersic_offcentre", "init_sersic_given", "init_sersic_big"} <= names
    # the exponential initialiser's swapped arguments: "Re" is the fitted amplitude
    d = cases.load_init("init_exp_64")
    assert d["value_Re"] < 0.5 * d["spec"]["params"]["Re"]
    # the 96 x 96 case reaches the nearest-pixel isophote sampler (radius >= 30)
    out = refinit.initialize(cases.load_init("init_sersic_big")["data"], "sersic", 1.0)
    assert out["iso_R"] >= 30


OBJECTIVES = [
    lambda x: (1 - x[0]) ** 2 + 100 * (x[1] - x[0] ** 2) ** 2 + (x[2] - 1) ** 2,
    lambda x: np.sum((x - np.array([0.3, -2.0, 5.0])) ** 2 * np.array([1, 10, 100])),
    lambda x: np.abs(x).sum(),
    lambda x: np.sum(x**2) + 0.01 * np.sin(1000 * x).sum(),  # rugged
    lambda x: -np.sum(np.log1p(np.abs(x))),  # unbounded: stops at the evaluation limit
]


@pytest.mark.parametrize("k", range(len(OBJECTIVES)))
def test_nelder_mead_matches_scipy(k):
    from scipy.optimize import minimize

    rng = np.random.default_rng(k)
    f = OBJECTIVES[k]
    for _ in range(3):
        x0 = rng.normal(size=3) * 2
        x, ok, calls = refinit.nelder_mead(f, x0)
        r = minimize(f, x0=x0, method="Nelder-Mead")
        assert np.array_equal(x, r.x)
        assert ok == r.success and calls == r.nfev
    if k == len(OBJECTIVES) - 1:
        assert not ok


def test_percentile_and_clip_helpers():
    rng = np.random.default_rng(5)
    v = rng.normal(size=101)
    assert refinit.iqr_half(v) == (np.percentile(v, 84) - np.percentile(v, 16)) / 2
    lim = refinit.sigma_clip_upper(np.r_[v, 40.0, 55.0], 10, 3)
    assert 2.0 < lim < 40.0
