"""Host-side tables of the scene's fixed-order sums (no GPU): the entries and contributions of
J^T W J and J^T v, against a dense accumulation of the same block partial sums, with linked
centres (several sources sharing joint-vector entries) and a whole-image entry."""

import numpy as np
import pytest

pytest.importorskip("torch")

from astrophot_gb300.scene import gather_table, hess_contributions, jt_contributions  # noqa: E402


def _gather(entries, contribs, part, n_out):
    """What ap_gather_sum computes: each entry the sum of its contributions, in table order."""
    uniq, ptr, c = gather_table(entries, contribs)
    out = np.zeros(n_out)
    for e in range(len(uniq)):
        t = 0.0
        for k in range(ptr[e], ptr[e + 1]):
            t += part[c[k]]
        out[uniq[e]] = t
    return out, uniq, ptr, c


def _scene(rng, n_src=7):
    # sources with 5-7 free slots; source 2k + 1 shares the first two slots (its centre) of 2k
    nf = rng.integers(5, 8, size=n_src)
    gid = np.full((n_src + 1, 8), -1, dtype=np.int64)
    g = 0
    for s in range(n_src):
        for c in range(nf[s]):
            if s % 2 == 1 and c < 2:
                gid[s, c] = gid[s - 1, c]
            else:
                gid[s, c] = g
                g += 1
    # whole-image entry: one column (a free sky)
    gid[n_src, 0] = g
    g += 1
    return np.append(nf, 1), gid, g


def test_jt_table_sums_every_source_slot_once():
    rng = np.random.default_rng(3)
    nf, gid, P = _scene(rng)
    part = rng.normal(size=len(nf) * 8)
    out, uniq, ptr, c = _gather(*jt_contributions(nf, gid), part, P)
    want = np.zeros(P)
    for s in range(len(nf)):
        for k in range(nf[s]):
            want[gid[s, k]] += part[8 * s + k]
    assert np.allclose(out, want, rtol=1e-15, atol=0)
    assert np.all(np.diff(uniq) > 0) and np.all(np.diff(ptr) > 0)
    for e in range(len(uniq)):  # contributions in ascending order: one summation order
        assert np.all(np.diff(c[ptr[e] : ptr[e + 1]]) > 0)


def test_hess_table_matches_dense_accumulation_and_is_symmetric():
    rng = np.random.default_rng(5)
    nf, gid, P = _scene(rng)
    ns = len(nf)
    pairs = [(a, b) for a in range(ns) for b in range(a, ns) if rng.random() < 0.6 or a == b]
    # block partial sums of a symmetric product: pair (a, a)'s block symmetric
    part = rng.normal(size=len(pairs) * 64)
    for p, (a, b) in enumerate(pairs):
        if a == b:
            blk = part[64 * p : 64 * p + 64].reshape(8, 8)
            part[64 * p : 64 * p + 64] = ((blk + blk.T) / 2).reshape(-1)
    out, _, _, _ = _gather(*hess_contributions(nf, gid, pairs, P), part, P * P)
    H = out.reshape(P, P)
    want = np.zeros((P, P))
    for p, (a, b) in enumerate(pairs):
        blk = part[64 * p : 64 * p + 64].reshape(8, 8)
        for i in range(nf[a]):
            for k in range(nf[b]):
                want[gid[a, i], gid[b, k]] += blk[i, k]
                if a != b:
                    want[gid[b, k], gid[a, i]] += blk[i, k]
    assert np.allclose(H, want, rtol=1e-12, atol=1e-12)
    assert np.array_equal(H, H.T)


def test_no_pairs_gives_an_empty_table():
    uniq, ptr, c = gather_table(*hess_contributions(np.array([3]), np.zeros((1, 8), dtype=np.int64), [], 3))
    assert len(uniq) == 0 and list(ptr) == [0] and len(c) == 0
