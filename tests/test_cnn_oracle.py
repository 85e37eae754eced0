"""The FP64 CNN oracle (checker of the learned-initial-guess kernels) against finite
differences, and the host-side pieces of the learned initial guess that need no GPU."""

import math

import numpy as np
import pytest

from oracle import cnn as C


def random_params(rng, scale=1.0):
    p = np.zeros(C.PARAM_COUNT)
    for l, (cin, cout, hin, hout, K, N) in enumerate(C.LAYERS):
        fan = 9 * cin if l < C.N_CONV else K
        W = rng.normal(0, scale * math.sqrt(2.0 / fan), size=(N, K))
        if l == 0:
            W[:, 9:] = 0
        p[C.W_OFF[l] : C.W_OFF[l] + N * K] = W.reshape(-1)
        p[C.B_OFF[l] : C.B_OFF[l] + N] = rng.normal(0, 0.05, N)
    return p


def test_layer_table_matches_parameter_count():
    assert C.PARAM_COUNT == 1_176_008 + 7 * 32 + 8 * 192 + 8  # padding of layer 1 K and layer 6 rows
    trainable = sum(9 * cin * cout + cout for cin, cout, *_ in C.LAYERS[:4]) + 4096 * 192 + 192 + 192 * 8 + 8
    assert trainable == 1_176_008


def test_im2col_col2im_are_adjoint():
    rng = np.random.default_rng(0)
    x = rng.normal(size=(2, 8, 8, 3))
    y = rng.normal(size=(2 * 16, 27))
    assert np.dot(C.im2col(x).reshape(-1), y.reshape(-1)) == pytest.approx(np.sum(x * C.col2im(y, 2, 8, 3)), rel=1e-12)


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = random_params(rng)
    x = rng.normal(size=(2, 64, 64))
    t = rng.normal(size=(2, 8))

    def loss(pp):
        out, _ = C.forward(pp, x)
        return C.mse(out, t)[0]

    out, cache = C.forward(p, x)
    _, dout = C.mse(out, t)
    g = C.backward(p, cache, dout)
    for l, (cin, cout, hin, hout, K, N) in enumerate(C.LAYERS):
        kmax = 9 * cin if l < C.N_CONV else K
        nmax = 8 if l == len(C.LAYERS) - 1 else N
        idx = [C.W_OFF[l] + int(rng.integers(nmax)) * K + int(rng.integers(kmax)) for _ in range(4)]
        idx += [C.B_OFF[l] + int(rng.integers(nmax)) for _ in range(2)]
        for i in idx:
            h = 1e-6
            pp, pm = p.copy(), p.copy()
            pp[i] += h
            pm[i] -= h
            fd = (loss(pp) - loss(pm)) / (2 * h)
            assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)) + 1e-9, (l, i, fd, g[i])


def test_stamp_parameter_draws_and_psf_bank():
    from astrophot_gb300 import cnn

    p = cnn.draw_stamp_params(np.random.default_rng(3), 20000)
    assert np.all(np.abs(p[:, 0] - 32) <= 1) and np.all(np.abs(p[:, 1] - 32) <= 1)
    assert p[:, 2].min() >= 0.3 and p[:, 2].max() < 0.999
    assert p[:, 3].min() >= 0 and p[:, 3].max() < math.pi
    assert p[:, 4].min() >= 0.5 and p[:, 4].max() <= 4
    assert p[:, 5].min() >= 5 and p[:, 5].max() <= 20
    assert p[:, 6].min() >= 0 and p[:, 6].max() <= 2 and np.all(p[:, 7] == 0)
    bank = cnn.psf_bank()
    assert len(bank) == 64
    sides = [k.shape[0] for k in bank]
    assert sides[0] == 9 and sides[-1] == 21 and all(s % 2 == 1 for s in sides)
    assert all(np.isclose(k.sum(), 1.0) for k in bank)
    # centred: the peak sits in the middle pixel
    assert all(k.argmax() == (k.shape[0] // 2) * (k.shape[1] + 1) for k in bank)


def test_committed_weights_have_the_network_layout():
    import os

    from astrophot_gb300 import cnn

    if not os.path.exists(cnn.WEIGHTS_PATH):
        pytest.skip("no trained weights in the tree")
    z = np.load(cnn.WEIGHTS_PATH)
    assert z["params"].shape == (C.PARAM_COUNT,)
    assert np.all(np.isfinite(z["params"]))
    assert z["mean"].shape == (8,) and np.all(z["std"] > 0)
    # padding entries stay zero through training (zero gradient, zero moments)
    W1 = z["params"][C.W_OFF[0] : C.W_OFF[0] + 32 * 16].reshape(32, 16)
    assert np.all(W1[:, 9:] == 0)
