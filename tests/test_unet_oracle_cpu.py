"""The NumPy U-Net oracle (the checker of the CUDA training kernels),
pinned by central finite differences of its own loss."""

import numpy as np
import pytest

from oracle import unet_oracle as U


def test_layout_counts():
    assert U.n_params() == sum(9 * ci * co + co for _, ci, co in U.CONVS) \
        + 2 * 32 + 2
    flat = np.arange(U.n_params(), dtype=float)
    assert np.array_equal(U.flatten(U.unflatten(flat)), flat)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -3.14159, 0.0])
    r = U.bf16(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                       # tie to even
    assert r[2] == 1.0 + 4 * 2 ** -8         # tie to even (upwards)
    assert abs(r[3] + 3.140625) < 1e-12
    assert r[4] == 0.0


def test_gradients_match_finite_differences():
    rng = np.random.default_rng(3)
    p = U.init_params(seed=1)
    for k in p:                      # non-zero biases exercise db
        if k.endswith(".b"):
            p[k] = rng.normal(size=p[k].shape) * 0.05
    x = rng.normal(size=(2, 8, 8, U.C_IN))
    x[..., 17:] = 0.0
    t = rng.normal(size=(2, 8, 8, 2))
    y, cache = U.forward(p, x)
    g = U.backward(p, cache, y, t)
    h = 1e-6
    for name in ("e0a.W", "e1b.W", "ba.b", "bb.W", "d2a.W", "d0b.b",
                 "head.W", "head.b"):
        for _ in range(3):
            idx = tuple(rng.integers(0, n) for n in p[name].shape)
            old = p[name][idx]
            p[name][idx] = old + h
            lp = U.loss(U.forward(p, x)[0], t)
            p[name][idx] = old - h
            lm = U.loss(U.forward(p, x)[0], t)
            p[name][idx] = old
            fd = (lp - lm) / (2 * h)
            assert g[name][idx] == pytest.approx(fd, rel=1e-4, abs=1e-9), \
                (name, idx)
