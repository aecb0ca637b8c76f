"""Fits the polynomial of atan2_fast (volterra.cuh).

atan(t) = t P(t^2) on [0, 1], P of degree 7 in t^2 (an odd polynomial of
degree 15), minimax in absolute error by Lawson's algorithm (iteratively
re-weighted least squares), coefficients rounded to float32.  Prints the
coefficients and the float32 evaluation error.

    python dyfox_gb300/csrc/fit_atan.py
"""

import numpy as np


def fit(n_coef=8, iters=200):
    t = np.sort(np.concatenate([0.5 + 0.5 * np.cos(np.linspace(0, np.pi, 4000)),
                                np.linspace(0.0, 1.0, 4000)]))
    A = np.stack([t ** (2 * k + 1) for k in range(n_coef)], 1)
    y = np.arctan(t)
    w = np.ones_like(t)
    for _ in range(iters):
        c, *_ = np.linalg.lstsq(A * np.sqrt(w)[:, None], y * np.sqrt(w),
                                rcond=None)
        w = w * (np.abs(A @ c - y) + 1e-30)
        w /= w.sum()
    return c.astype(np.float32)


def eval_f32(c, t):
    t = np.asarray(t, np.float32)
    t2 = t * t
    p = c[-1]
    for k in range(len(c) - 2, -1, -1):
        p = p * t2 + c[k]
    return p * t


if __name__ == "__main__":
    c = fit()
    tt = np.linspace(0, 1, 200001)
    err = np.abs(eval_f32(c, tt).astype(np.float64) - np.arctan(tt)).max()
    print("coefficients:", ", ".join(f"{float(v)!r}f" for v in c))
    print(f"max |error| in float32: {err:.3e}")
