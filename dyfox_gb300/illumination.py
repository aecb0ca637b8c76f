"""Sampling a beam that is not a single coherent plane wave.

Drop-in for DYFOX ``illumination.py:16-86`` (host NumPy, same nodes and
weights):

    condenser_angles             incidence angles and weights for a
                                 focused beam
    gauss_hermite_offsets        n*n offsets and weights for a Gaussian
                                 source
    convergence_bandwidth_nodes  joint quadrature over incidence angle and
                                 energy band, ordered from the Bragg
                                 condition outward: the uneven deviation
                                 sets that feed batched scans
"""

import numpy as np


def condenser_angles(w_D, reach=75.0):
    """Angles every w_D across +-4 w_D, then every 5 units out to
    ``reach``; weights are the node spacing."""
    fine = np.arange(-4.0 * w_D, 4.0 * w_D + 1e-9, w_D)
    coarse = np.arange(-reach, reach + 1e-9, 5.0)
    a = np.unique(np.concatenate([fine, coarse, [0.0]]))
    return a, np.gradient(a)


def gauss_hermite_offsets(sigma, n=8):
    """n*n offsets of a Gaussian source of rms ``sigma`` and weights
    summing to one (probabilists' Gauss-Hermite nodes)."""
    x, w = np.polynomial.hermite_e.hermegauss(n)
    X, Y = np.meshgrid(x, x)
    WX, WY = np.meshgrid(w, w)
    offs = np.stack([X.ravel() * sigma, Y.ravel() * sigma], axis=1)
    wts = (WX * WY).ravel()
    return offs, wts / wts.sum()


def convergence_bandwidth_nodes(xtal, sig_psi, sig_delta, n_psi, psi_max,
                                n_delta, del_max, *, matched=None,
                                vignette_f=None):
    """An n_psi x n_delta grid over angular spread and energy band with
    Gaussian weights; ``matched`` ("psi" or "delta") ties the two;
    ``vignette_f`` drops nodes whose chromatic carrier lies outside the
    objective.  Returns (deviation parameters, chromatic arguments,
    weights) sorted by |s| and a dict of node counts."""
    lam = float(xtal.lam)
    theta_B = float(xtal.theta_B)
    sin_2tB = float(xtal.sin_2tB)
    tan2t = np.tan(2 * theta_B)
    psi = np.linspace(-psi_max, psi_max, n_psi)
    del_ = np.linspace(-del_max, del_max, n_delta)
    w_psi = np.exp(-0.5 * (psi / sig_psi) ** 2)
    w_del = (np.exp(-0.5 * (del_ / sig_delta) ** 2) if sig_delta > 0
             else np.ones_like(del_))
    PSI, DEL = np.meshgrid(psi, del_, indexing="ij")
    if matched == "psi":
        PSI = PSI - np.tan(theta_B) * DEL
    if matched == "delta":
        DEL = -PSI / np.tan(theta_B)
    W = np.outer(w_psi, w_del)
    W /= W.sum()
    S_DEV = (PSI + np.tan(theta_B) * DEL) * sin_2tB / lam
    D_ARG = DEL + PSI / tan2t
    order = np.argsort(np.abs(S_DEV).ravel())
    S_flat = S_DEV.ravel()[order]
    D_flat = D_ARG.ravel()[order]
    W_flat = W.ravel()[order]
    info = {"n_total": len(S_flat), "n_kept": len(S_flat),
            "band_fraction": 1.0}
    if vignette_f is not None:
        keep = np.abs(sin_2tB * D_flat / lam) <= vignette_f
        if not keep.all():
            S_flat, D_flat, W_flat = S_flat[keep], D_flat[keep], W_flat[keep]
            info["n_kept"] = int(keep.sum())
            info["band_fraction"] = float(W_flat.sum())
    return S_flat, D_flat, W_flat, info
