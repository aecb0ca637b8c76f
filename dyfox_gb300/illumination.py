"""Quadrature nodes for a beam that is not one coherent plane wave.

Drop-in for DYFOX ``illumination.py:16-86`` (host NumPy; the same nodes,
weights and node order, since they decide which deviation parameters get
solved and in which order):

    condenser_angles             incidence angles and weights of a focused
                                 (condenser) beam
    gauss_hermite_offsets        n x n lateral offsets and weights of a
                                 Gaussian source
    convergence_bandwidth_nodes  product rule over incidence angle and
                                 energy band, ordered from the Bragg
                                 condition outward: the uneven deviation
                                 sets that feed batched scans

The rules, as used here:

* Condenser: nodes every ``w_D`` across +-4 ``w_D`` of the Bragg
  condition, plus every multiple of 5 (angle units) out to ``reach``, and
  0; each node weighs the spacing around it -- half the distance between
  its two neighbours, the distance to the single neighbour at the two
  ends.  Both node runs follow the floating-point arithmetic of DYFOX's
  node list (a run from a0 by h holds a0, a0 + h, then a0 + i (a1 - a0)
  with a1 = a0 + h as rounded; as many nodes as cover the span + 1e-9), so
  that the node set is the same to the bit: for some w_D (3.6, for one)
  the fifth fine node lands a rounding error away from 0 and, with the
  exact 0, leaves two nodes that share the weight about 0.
* Gaussian source: the tensor product of the n-point Gauss-Hermite rule
  for the weight exp(-t^2 / 2) along each lateral axis, scaled by the rms
  width, with the first axis varying fastest; weights normalised to one.
* Angle x band: equispaced angle offsets psi on [-psi_max, psi_max] and
  band offsets delta on [-del_max, del_max], each weighted by its Gaussian
  (a flat band when ``sig_delta`` <= 0), weights normalised over the grid.
  A node's deviation parameter is s = (psi + tan(theta_B) delta)
  sin(2 theta_B) / lambda and its chromatic argument d = delta + psi /
  tan(2 theta_B).  ``matched="psi"`` shifts every angle by -tan(theta_B)
  delta (each energy brought back onto the Bragg condition);
  ``matched="delta"`` replaces the band offset by -psi / tan(theta_B)
  (the band fully correlated with the angle).  ``vignette_f`` removes the
  nodes whose chromatic carrier |sin(2 theta_B) d / lambda| exceeds it,
  without renormalising: the kept weight is reported as the band fraction.
"""

import numpy as np


def _run(a0, end, h):
    """Nodes from a0 by h below ``end``, in the rounding of DYFOX's list:
    a0, a0 + h, then a0 + i (a1 - a0) with a1 the rounded a0 + h."""
    n = max(int(np.ceil((end - a0) / h)), 0)
    a1 = a0 + h
    out = a0 + np.arange(n, dtype=float) * (a1 - a0)
    if n > 1:
        out[1] = a1
    return out


def condenser_angles(w_D, reach=75.0):
    """(angles, weights) of the condenser rule: multiples of ``w_D`` within
    +-4 ``w_D`` and multiples of 5 within +-``reach``, merged and sorted;
    each weight is the node spacing about its node."""
    near = _run(-4.0 * w_D, 4.0 * w_D + 1e-9, w_D)
    far = _run(-reach, reach + 1e-9, 5.0)
    nodes = np.unique(np.concatenate([near, far, [0.0]]))
    spacing = np.empty_like(nodes)
    if len(nodes) == 1:
        spacing[:] = 0.0
        return nodes, spacing
    spacing[1:-1] = 0.5 * (nodes[2:] - nodes[:-2])
    spacing[0] = nodes[1] - nodes[0]
    spacing[-1] = nodes[-1] - nodes[-2]
    return nodes, spacing


def gauss_hermite_offsets(sigma, n=8):
    """(offsets (n*n, 2), weights (n*n,)) of a Gaussian source of rms
    ``sigma``: probabilists' Gauss-Hermite nodes on both axes, the first
    axis varying fastest, weights summing to one."""
    t, w = np.polynomial.hermite_e.hermegauss(n)
    first = np.tile(t, n)                 # fastest axis
    second = np.repeat(t, n)
    weight = np.tile(w, n) * np.repeat(w, n)
    offsets = sigma * np.column_stack([first, second])
    return offsets, weight / weight.sum()


def _gauss_weights(t, sigma):
    return np.exp(-0.5 * (t / sigma) ** 2)


def convergence_bandwidth_nodes(xtal, sig_psi, sig_delta, n_psi, psi_max,
                                n_delta, del_max, *, matched=None,
                                vignette_f=None):
    """Product quadrature over angular spread and energy band.

    Returns (s, d, w, info): deviation parameters (1/m), chromatic
    arguments and weights of the kept nodes, ordered by |s| from the Bragg
    condition outward, and {"n_total", "n_kept", "band_fraction"}."""
    lam, theta = float(xtal.lam), float(xtal.theta_B)
    sin_2t = float(xtal.sin_2tB)
    tan_t, tan_2t = np.tan(theta), np.tan(2 * theta)

    psi_axis = np.linspace(-psi_max, psi_max, n_psi)
    band_axis = np.linspace(-del_max, del_max, n_delta)
    psi_w = _gauss_weights(psi_axis, sig_psi)
    band_w = (_gauss_weights(band_axis, sig_delta) if sig_delta > 0
              else np.ones_like(band_axis))

    # (angle, band) grid, angle index first.
    psi = np.broadcast_to(psi_axis[:, None], (n_psi, n_delta))
    band = np.broadcast_to(band_axis[None, :], (n_psi, n_delta))
    if matched == "psi":
        psi = psi - tan_t * band
    if matched == "delta":
        band = -psi / tan_t
    weight = psi_w[:, None] * band_w[None, :]
    weight = weight / weight.sum()
    s = (psi + tan_t * band) * sin_2t / lam
    d = band + psi / tan_2t

    order = np.argsort(np.abs(s).ravel())          # near-Bragg first
    s, d, weight = (a.ravel()[order] for a in (s, d, weight))
    info = {"n_total": int(s.size), "n_kept": int(s.size),
            "band_fraction": 1.0}
    if vignette_f is not None:
        inside = np.abs(sin_2t * d / lam) <= vignette_f
        if not inside.all():
            s, d, weight = s[inside], d[inside], weight[inside]
            info["n_kept"] = int(inside.sum())
            info["band_fraction"] = float(weight.sum())
    return s, d, weight, info
