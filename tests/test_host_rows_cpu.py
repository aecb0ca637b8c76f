"""WaveCache keys and illumination nodes against the reference's own
values (tests/golden/host_rows.npz)."""

import json

import numpy as np

from conftest import golden


def test_cache_keys_match_the_reference(diamond400):
    from dyfox_gb300.backend import FP32, FP64
    from dyfox_gb300.cache import WaveCache
    from dyfox_gb300.grid import LaueGrid
    g = golden("host_rows")
    q = g["seg"][0]
    seg = [(q[:3], q[3:6], q[6:])]
    grid = LaueGrid(diamond400, t_crystal=200e-6, dx=0.25e-6,
                    beam_width=120e-6)
    got = [WaveCache("w").key(seg, [0.0, 1e3], grid, diamond400, FP64),
           WaveCache("w").key(seg, [0.0, 1e3], grid, diamond400, FP32),
           WaveCache("w", store_dtype=np.complex128).key(
               seg, [-2.5e3], grid, diamond400, FP64),
           WaveCache("w", version=8).key(seg, [0.0], grid, diamond400, FP64)]
    assert got == list(g["cache_keys"])
    p = WaveCache("dir").path(seg, [0.0], grid, diamond400, FP32, tag="e")
    assert p.startswith("dir/fp32_e_") and p.endswith(".npy")


def test_illumination_nodes_match_the_reference(diamond400):
    from dyfox_gb300.illumination import (condenser_angles,
                                          convergence_bandwidth_nodes,
                                          gauss_hermite_offsets)
    g = golden("host_rows")
    a, w = condenser_angles(3.6)
    assert np.array_equal(a, g["cond_a"]) and np.array_equal(w, g["cond_w"])
    o, wo = gauss_hermite_offsets(1.5e-6, n=5)
    assert np.allclose(o, g["gh_offs"], rtol=1e-15, atol=0)
    assert np.allclose(wo, g["gh_w"], rtol=1e-15, atol=0)
    for name, kw in (("plain", {}), ("psi", {"matched": "psi"}),
                     ("delta", {"matched": "delta"}),
                     ("vignette", {"vignette_f": 2.0e4})):
        S, D, W, info = convergence_bandwidth_nodes(
            diamond400, 20e-6, 1e-4, 9, 40e-6, 7, 3e-4, **kw)
        assert np.allclose(S, g[name + "_S"], rtol=1e-14, atol=0), name
        assert np.allclose(D, g[name + "_D"], rtol=1e-14, atol=0), name
        assert np.allclose(W, g[name + "_W"], rtol=1e-14, atol=0), name
        assert json.dumps(info, sort_keys=True) == str(g[name + "_info"])


def test_bragg_segment_builders_match_the_reference(diamond400):
    """threading_segment (edge and screw, both signs, three tilts and
    azimuths) and edge_segment (default and given depth, both signs)
    against the reference's builders (bragg/geometry.py:69-109)."""
    from dyfox_gb300.bragg_geometry import edge_segment, threading_segment
    g = golden("host_rows")

    class Slab:
        t_crystal = 20e-6

    built = []
    for kind in ("Edge", "Screw"):
        for sign in (1, -1):
            for psi, az in ((np.pi / 4, 0.0), (0.3, 30.0), (1.1, -75.0)):
                built.append(threading_segment(kind, sign, diamond400.b_mag,
                                               4.0e10, psi, 0.3e-6, -0.2e-6,
                                               az))
    for depth in (None, 3e-6):
        for sign in (1, -1):
            built.append(edge_segment(sign, Slab, diamond400.b_mag, depth))
    got = np.array([np.concatenate([np.asarray(q, float) for q in b[0]])
                    for b in built])
    np.testing.assert_allclose(got, g["builders"], rtol=1e-15, atol=1e-30)
