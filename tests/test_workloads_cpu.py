"""The seeded workload generators (host only)."""

import numpy as np

from dyfox_gb300.workloads import batched_uneven


def test_batched_uneven_mix_and_ranges():
    a = batched_uneven(n=64, seed=7)
    b = batched_uneven(n=64, seed=7)
    kinds = [w["kind"] for w in a]
    assert kinds.count("laue") == round(0.7 * 64)
    assert kinds == [w["kind"] for w in b]
    for w, v in zip(a, b):
        assert np.array_equal(w["s"], v["s"])
        assert 1 <= len(w["s"]) <= 64
        assert 1 <= len(w["segs"]) <= 128
        if w["kind"] == "laue":
            g = w["grid"]
            Nx, Ny, dz, ds, shift = g.geometry()
            assert 128 <= Ny <= 1024 and 128 <= Nx <= 512 and Nx <= Ny
            assert Nx % 2 == 0 and shift == 1.0
            assert 50e-6 - dz <= g.t_crystal <= 400e-6 + dz
            assert g.dx in (0.125e-6, 0.25e-6, 0.5e-6)
        else:
            c = w["cfg"]
            assert 1 <= len(w["ys"]) <= 8
            assert 5e-6 - c.dz <= c.t_crystal <= 20e-6 + c.dz
            assert c.Nx == 2 * (round(c.half_x / c.dx) + 2 * c.Nz + 16)
