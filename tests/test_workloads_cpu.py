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


def test_batch_shape_pick_breaks_near_ties_toward_fewer_warps():
    from dyfox_gb300.batch import pick_shape
    t = {(5, 8): 433.8, (5, 4): 433.9, (7, 8): 510.2, (5, 16): 532.3}
    assert pick_shape(t) == (5, 4)
    # outside the 1% window the faster shape wins
    assert pick_shape({(5, 8): 400.0, (5, 4): 420.0}) == (5, 8)
    # among equal warps, the faster
    assert pick_shape({(5, 4): 101.0, (7, 4): 100.0}) == (7, 4)
