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


def test_rocking_scan_configuration():
    """544 x 1056 x 490, 256 deviation parameters over +-300 urad, 64
    segments along signed <110> with (a/2)<110> Burgers vectors, midpoints
    in the illuminated volume, lengths in [20, 800] um."""
    from dyfox_gb300.units import deviation_from_urad
    from dyfox_gb300.workloads import DIRS_110, laue_rocking_scan
    x, grid, segs, s = laue_rocking_scan()
    Nx, Ny, dz, ds, shift = grid.geometry()
    assert (Ny, Nx, grid.Nz, shift) == (544, 1056, 490, 1.0)
    assert len(s) == 256
    assert np.allclose(s[[0, -1]], deviation_from_urad([-300.0, 300.0], x))
    assert len(segs) == 64
    t = grid.t_crystal
    dirs = DIRS_110 / np.sqrt(2.0)
    n_edge = 0
    for ra, rb, b in segs:
        ra, rb, b = (np.asarray(v, float) for v in (ra, rb, b))
        L = np.linalg.norm(rb - ra)
        assert 20e-6 * (1 - 1e-12) <= L <= 800e-6 * (1 + 1e-12)
        xi = (rb - ra) / L
        assert np.min(np.linalg.norm(dirs - xi, axis=1)) < 1e-12
        assert abs(np.linalg.norm(b) - x.b_mag) < 1e-12 * x.b_mag
        assert np.min(np.linalg.norm(dirs - b / x.b_mag, axis=1)) < 1e-12
        n_edge += abs(np.dot(xi, b)) < 1e-12 * x.b_mag
        c = (ra + rb) / 2
        assert abs(c[0]) <= t * x.tan_tB and abs(c[1]) < 60e-6
        assert 0.0 <= c[2] <= t
    # about half pure edge by construction, plus the perpendicular draws
    # among the "any of the 12" half
    assert 20 <= n_edge <= 56


def test_bragg_config1():
    from dyfox_gb300.workloads import bragg_config1
    x, cfg, seg, s, ys, g = bragg_config1()
    assert (cfg.Nz, cfg.Nx) == (90, 456)
    assert len(s) == 21 and np.isclose(s[10], 0.0, atol=1e-30)
    assert len(ys) == 64 and np.isclose(ys[32] - ys[31], cfg.dx)
    assert np.isclose(ys.mean(), 0.0, atol=1e-18)
    assert len(seg) == 1
    assert np.allclose(g[:2], 0.0) and g[2] > 0


def test_learned_guess_instances():
    """Thickness on the asked range (Nz 90 to 894 at dx = 0.25 um over
    10-100 um; with half_x set by the 256-px field, Nx 648 to 3864), 256
    planes, the field centred in the padded grid, 1-32 segments whose
    midpoints lie within 5 um of the surface, 64 deviation parameters over
    +-5 Darwin widths."""
    from dyfox_gb300.bragg_geometry import BraggConfig
    from dyfox_gb300.workloads import diamond_400, learned_guess_instances
    x = diamond_400()
    lo = BraggConfig(x, t_crystal=10e-6, dx=0.25e-6, half_x=32e-6)
    hi = BraggConfig(x, t_crystal=100e-6, dx=0.25e-6, half_x=32e-6)
    assert (lo.Nz, lo.Nx, hi.Nz, hi.Nx) == (90, 648, 894, 3864)
    inst = learned_guess_instances(12)
    for w in inst:
        c = w["cfg"]
        assert lo.Nz <= c.Nz <= hi.Nz and lo.Nx <= c.Nx <= hi.Nx
        assert len(w["ys"]) == 256 and len(w["s"]) == 64
        assert w["col0"] == c.Nx // 2 - 128 and w["field"] == 256
        assert 1 <= len(w["segs"]) <= 32
        for ra, rb, b in w["segs"]:
            mid = (np.asarray(ra) + np.asarray(rb)) / 2
            assert 0.0 <= mid[2] <= 5e-6 + 1e-18
            assert abs(mid[0]) <= 32e-6 and abs(mid[1]) <= 32e-6
