"""The oracle and the host-side inputs, pinned to the reference's golden
vectors (CPU only).

tests/golden was generated from the DYFOX reference itself by
tests/golden/make_golden.py; oracle/_ref (when built) is the reference's
Laue kernel text compiled for the CPU.
"""

import numpy as np
import pytest

from conftest import golden, rel_l2
from oracle import closed_forms as CF
from oracle import oracle as O


def test_crystal_parameters_match_the_reference(diamond400):
    g = golden("crystal")
    for name in ("sig0", "sig_h", "sig_hbar", "lam", "theta_B", "tan_tB",
                 "cos_tB", "sin_tB", "sin_2tB", "xi_g", "b_mag", "a_core",
                 "nu", "F_g"):
        assert getattr(diamond400, name) == pytest.approx(complex(g[name]),
                                                          rel=1e-15), name
    np.testing.assert_allclose(diamond400.g_vec, g["g_vec"], rtol=1e-15)


def test_known_answers(diamond400):
    """Independent first-principles values (reference tests/test_crystal.py,
    test_bragg.py, test_units.py)."""
    assert diamond400.lam * 1e10 == pytest.approx(0.72932, abs=1e-5)
    assert np.degrees(diamond400.theta_B) == pytest.approx(24.137, abs=1e-3)
    assert abs(diamond400.F_g) == pytest.approx(12.736, abs=1e-3)
    assert diamond400.sig0.real == pytest.approx(-72.45, abs=0.01)
    assert diamond400.xi_g * 1e6 == pytest.approx(54.47, abs=0.01)
    assert CF.darwin_width_urad(diamond400) == pytest.approx(3.588, abs=0.01)


def test_deviation_parameter(diamond400):
    from dyfox_gb300.units import deviation_from_urad, urad_from_deviation
    g = golden("crystal")
    np.testing.assert_allclose(deviation_from_urad(g["urads"], diamond400),
                               g["s_dev"], rtol=1e-15)
    np.testing.assert_allclose(urad_from_deviation(g["s_dev"], diamond400),
                               g["urads"], rtol=1e-12, atol=1e-12)
    assert CF.darwin_width_urad(diamond400) == pytest.approx(
        float(g["darwin_urad"]), rel=1e-14)


def test_laue_grid_rules_match_the_reference(diamond400):
    from dyfox_gb300.grid import LaueGrid
    for row in golden("grids")["laue"]:
        t, dx, bw, bt, sig, nz, pad = row[:7]
        g = LaueGrid(diamond400, t, dx, bw, beam_thickness=bt,
                     beam_sigma=sig, Nz=None if nz < 0 else int(nz),
                     grid_pad=int(pad))
        Nx, Ny, dz, ds, sp = g.geometry()
        assert (Nx, Ny, g.Nz) == (row[7], row[8], row[9])
        assert [dz, ds, sp, g.t_crystal, float(g.exact), g.sheet_arg()] == \
            pytest.approx(list(row[10:16]), rel=1e-15)


def test_bragg_grid_rules_match_the_reference(diamond400):
    from dyfox_gb300.bragg_geometry import BraggConfig
    for t, dx, hx, Nz, Nx, dz, ds, tc in golden("grids")["bragg"]:
        c = BraggConfig(diamond400, t_crystal=t, dx=dx, half_x=hx)
        assert (c.Nz, c.Nx) == (Nz, Nx)
        assert [c.dz, c.ds, c.t_crystal] == pytest.approx([dz, ds, tc],
                                                          rel=1e-15)


@pytest.mark.parametrize("name", ["n", "x", "r", "screw", "zero"])
def test_oracle_frames_match_volterra_frame(diamond400, name):
    v = golden("volterra")
    segs = v[f"segs_{name}"]
    fr = O.segment_frames([(s[:3], s[3:6], s[6:]) for s in segs],
                          diamond400.g_vec)
    want = v[f"frames_{name}"]
    assert len(fr) == len(want)
    for f, w in zip(fr, want):
        # golden row: b_screw, b_perp, e1, e2; oracle row: see OSEG layout
        assert f[15] == pytest.approx(w[1], rel=1e-14, abs=1e-30)
        np.testing.assert_allclose(f[6:9], w[2:5], atol=1e-15)
        np.testing.assert_allclose(f[9:12], w[5:8], atol=1e-15)


@pytest.mark.parametrize("name", ["n", "x", "r", "screw", "zero"])
def test_oracle_h_matches_h_plane(diamond400, name):
    v = golden("volterra")
    segs = [(s[:3], s[3:6], s[6:]) for s in v[f"segs_{name}"]]
    H = O.h_rows(segs, diamond400.g_vec, diamond400.nu, diamond400.a_core,
                 int(v["Nx"]), int(v["Nz"]), float(v["dx"]), float(v["dz"]),
                 v["y_planes"])
    want = v[f"H_{name}"]
    scale = max(np.abs(want).max(), 1.0)
    assert np.abs(H - want).max() <= 1e-13 * scale
    if name == "zero":
        assert np.abs(H).max() == 0.0


def _small(diamond400, small_grid):
    from dyfox_gb300.grid import grid_arrays
    return grid_arrays(small_grid)


def test_oracle_march_matches_reference_kernel(diamond400, small_grid):
    """The C restatement against the reference's CUDA text run on the CPU
    (golden), for the full-field, pristine and closed-form kernels."""
    g = golden("laue_small")
    v = golden("volterra")
    geo = _small(diamond400, small_grid)
    rows = g["rows"]
    s = g["s_dev"]
    segs = [(q[:3], q[3:6], q[6:]) for q in v["segs_n"]]
    H = O.h_rows(segs, diamond400.g_vec, diamond400.nu, diamond400.a_core,
                 geo["Nx"], geo["Nz"], geo["dx"], geo["dz"],
                 O.grid_y(geo["Ny"], geo["dx"], rows))
    got = O.laue_march("fullfield", diamond400, s, geo, H_rows=H, rows=rows)
    assert rel_l2(got, g["fullfield"]) < 1e-13
    got = O.laue_march("pristine", diamond400, s, geo, rows=rows)
    assert rel_l2(got, g["pristine"]) < 1e-15
    got = O.laue_march("analytic", diamond400, s, geo, an=v["analytic_x"],
                       rows=rows)
    assert rel_l2(got, g["analytic"]) < 1e-15


def test_oracle_interpolating_march_matches_reference(diamond400):
    g = golden("laue_small")
    Nx, Ny, Nz, dz, ds, sp = g["interp_geo"]
    assert sp != 1.0
    geo = dict(Nx=int(Nx), Ny=int(Ny), Nz=int(Nz), dz=dz, ds=ds, shift_px=sp,
               dx=0.25e-6, sheet_hw=0.5e-6, fov_hy=4e-6)
    got = O.laue_march("pristine", diamond400, g["s_dev"], geo,
                       rows=g["rows"])
    assert rel_l2(got, g["interp_pristine"]) < 1e-15


def test_oracle_is_bit_identical_to_reference_cpu_build(diamond400,
                                                         small_grid):
    """When oracle/_ref is built here, the restatement and the reference
    text give the same bits (same compiler, same flags)."""
    if O.ref_cpu() is None:
        pytest.skip("oracle/_ref not generated (no reference here)")
    geo = _small(diamond400, small_grid)
    s = golden("laue_small")["s_dev"]
    for mode in ("pristine",):
        a = O.laue_march(mode, diamond400, s, geo)
        r = O.ref_laue_march(mode, diamond400, s, geo)
        assert np.array_equal(a, r)


def test_closed_forms_match_the_reference(diamond400):
    b = golden("bragg_small")
    s = np.asarray(b["riccati_urad"])
    from dyfox_gb300.units import deviation_from_urad
    sd = deviation_from_urad(s, diamond400)
    np.testing.assert_allclose(CF.reflectivity_semi_infinite(sd, diamond400),
                               b["semi_inf"], rtol=1e-13)
    Nz, dz = b["cfg"][3], b["cfg"][5]
    got = CF.reflectivity_riccati(sd, float((Nz - 1) * dz), diamond400)
    np.testing.assert_allclose(got, b["riccati_6um"], rtol=1e-9)


# ------------------------------------------------------------------- Bragg
def _bragg_small(diamond400):
    from dyfox_gb300.bragg_geometry import BraggConfig, bragg_g_vector
    b = golden("bragg_small")
    t, dx, hx = b["cfg"][:3]
    cfg = BraggConfig(diamond400, t_crystal=t, dx=dx, half_x=hx)
    seg = [(q[:3], q[3:6], q[6:]) for q in b["segs"]]
    return b, cfg, seg, bragg_g_vector(diamond400)


def test_bragg_oracle_march_and_symbol_match_the_reference(diamond400):
    from oracle import bragg_oracle as BO
    b, cfg, seg, g = _bragg_small(diamond400)
    s = float(b["s_dev"])
    matvec, d, H, T22s = BO.system(seg, s, cfg, diamond400, g)
    np.testing.assert_allclose(H[0], b["H_row0"], rtol=0, atol=1e-13)
    assert rel_l2(d, b["d"]) < 1e-12
    assert rel_l2(matvec(b["v"]), b["Av"]) < 1e-12
    e0, eg = BO.step_factors(diamond400, s, cfg.ds)
    T21, T22 = BO.perfect_symbol(e0, eg, cfg.ds, cfg.Nz, cfg.Nx, diamond400)
    assert rel_l2(T21, b["T21"]) < 1e-14 and rel_l2(T22, b["T22"]) < 1e-14


def test_bragg_oracle_solutions_match_the_reference(diamond400):
    from oracle import bragg_oracle as BO
    b, cfg, seg, g = _bragg_small(diamond400)
    s = float(b["s_dev"])
    ew, v, res, code = BO.solve_plane(seg, s, cfg, diamond400, g)
    assert code == 0 and res < 1e-10
    assert rel_l2(ew, b["exit_wave"]) < 1e-8
    dense, _ = BO.dense_solve(seg, s, cfg, diamond400, g)
    assert rel_l2(dense, b["exit_wave"]) < 1e-8
    out, info = BO.solve_surface(seg, s, cfg, b["ys"], diamond400, g)
    assert info["converged"]
    assert rel_l2(out, b["surface"]) < 1e-8


def test_single_precision_atan2_polynomial():
    """The polynomial of atan2_fast (csrc/volterra.cuh), evaluated in float32
    with the same octant folding, against numpy.arctan2."""
    import importlib.util
    import os
    from conftest import ROOT
    spec = importlib.util.spec_from_file_location(
        "fit_atan", os.path.join(ROOT, "dyfox_gb300", "csrc", "fit_atan.py"))
    fa = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(fa)
    c = np.array([0.9999993443489075, -0.33329859375953674,
                  0.19946564733982086, -0.1390862762928009,
                  0.09642191231250763, -0.05591224133968353,
                  0.021862896159291267, -0.004054549150168896], np.float32)
    np.testing.assert_allclose(fa.fit(), c, rtol=1e-5, atol=1e-7)
    rng = np.random.default_rng(1)
    y = (rng.normal(size=200000) * 10 ** rng.uniform(-3, 3, 200000)).astype(
        np.float32)
    x = (rng.normal(size=200000) * 10 ** rng.uniform(-3, 3, 200000)).astype(
        np.float32)
    ax, ay = np.abs(x), np.abs(y)
    t = np.minimum(ax, ay) / np.maximum(ax, ay)
    r = fa.eval_f32(c, t)
    # The octant folds in float32 with pi / 2 and pi as hi + lo float pairs
    # (the kernel's kPio2Hi/Lo, kPiHi/Lo).
    f32 = np.float32
    pio2_hi, pio2_lo = f32(1.5707963705062866), f32(-4.371138828673793e-08)
    pi_hi, pi_lo = f32(3.1415927410125732), f32(-8.742277657347586e-08)
    assert abs(float(pio2_hi) + float(pio2_lo) - np.pi / 2) < 1e-14
    assert abs(float(pi_hi) + float(pi_lo) - np.pi) < 1e-14
    r = np.where(ay > ax, ((pio2_hi - r).astype(f32) + pio2_lo), r)
    r = r.astype(f32)
    r = np.where(x < 0, ((pi_hi - r).astype(f32) + pi_lo), r).astype(f32)
    err = np.copysign(r, y).astype(np.float64) - np.arctan2(
        y.astype(float), x.astype(float))
    assert np.abs(err).max() < 4e-7
    assert np.sqrt(np.mean(err ** 2)) < 1e-7


def _bragg_cfg1(diamond400):
    from dyfox_gb300.bragg_geometry import BraggConfig, bragg_g_vector
    b = golden("bragg_cfg1")
    t, dx, hx = b["cfg"][:3]
    cfg = BraggConfig(diamond400, t_crystal=t, dx=dx, half_x=hx)
    seg = [(q[:3], q[3:6], q[6:]) for q in b["segs"]]
    return b, cfg, seg, bragg_g_vector(diamond400)


def test_bragg_oracle_at_the_plain_bragg_configuration(diamond400):
    """t = 20 um, dx = 0.5 um (Nz 90, Nx 456): the oracle's dense direct
    solve against the reference's chunked SciPy GMRES answers (<= 1e-7,
    the reference's own batched-vs-single tolerance) and its closed forms
    against the reference's Riccati reflectivity at 20 um."""
    from oracle import bragg_oracle as BO
    b, cfg, seg, g = _bragg_cfg1(diamond400)
    assert (cfg.Nz, cfg.Nx) == (90, 456)
    s_all, ys = b["s_dev"], b["ys"]
    for i, k in enumerate(b["s_pick"][::2]):
        j = int(b["y_pick"][i + 1])
        dense, _ = BO.dense_solve(seg, float(s_all[k]), cfg, diamond400, g,
                                  y=float(ys[j]))
        want = b["surface"][2 * i, i + 1]
        assert np.abs(dense - want).max() < 1e-7 * np.abs(want).max()
    got = CF.reflectivity_riccati(s_all, cfg.t_crystal, diamond400)
    np.testing.assert_allclose(got, b["riccati_20um"], rtol=1e-9)
