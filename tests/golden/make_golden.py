"""Golden vectors from the DYFOX reference itself.

Run in a container that has the reference (read-only, no bytecode written):

    python tests/golden/make_golden.py [--reference /root/reference]

Writes small .npz fixtures next to this script.  Every number in them comes
from the reference's own code: its crystal, grid and Volterra routines, its
NumPy Bragg solver (SciPy GMRES), its closed-form reflectivities, and its
Laue CUDA kernel text compiled for the CPU by oracle/make_ref.py (blockDim 1,
see oracle/ref_cpu_shim.h).  The fixtures pin the oracle (oracle/) and the
GPU path; nothing at test time reads the reference.
"""

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def optics_golden():
    """Pupils and images from the reference's optics.py (NumPy): an
    Optics of the Diamond (400) 17 keV crystal on a 32 x 48 grid, charges
    0, 2 and -1, offsets of the singularity and of the aperture, phase
    levels, the three DC policies; images of a seeded stack of 3 exit waves
    through three of the pupils."""
    from crystal import DIAMOND, CrystalParams
    from optics import Optics, image_intensity
    x = CrystalParams.from_reflection(DIAMOND, (4, 0, 0), 17.0,
                                      f_prime=0.003, f_dprime=0.002,
                                      label="Diamond(400)")
    Ny, Nx, dx = 32, 48, 0.25e-6
    lens = Optics(NA=6e-5, f_lens=0.274, xtal=x, xp=np)
    step = 1.0 / (Nx * dx)
    cases = [  # (ell, aperture_f, singularity_f, dc_zero, levels)
        (0, (0.0, 0.0), (0.0, 0.0), "exact", 0),
        (2, (0.0, 0.0), (0.0, 0.0), "exact", 0),
        (-1, (0.0, 0.0), (0.0, 0.0), "never", 0),
        (2, (0.0, 0.0), (0.3 * step, -0.2 * step), "half_bin", 0),
        (1, (0.0, 0.0), (0.7 * step, 0.0), "half_bin", 0),
        (2, (1.5 * step, 0.0), (1.5 * step, 0.0), "never", 0),
        (3, (0.0, 2.0 * step), (0.0, 0.0), "exact", 4),
    ]
    pupils = np.array([lens.pupil(Nx, Ny, dx, ell, aperture_f=af,
                                  singularity_f=sf, dc_zero=dc, levels=lv,
                                  cache=False)
                       for ell, af, sf, dc, lv in cases])
    rng = np.random.default_rng(20260909)
    stack = (rng.normal(size=(3, Ny, Nx))
             + 1j * rng.normal(size=(3, Ny, Nx)))
    images = np.array([image_intensity(stack, pupils[k]) for k in (0, 1, 3)])
    phi = np.array([-12.5, 0.0, 40.0])
    np.savez_compressed(os.path.join(HERE, "optics_small.npz"),
                        Ny=Ny, Nx=Nx, dx=dx, NA=6e-5, f_lens=0.274,
                        lam=x.lam, case_ell=np.array([c[0] for c in cases]),
                        case_aperture=np.array([c[1] for c in cases]),
                        case_singularity=np.array([c[2] for c in cases]),
                        case_dc=np.array([c[3] for c in cases]),
                        case_levels=np.array([c[4] for c in cases]),
                        pupils=pupils, stack=stack, images=images,
                        image_pupils=np.array([0, 1, 3]), phi=phi)


def host_rows_golden():
    """Cache keys of the reference's laue/cache.py WaveCache and the
    nodes of its illumination.py, for a few inputs."""
    import json
    from backend import FP32, FP64
    from crystal import DIAMOND, CrystalParams
    from dislocations import burgers_vector, straight_segment
    from illumination import (condenser_angles, convergence_bandwidth_nodes,
                              gauss_hermite_offsets)
    from laue import LaueGrid
    from laue.cache import WaveCache
    x = CrystalParams.from_reflection(DIAMOND, (4, 0, 0), 17.0,
                                      f_prime=0.003, f_dprime=0.002,
                                      label="Diamond(400)")
    grid = LaueGrid(x, t_crystal=200e-6, dx=0.25e-6, beam_width=120e-6)
    b = burgers_vector(x.U_lab, [1, 0, -1], x.b_mag, +1)
    seg = straight_segment(np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0), b,
                           [0.0, 0.0, 100e-6], 800e-6)
    keys = []
    for cache, prec, s in ((WaveCache("w"), FP64, [0.0, 1e3]),
                           (WaveCache("w"), FP32, [0.0, 1e3]),
                           (WaveCache("w", store_dtype=np.complex128), FP64,
                            [-2.5e3]),
                           (WaveCache("w", version=8), FP64, [0.0])):
        keys.append(cache.key(seg, s, grid, x, prec))
    a, wa = condenser_angles(3.6)
    offs, wo = gauss_hermite_offsets(1.5e-6, n=5)
    out = {}
    for name, kw in (("plain", {}), ("psi", {"matched": "psi"}),
                     ("delta", {"matched": "delta"}),
                     ("vignette", {"vignette_f": 2.0e4})):
        S, D, W, info = convergence_bandwidth_nodes(
            x, 20e-6, 1e-4, 9, 40e-6, 7, 3e-4, **kw)
        out[name + "_S"], out[name + "_D"], out[name + "_W"] = S, D, W
        out[name + "_info"] = json.dumps(info, sort_keys=True)
    from bragg import edge_segment, threading_segment

    class _Slab:
        t_crystal = 20e-6

    built = []
    for kind in ("Edge", "Screw"):
        for sign in (1, -1):
            for psi, az in ((np.pi / 4, 0.0), (0.3, 30.0), (1.1, -75.0)):
                built.append(threading_segment(kind, sign, x.b_mag, 4.0e10,
                                               psi, 0.3e-6, -0.2e-6, az))
    for depth in (None, 3e-6):
        for sign in (1, -1):
            built.append(edge_segment(sign, _Slab, x.b_mag, depth))
    out["builders"] = np.array([np.concatenate([np.asarray(q, float)
                                                for q in b[0]])
                                for b in built])
    np.savez_compressed(os.path.join(HERE, "host_rows.npz"),
                        cache_keys=np.array(keys), seg=np.array(
                            [np.concatenate([np.asarray(q, float)
                                             for q in seg[0]])]),
                        cond_a=a, cond_w=wa, gh_offs=offs, gh_w=wo, **out)


def bragg_config1_golden():
    """The plain Bragg configuration at its own size, from the reference's
    NumPy solver: diamond (400) at 17 keV, t = 20 um, dx = 0.5 um, half_x =
    16 um (Nz 90, Nx 456); one edge dislocation (line [101], b = (a/2)[10-1],
    through the column at depth t/2, half-length 800 um); 21 deviation
    parameters evenly over +-3 Darwin widths, y-planes at (j - 32 + 1/2) dx.

    Stored: ``solve_surface_batch(xp=np)`` (SciPy GMRES, tol 1e-10) on 4 of
    the 64 planes for 3 of the 21 deviations, with its info; the perfect
    crystal's |D_g| at the grid centre for all 21 deviations
    (``solve_surface_batch`` of no segment, plane y = 0); and the
    finite-thickness Riccati reflectivity at 20 um for the same
    deviations."""
    from bragg import (BraggConfig, bragg_g_vector, darwin_width_urad,
                       reflectivity_riccati, solve_surface_batch)
    from crystal import DIAMOND, CrystalParams
    from dislocations import burgers_vector, straight_segment
    from units import deviation_from_urad
    x = CrystalParams.from_reflection(DIAMOND, (4, 0, 0), 17.0,
                                      f_prime=0.003, f_dprime=0.002,
                                      label="Diamond(400)")
    cfg = BraggConfig(x, t_crystal=20e-6, dx=0.5e-6, half_x=16e-6)
    g = bragg_g_vector(x)
    b = burgers_vector(np.eye(3), [1, 0, -1], x.b_mag, +1)
    seg = straight_segment(np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0), b,
                           [0.0, 0.0, cfg.t_crystal / 2], 800e-6)
    w = darwin_width_urad(x)
    urad = np.linspace(-3 * w, 3 * w, 21)
    s_all = deviation_from_urad(urad, x)
    ys_all = (np.arange(64) - 32 + 0.5) * cfg.dx
    s_pick = np.array([2, 10, 17])
    y_pick = np.array([0, 21, 32, 63])
    surface, resid, iters = [], [], []
    for k in s_pick:
        out, info = solve_surface_batch(seg, float(s_all[k]), cfg,
                                        ys_all[y_pick], x, g, xp=np)
        assert info["converged"], info
        surface.append(out)
        resid.append(info["residual"])
        iters.append(info["iterations"])
    centre = []
    for sd in s_all:
        out, info = solve_surface_batch([], float(sd), cfg, np.array([0.0]),
                                        x, g, xp=np)
        assert info["converged"], info
        centre.append(abs(out[0, cfg.Nx // 2]))
    np.savez_compressed(
        os.path.join(HERE, "bragg_cfg1.npz"),
        cfg=np.array([20e-6, 0.5e-6, 16e-6, cfg.Nz, cfg.Nx, cfg.dz, cfg.ds]),
        segs=np.array([np.concatenate([np.asarray(q, float)
                                       for q in seg[0]])]),
        g=g, urad=urad, s_dev=s_all, ys=ys_all, s_pick=s_pick,
        y_pick=y_pick, surface=np.array(surface), residual=np.array(resid),
        iterations=np.array(iters), pristine_centre=np.array(centre),
        riccati_20um=reflectivity_riccati(s_all, cfg.t_crystal, x))


def bragg_thick_golden():
    """Where the reference's Bragg solve stops converging: one plane of a
    100 um and of a 200 um slab (dx = 0.5 um, a 16-px field: Nz 447 / 894,
    Nx 1852 / 3640) with 16 seeded <110> segments in the slab (the segment
    generator of the batched configuration), s = 0.  Stored: the reference's
    ``solve_surface_batch(xp=np)`` info with its default budget (tol 1e-10,
    restart 40, maxiter 25, accept 1e-7)."""
    from bragg import BraggConfig, bragg_g_vector, solve_surface_batch
    from crystal import DIAMOND, CrystalParams
    from dyfox_gb300.workloads import _segments_in_box
    x = CrystalParams.from_reflection(DIAMOND, (4, 0, 0), 17.0,
                                      f_prime=0.003, f_dprime=0.002,
                                      label="Diamond(400)")
    g = bragg_g_vector(x)
    dx = 0.5e-6
    rows = {}
    for name, t in (("t100", 100e-6), ("t200", 200e-6)):
        cfg = BraggConfig(x, t_crystal=t, dx=dx, half_x=16 * dx)
        segs = _segments_in_box(x, np.random.default_rng(3), 16, 16 * dx,
                                dx, 0.0, cfg.t_crystal)
        _, info = solve_surface_batch(segs, 0.0, cfg, np.array([0.25 * dx]),
                                      x, g, xp=np)
        rows[name + "_cfg"] = np.array([t, dx, 16 * dx, cfg.Nz, cfg.Nx])
        rows[name + "_segs"] = np.array([np.concatenate(
            [np.asarray(q, float) for q in s]) for s in segs])
        rows[name + "_info"] = np.array([info["residual"],
                                         info["iterations"],
                                         float(info["converged"])])
    np.savez_compressed(os.path.join(HERE, "bragg_thick.npz"), y=0.25 * dx,
                        **rows)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--only", choices=["optics", "host_rows", "bragg_cfg1",
                                       "bragg_thick"],
                    default=None, help="write only this fixture")
    args = ap.parse_args()
    sys.dont_write_bytecode = True
    sys.path.insert(0, ROOT)
    sys.path.insert(0, args.reference)
    if args.only == "optics":
        optics_golden()
        print("optics fixture written to", HERE)
        return
    if args.only == "host_rows":
        host_rows_golden()
        print("host_rows fixture written to", HERE)
        return
    if args.only == "bragg_cfg1":
        bragg_config1_golden()
        print("bragg_cfg1 fixture written to", HERE)
        return
    if args.only == "bragg_thick":
        bragg_thick_golden()
        print("bragg_thick fixture written to", HERE)
        return
    import subprocess
    subprocess.check_call([sys.executable, os.path.join(ROOT, "oracle",
                                                        "make_ref.py"),
                           "--reference", args.reference])
    from oracle import oracle as O
    O.build()

    from bragg import (BraggConfig, bragg_g_vector, darwin_width_urad,
                       perfect_symbol, reflectivity_riccati,
                       reflectivity_semi_infinite, solve_bragg_stable,
                       solve_surface_batch, threading_segment)
    from bragg.solver import _march_down
    from crystal import DIAMOND, CrystalParams
    from dislocations import (H_plane, analytic_line_params, burgers_vector,
                              straight_segment, volterra_frame)
    from laue import LaueGrid
    from units import deviation_from_urad

    x = CrystalParams.from_reflection(DIAMOND, (4, 0, 0), 17.0,
                                      f_prime=0.003, f_dprime=0.002,
                                      label="Diamond(400)")
    urads = np.array([0.0, 117.5, -300.0, 300.0, -6.5])
    np.savez_compressed(os.path.join(HERE, "crystal.npz"),
             sig0=x.sig0, sig_h=x.sig_h, sig_hbar=x.sig_hbar, lam=x.lam,
             theta_B=x.theta_B, tan_tB=x.tan_tB, cos_tB=x.cos_tB,
             sin_tB=x.sin_tB, sin_2tB=x.sin_2tB, xi_g=x.xi_g, g_vec=x.g_vec,
             b_mag=x.b_mag, a_core=x.a_core, nu=x.nu, F_g=x.F_g,
             urads=urads, s_dev=deviation_from_urad(urads, x),
             darwin_urad=darwin_width_urad(x))

    # --------------------------------------------------------------- grids
    laue_cases = [  # t, dx, bw, bt, sigma, Nz, pad
        (40e-6, 0.25e-6, 8e-6, 1e-6, 0.0, None, 30),
        (200e-6, 0.25e-6, 120e-6, 1e-6, 0.0, None, 30),
        (273e-6, 0.25e-6, 120e-6, 1e-6, 0.0, None, 30),
        (273.4037251665087e-6, 0.25e-6, 120e-6, 1e-6, 0.0, None, 30),
        (400e-6, 0.125e-6, 53e-6, 1e-6, 0.5e-6, None, 14),
        (40e-6, 0.25e-6, 8e-6, 1e-6, 0.0, 301, 30),
        (20e-6, 0.25e-6, 40e-6, 1e-6, 0.0, 101, 30),
    ]
    rows = []
    for t, dx, bw, bt, sig, nz, pad in laue_cases:
        g = LaueGrid(x, t, dx, bw, beam_thickness=bt, beam_sigma=sig, Nz=nz,
                     grid_pad=pad)
        Nx, Ny, dz, ds, sp = g.geometry()
        rows.append([t, dx, bw, bt, sig, -1 if nz is None else nz, pad,
                     Nx, Ny, g.Nz, dz, ds, sp, g.t_crystal, float(g.exact),
                     g.sheet_arg()])
    bragg_cases = [(20e-6, 0.5e-6, 16e-6), (30e-6, 0.05e-6, 12e-6),
                   (6e-6, 0.1e-6, 3e-6), (100e-6, 0.25e-6, 32e-6)]
    brows = []
    for t, dx, hx in bragg_cases:
        c = BraggConfig(x, t_crystal=t, dx=dx, half_x=hx)
        brows.append([t, dx, hx, c.Nz, c.Nx, c.dz, c.ds, c.t_crystal])
    np.savez_compressed(os.path.join(HERE, "grids.npz"), laue=np.array(rows),
             bragg=np.array(brows))

    # ------------------------------------------------------------ Volterra
    small = LaueGrid(x, 40e-6, 0.25e-6, 8e-6, beam_thickness=1e-6)
    Nx, Ny, dz, ds, sp = small.geometry()
    Nz = small.Nz
    z0 = small.t_crystal / 2
    xi_n = np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0)
    b_n = burgers_vector(np.eye(3), [1, 0, -1], x.b_mag, +1)
    seg_n = straight_segment(xi_n, b_n, [-z0 * x.tan_tB, 0.0, z0], 400e-6)
    b_x = burgers_vector(np.eye(3), [1, 1, 0], x.b_mag, +1)
    seg_x = straight_segment([1.0, 0.0, 0.0], b_x,
                             [0.0, small.dx / 2, small.t_crystal / 2], 400e-6)
    rng = np.random.default_rng(20260909)
    dirs = np.array([v for v in [[1, 1, 0], [1, -1, 0], [1, 0, 1],
                                 [1, 0, -1], [0, 1, 1], [0, 1, -1]]], float)
    seg_r = []
    for _ in range(5):
        xi = dirs[rng.integers(6)] * rng.choice([-1, 1])
        xi = xi / np.linalg.norm(xi)
        b = dirs[rng.integers(6)] * rng.choice([-1, 1])
        b = x.b_mag * b / np.linalg.norm(b)
        c = np.array([rng.uniform(-10e-6, 10e-6), rng.uniform(-3e-6, 3e-6),
                      rng.uniform(5e-6, 35e-6)])
        seg_r += straight_segment(xi, b, c, rng.uniform(10e-6, 400e-6))
    screw = straight_segment(xi_n, x.b_mag * xi_n, [0.0, 0.3e-6, 20e-6],
                             100e-6)
    sets = {"n": seg_n, "x": seg_x, "r": seg_r, "screw": screw,
            "zero": [(seg_n[0][0], seg_n[0][1], np.zeros(3))]}

    class Cfg:
        pass

    cfg = Cfg()
    cfg.Nx, cfg.Nz, cfg.dx, cfg.dz = Nx, Nz, small.dx, dz
    vol = {}
    y_planes = np.array([(Ny // 2 + 3 - Ny / 2) * small.dx, 1.1e-6])
    for name, sl in sets.items():
        arr = np.array([np.concatenate([np.asarray(v, float) for v in s])
                        for s in sl])
        vol[f"segs_{name}"] = arr
        frames = []
        for (ra, rb, bv) in sl:
            t = rb - ra
            xi = t / np.linalg.norm(t)
            bs, bp, e1, e2 = volterra_frame(xi, bv)
            frames.append(np.concatenate([[bs, bp], e1, e2]))
        vol[f"frames_{name}"] = np.array(frames)
        vol[f"H_{name}"] = np.stack([H_plane(sl, cfg, x.g_vec, x.nu,
                                             x.a_core, xp=np, y_plane=y)
                                     for y in y_planes])
    ap_x = analytic_line_params(seg_x, x)
    vol["analytic_x"] = O.analytic_vector(ap_x)
    np.savez_compressed(os.path.join(HERE, "volterra.npz"), y_planes=y_planes,
             Nx=Nx, Nz=Nz, dx=small.dx, dz=dz, **vol)

    # -------------------------------------------------- Laue (reference CUDA)
    geo = dict(Nx=Nx, Ny=Ny, Nz=Nz, dz=dz, ds=ds, shift_px=sp, dx=small.dx,
               sheet_hw=small.sheet_arg(), fov_hy=small.beam_width / 2)
    s = deviation_from_urad(np.array([0.0, 117.5, -300.0]), x)
    keep = np.arange(Ny // 2 - 4, Ny // 2 + 4)
    y_all = (np.arange(Ny) - Ny / 2) * small.dx
    H_full = np.stack([H_plane(seg_n, cfg, x.g_vec, x.nu, x.a_core, xp=np,
                               y_plane=float(y)) for y in y_all])
    laue = dict(s_dev=s, rows=keep)
    laue["fullfield"] = O.ref_laue_march("fullfield", x, s, geo, H_grid=H_full,
                                         rows=keep)
    laue["fullfield_f32"] = O.ref_laue_march("fullfield", x, s, geo,
                                             H_grid=H_full, rows=keep,
                                             fp32=True)
    laue["pristine"] = O.ref_laue_march("pristine", x, s, geo, rows=keep)
    laue["analytic"] = O.ref_laue_march("analytic", x, s, geo,
                                        an=O.analytic_vector(ap_x), rows=keep)
    # An interpolating grid (Nz forced): bilinear transport.
    gi = LaueGrid(x, 40e-6, 0.25e-6, 8e-6, beam_thickness=1e-6, Nz=301)
    Nxi, Nyi, dzi, dsi, spi = gi.geometry()
    geoi = dict(Nx=Nxi, Ny=Nyi, Nz=gi.Nz, dz=dzi, ds=dsi, shift_px=spi,
                dx=gi.dx, sheet_hw=gi.sheet_arg(), fov_hy=gi.beam_width / 2)
    laue["interp_pristine"] = O.ref_laue_march("pristine", x, s, geoi,
                                               rows=keep)
    laue["interp_geo"] = np.array([Nxi, Nyi, gi.Nz, dzi, dsi, spi])
    np.savez_compressed(os.path.join(HERE, "laue_small.npz"), **laue)

    # --------------------------------------------------------------- Bragg
    g = bragg_g_vector(x)
    bc = BraggConfig(x, t_crystal=6e-6, dx=0.1e-6, half_x=3e-6)
    sd = float(deviation_from_urad(-6.5, x))
    seg_b = threading_segment("Edge", +1, x.b_mag, float(g[2]))
    Hb = H_plane(seg_b, bc, g, x.nu, x.a_core, xp=np, y_plane=0.0)
    Ch = (complex(x.sig_h) * np.exp(-1j * Hb)).astype(np.complex128)
    Cb = (complex(x.sig_hbar) * np.exp(+1j * Hb)).astype(np.complex128)
    alpha = -2.0 * np.pi * sd
    e0 = complex(np.exp(complex(x.sig0) * bc.ds))
    eg = complex(np.exp((complex(x.sig0) + 1j * alpha) * bc.ds))
    inc = bc.incident(xp=np, n=1)[0]
    zero = np.zeros(bc.Nx, complex)
    d = _march_down(inc, zero, Ch, Cb, e0, eg, bc.ds, bc.Nz, np)
    v = rng.normal(size=bc.Nx) + 1j * rng.normal(size=bc.Nx)
    Av = _march_down(zero, v, Ch, Cb, e0, eg, bc.ds, bc.Nz, np)
    T21, T22 = perfect_symbol(e0, eg, bc.ds, bc.Nz, bc.Nx, x)
    ew, info = solve_bragg_stable(seg_b, sd, bc, x, g, xp=np)
    ew0, info0 = solve_bragg_stable([], sd, bc, x, g, xp=np)
    ys = np.array([-0.2e-6, 0.0, 0.3e-6])
    sb, sinfo = solve_surface_batch(seg_b, sd, bc, ys, x, g, xp=np)
    urad_r = np.array([-6.5, -3.0, 1.0])
    sd_r = deviation_from_urad(urad_r, x)
    np.savez_compressed(os.path.join(HERE, "bragg_small.npz"),
             cfg=np.array([6e-6, 0.1e-6, 3e-6, bc.Nz, bc.Nx, bc.dz, bc.ds]),
             s_dev=sd, segs=np.array([np.concatenate(
                 [np.asarray(q, float) for q in seg_b[0]])]), g=g,
             H_row0=Hb[0],
             d=d, v=v, Av=Av, T21=T21, T22=T22, exit_wave=ew,
             gmres_code=info["gmres_code"], iterations=info["iterations"],
             residual=info["residual"], exit_wave_pristine=ew0,
             ys=ys, surface=sb, surface_residual=sinfo["residual"],
             riccati_urad=urad_r,
             riccati_6um=reflectivity_riccati(sd_r, bc.t_crystal, x),
             semi_inf=reflectivity_semi_infinite(sd_r, x))
    optics_golden()
    host_rows_golden()
    bragg_config1_golden()
    bragg_thick_golden()
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
