"""Seeded synthetic instances of the benchmark configurations.

Each function returns the inputs of one configuration as plain objects
(crystal, grid, segments, deviation parameters, ...).  The geometry follows
the configuration text; where it leaves a choice open, the rule taken is
written in the docstring.

    laue_readme()        Laue drop-in at the README size
    laue_rocking_scan()  256-angle rocking scan over 64 random segments
    bragg_config1()      21 deviation parameters x 64 planes, one edge
    random_110_segments  the segment generator of the scan configurations
"""

import numpy as np

from .bragg_geometry import BraggConfig, bragg_g_vector, darwin_width_urad
from .crystal import diamond_400
from .dislocations import burgers_vector, straight_segment
from .grid import LaueGrid
from .units import deviation_from_urad

SEED = 20260909

# The 12 signed <110> directions.
DIRS_110 = np.array([[s1, s2, 0] for s1 in (1, -1) for s2 in (1, -1)]
                    + [[s1, 0, s2] for s1 in (1, -1) for s2 in (1, -1)]
                    + [[0, s1, s2] for s1 in (1, -1) for s2 in (1, -1)],
                    dtype=float)


def random_110_segments(xtal, grid, n, rng, near_surface=None):
    """n straight segments in the illuminated volume of a Laue grid.

    * line direction: uniform over the 12 signed <110>;
    * Burgers vector (a/2)<110> with a random sign: with probability 1/2
      one of the <110> perpendicular to the line (pure edge), otherwise any
      of the 12 (mixed or screw);
    * midpoint uniform over x in [-t tan(theta_B), t tan(theta_B)],
      |y| < beam_width / 2, z in [0, t] (z in [0, near_surface] when given);
    * length L log-uniform on [20, 800] um, half-length L / 2.
    """
    t = grid.t_crystal
    segs = []
    for _ in range(n):
        xi = DIRS_110[rng.integers(12)]
        if rng.random() < 0.5:
            perp = DIRS_110[np.abs(DIRS_110 @ xi) < 1e-12]
            b = perp[rng.integers(len(perp))]
        else:
            b = DIRS_110[rng.integers(12)]
        b = rng.choice([-1.0, 1.0]) * xtal.b_mag * b / np.linalg.norm(b)
        zmax = t if near_surface is None else near_surface
        c = [rng.uniform(-t * xtal.tan_tB, t * xtal.tan_tB),
             rng.uniform(-grid.beam_width / 2, grid.beam_width / 2),
             rng.uniform(0.0, zmax)]
        L = np.exp(rng.uniform(np.log(20e-6), np.log(800e-6)))
        segs += straight_segment(xi / np.linalg.norm(xi), b, c, L / 2)
    return segs


def laue_readme():
    """Diamond (400) 17 keV, t = 200 um, dx = 0.25 um, beam 120 um
    (544 x 800, Nz 359); one edge dislocation, line [101], b = (a/2)[10-1],
    crossing the beam column at t/2, half a pixel off the sampled rows;
    s at 0 and 117.5 urad."""
    x = diamond_400()
    grid = LaueGrid(x, t_crystal=200e-6, dx=0.25e-6, beam_width=120e-6)
    b = burgers_vector(x.U_lab, [1, 0, -1], x.b_mag, +1)
    z0 = grid.t_crystal / 2
    seg = straight_segment(np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0), b,
                           [-z0 * x.tan_tB, grid.dx / 2, z0], 800e-6)
    return x, grid, seg, deviation_from_urad([0.0, 117.5], x)


def laue_rocking_scan(n_angles=256, n_segments=64, seed=SEED):
    """Diamond (400) 17 keV, t = 273 um, dx = 0.25 um, beam 120 um
    (544 x 1056, Nz 490); 64 random <110> segments; 256 deviation
    parameters uniform on [-300, +300] urad."""
    x = diamond_400()
    grid = LaueGrid(x, t_crystal=273e-6, dx=0.25e-6, beam_width=120e-6)
    rng = np.random.default_rng(seed)
    segs = random_110_segments(x, grid, n_segments, rng)
    s = deviation_from_urad(np.linspace(-300.0, 300.0, n_angles), x)
    return x, grid, segs, s


def bragg_config1():
    """Diamond (400) 17 keV, t = 20 um, dx = 0.5 um, half_x = 16 um
    (Nz 90, Nx 456); 64 y-planes at (j - 32 + 1/2) dx; 21 deviation
    parameters evenly over +-3 Darwin widths; one edge dislocation
    (line [101], b = (a/2)[10-1]) through the column at depth t/2."""
    x = diamond_400()
    cfg = BraggConfig(x, t_crystal=20e-6, dx=0.5e-6, half_x=16e-6)
    b = burgers_vector(np.eye(3), [1, 0, -1], x.b_mag, +1)
    seg = straight_segment(np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0), b,
                           [0.0, 0.0, cfg.t_crystal / 2], 800e-6)
    w = darwin_width_urad(x)
    s = deviation_from_urad(np.linspace(-3 * w, 3 * w, 21), x)
    ys = (np.arange(64) - 32 + 0.5) * cfg.dx
    return x, cfg, seg, s, ys, bragg_g_vector(x)


# ---------------------------------------------------------------------------
# Batched uneven instances

class ExplicitLaueGrid:
    """A Laue sampling whose transverse shape (Ny x Nx) is set directly
    rather than by LaueGrid's fan rule; exact advection (dz = dx /
    tan(theta_B), Nz = round(t / dz) + 1, shift 1 px per step), top-hat
    beam of half-width ``sheet_hw`` on the entrance face, rows with
    |y| < beam_width / 2 illuminated.  The march zero-fills beyond the x
    edges, so a fan wider than Nx leaves the grid."""

    def __init__(self, xtal, t_crystal, dx, Ny, Nx, beam_width, sheet_hw):
        self.xtal = xtal
        self.dx = float(dx)
        step = self.dx / xtal.tan_tB
        self.Nz = int(round(float(t_crystal) / step)) + 1
        self.t_crystal = (self.Nz - 1) * step
        self.Ny, self.Nx = int(Ny), int(Nx)
        self.beam_width = float(beam_width)
        self.sheet_hw = float(sheet_hw)

    def geometry(self):
        dz = self.t_crystal / (self.Nz - 1)
        return self.Nx, self.Ny, dz, dz / self.xtal.cos_tB, 1.0

    def sheet_arg(self):
        return self.sheet_hw

    @property
    def shape(self):
        return self.Ny, self.Nx


def _loguniform_int(rng, lo, hi):
    return int(min(hi, max(lo, round(np.exp(rng.uniform(np.log(lo),
                                                        np.log(hi)))))))


def _segments_in_box(xtal, rng, n, half_x, half_y, z_lo, z_hi):
    """n segments of the <110> generator of ``random_110_segments`` with
    midpoints uniform in the box |x| < half_x, |y| < half_y,
    z in [z_lo, z_hi]."""
    segs = []
    for _ in range(n):
        xi = DIRS_110[rng.integers(12)]
        if rng.random() < 0.5:
            perp = DIRS_110[np.abs(DIRS_110 @ xi) < 1e-12]
            b = perp[rng.integers(len(perp))]
        else:
            b = DIRS_110[rng.integers(12)]
        b = rng.choice([-1.0, 1.0]) * xtal.b_mag * b / np.linalg.norm(b)
        c = [rng.uniform(-half_x, half_x), rng.uniform(-half_y, half_y),
             rng.uniform(z_lo, z_hi)]
        L = np.exp(rng.uniform(np.log(20e-6), np.log(800e-6)))
        segs += straight_segment(xi / np.linalg.norm(xi), b, c, L / 2)
    return segs


def batched_uneven(n=512, seed=SEED, laue_fraction=0.7):
    """The batched-uneven configuration: ``n`` independent instances, a
    seeded 70 / 30 mix of Laue and Bragg (exact counts), diamond (400) at
    17 keV.  Each instance is a dict with ``kind`` "laue" or "bragg".

    Laue: t uniform in [50, 400] um; dx in {0.125, 0.25, 0.5} um; Ny =
    128 2^i (i = 0..3) and Nx = 128 2^j (j = 0..min(i, 2)), i.e. 128 x 128
    up to 1024 x 512, set directly (``ExplicitLaueGrid``); 90% of the rows
    illuminated; top-hat entrance beam over the central quarter of x;
    1-128 segments (log-uniform count) of the <110> generator with
    midpoints uniform in the illuminated volume; 1-64 deviation parameters
    evenly over [-300, +300] urad.

    Bragg: t uniform in [5, 20] um (shooting through about one extinction
    length: from 40 um at dx = 0.125 um on, restarted GMRES(40) itself
    stagnates above 1e-6 in double precision, and thicker slabs make the
    shooting operator exponentially ill-conditioned); dx in {0.125, 0.25,
    0.5} um; a lateral field of 32, 64 or 128 px padded by the BraggConfig
    rule Nx = 2 (half_x / dx + 2 Nz + 16); 1-8 y-planes (log-uniform);
    1-128 segments with midpoints in the slab; 1-64 deviation parameters
    evenly over +-3 Darwin widths.
    """
    x = diamond_400()
    rng = np.random.default_rng(seed)
    n_laue = int(round(laue_fraction * n))
    kinds = np.array(["laue"] * n_laue + ["bragg"] * (n - n_laue))
    rng.shuffle(kinds)
    w = darwin_width_urad(x)
    out = []
    for kind in kinds:
        dx = float(rng.choice([0.125e-6, 0.25e-6, 0.5e-6]))
        nseg = _loguniform_int(rng, 1, 128)
        n_e = int(rng.integers(1, 65))
        if kind == "laue":
            t = rng.uniform(50e-6, 400e-6)
            i = int(rng.integers(0, 4))
            j = int(rng.integers(0, min(i, 2) + 1))
            Ny, Nx = 128 << i, 128 << j
            grid = ExplicitLaueGrid(x, t, dx, Ny, Nx, beam_width=0.9 * Ny * dx,
                                    sheet_hw=Nx * dx / 8)
            segs = _segments_in_box(x, rng, nseg, Nx * dx / 2,
                                    0.45 * Ny * dx, 0.0, grid.t_crystal)
            s = deviation_from_urad(np.linspace(-300.0, 300.0, n_e), x)
            out.append(dict(kind="laue", xtal=x, grid=grid, segs=segs, s=s))
        else:
            t = rng.uniform(5e-6, 20e-6)
            field = int(rng.choice([32, 64, 128]))
            cfg = BraggConfig(x, t_crystal=t, dx=dx, half_x=field * dx / 2)
            n_y = _loguniform_int(rng, 1, 8)
            ys = (np.arange(n_y) - n_y / 2 + 0.5) * dx
            segs = _segments_in_box(x, rng, nseg, field * dx / 2,
                                    max(n_y, 1) * dx / 2, 0.0, cfg.t_crystal)
            s = deviation_from_urad(np.linspace(-3 * w, 3 * w, n_e), x)
            out.append(dict(kind="bragg", xtal=x, cfg=cfg, segs=segs, s=s,
                            ys=ys, g=bragg_g_vector(x)))
    return out


def learned_guess_instances(n, seed=SEED + 5, t_range=(10e-6, 100e-6),
                            n_planes=256, field=256, n_s=64,
                            max_segments=32):
    """The learned-shooting-guess configuration: ``n`` Bragg instances on
    diamond (400) at 17 keV, dx = 0.25 um; t uniform on ``t_range``; a
    lateral field of ``field`` px (half_x = field dx / 2, Nx by the
    BraggConfig rule); ``n_planes`` y-planes at (j - n/2 + 1/2) dx;
    1..``max_segments`` <110> segments (log-uniform count) with midpoints
    in the field, across the planes and within 5 um of the surface;
    ``n_s`` deviation parameters evenly over +-5 Darwin widths.  Each
    instance is a dict (xtal, cfg, segs, s, ys, g, col0, field)."""
    x = diamond_400()
    rng = np.random.default_rng(seed)
    w = darwin_width_urad(x)
    dx = 0.25e-6
    s = deviation_from_urad(np.linspace(-5 * w, 5 * w, n_s), x)
    ys = (np.arange(n_planes) - n_planes / 2 + 0.5) * dx
    out = []
    for _ in range(n):
        t = rng.uniform(*t_range)
        cfg = BraggConfig(x, t_crystal=t, dx=dx, half_x=field * dx / 2)
        nseg = _loguniform_int(rng, 1, max_segments)
        segs = _segments_in_box(x, rng, nseg, field * dx / 2,
                                n_planes * dx / 2, 0.0,
                                min(5e-6, cfg.t_crystal))
        out.append(dict(xtal=x, cfg=cfg, segs=segs, s=s.copy(), ys=ys,
                        g=bragg_g_vector(x), col0=cfg.Nx // 2 - field // 2,
                        field=field))
    return out
