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
