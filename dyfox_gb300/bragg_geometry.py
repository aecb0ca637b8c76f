"""Grid of a symmetric-Bragg (reflection) solve and segment builders.

``BraggConfig`` keeps the constructor and the sizing rules of DYFOX
``bragg/geometry.py:23-67`` (the returned surface wave lives on this grid):
``dz = dx tan(theta_B)`` (one pixel of lateral walk per depth step),
``Nz = round(t / dz) + 1`` with the thickness snapped to ``(Nz - 1) dz``,
a periodic lateral grid ``Nx = 2 (round(half_x / dx) + 2 Nz + 16)`` padded
past the round-trip walk, and ``ds = dz / sin(theta_B)``.
``bragg_g_vector`` puts g along the surface normal (``geometry.py:18-20``).

BraggConfig restates DYFOX's sizing rules (MIT licence: see NOTICE).
"""

import numpy as np


def bragg_g_vector(xtal):
    """g along the surface normal with the reflection's magnitude."""
    return np.array([0.0, 0.0, float(np.linalg.norm(xtal.g_vec))])


class BraggConfig:
    """Sampling of one symmetric-Bragg solve."""

    def __init__(self, xtal, t_crystal=30e-6, dx=0.05e-6, half_x=12e-6,
                 beam_thickness=None, beam_centre=0.0):
        self.xtal = xtal
        self.dx = float(dx)
        self.dz = float(dx) * xtal.tan_tB
        self.Nz = int(round(float(t_crystal) / self.dz)) + 1
        self.t_crystal = (self.Nz - 1) * self.dz
        self.half_x = float(half_x)
        self.Nx = int(2 * (round(half_x / self.dx) + 2 * self.Nz + 16))
        self.ds = self.dz / xtal.sin_tB
        self.beam_thickness = beam_thickness
        self.beam_centre = float(beam_centre)

    def incident(self, xp=np, n=1):
        """D_0 on the entrance face, shape (n, Nx): ones (plane wave) or a
        top hat of width ``beam_thickness`` about ``beam_centre``."""
        if self.beam_thickness is None:
            return xp.ones((n, self.Nx), dtype=xp.complex128)
        x = (xp.arange(self.Nx) - self.Nx / 2) * self.dx
        top = (xp.abs(x - self.beam_centre)
               < 0.5 * self.beam_thickness).astype(xp.complex128)
        return xp.broadcast_to(top, (n, self.Nx)).copy()

    def x_axis(self):
        return (np.arange(self.Nx) - self.Nx / 2) * self.dx

    def z_axis(self):
        return np.arange(self.Nz) * self.dz

    def __repr__(self):
        return (f"BraggConfig(t={self.t_crystal * 1e6:.2f}um, "
                f"dx={self.dx * 1e9:.0f}nm, dz={self.dz * 1e9:.0f}nm, "
                f"Nz={self.Nz}, Nx={self.Nx})")


def _line(core, direction, half_length, burgers):
    """One straight segment (r_start, r_end, b) centred on ``core``."""
    core = np.asarray(core, float)
    reach = half_length * np.asarray(direction, float)
    return [(core - reach, core + reach, np.asarray(burgers, float))]


def edge_segment(sign, cfg, b_mag, depth=None):
    """An edge dislocation parallel to the surface, across the plane of
    incidence: the line runs along y (half-length 400 um) through
    (0, 0, depth), by default a quarter of the slab down; b of length
    ``b_mag`` lies in the (x, z) plane at 45 degrees to the surface
    normal, so g.b = |g| |b| / sqrt 2 for g along the normal (2 for
    diamond (400)).  ``sign`` flips b (DYFOX bragg/geometry.py:69-81)."""
    z_core = 0.25 * cfg.t_crystal if depth is None else depth
    b = (sign * b_mag / np.sqrt(2.0)) * np.array([1.0, 0.0, 1.0])
    return _line([0.0, 0.0, z_core], [0.0, 1.0, 0.0], 400e-6, b)


def threading_segment(kind, sign, b_mag, g_mag, psi=np.pi / 4, y0=0.0,
                      x0=0.0, azimuth_deg=0.0):
    """A dislocation threading the surface at (x0, y0, 0), half-length
    300 um (DYFOX bragg/geometry.py:83-109).

    Line: tilted by ``psi`` from the surface normal towards +y, then turned
    by ``azimuth_deg`` about the normal (out of the plane of incidence).
    Burgers vector for g along the normal (|g| = ``g_mag``), scaled by
    ``sign``: "Screw" -- b_mag along the line; otherwise (edge) -- the
    normal component fixed by g.b = 2 (b_z = 2 / g_mag), the y component
    making b normal to the untilted-in-azimuth line (b_y = -b_z / tan psi),
    and the x component taking what is left of |b| = b_mag (zero if
    nothing is left).  The edge vector is built for the line before the
    azimuth turn."""
    line = np.array([0.0, np.sin(psi), np.cos(psi)])
    if azimuth_deg:
        phi = np.radians(azimuth_deg)
        turn = np.array([[np.cos(phi), -np.sin(phi), 0.0],
                         [np.sin(phi), np.cos(phi), 0.0],
                         [0.0, 0.0, 1.0]])
        line = np.array([turn[0, 0] * line[0] + turn[0, 1] * line[1],
                         turn[1, 0] * line[0] + turn[1, 1] * line[1],
                         line[2]])
    if kind == "Screw":
        b = sign * b_mag * line
    else:
        b_z = 2.0 / g_mag
        b_y = -b_z / np.tan(psi)
        b_x = np.sqrt(max(b_mag ** 2 - b_z ** 2 - b_y ** 2, 0.0))
        b = sign * np.array([b_x, b_y, b_z])
    return _line([x0, y0, 0.0], line, 300e-6, b)


def darwin_width_urad(xtal):
    """Full width (urad) of the symmetric-Bragg total-reflection domain:
    2 |sqrt(chi_h chi_hbar)| / sin(2 theta_B), with chi = lambda sigma /
    (i pi) (DYFOX bragg/reference.py:59-67)."""
    sh, sb = complex(xtal.sig_h), complex(xtal.sig_hbar)
    chi = np.sqrt(sh * sb) * xtal.lam / (1j * np.pi)
    return float(2.0 * abs(chi) / xtal.sin_2tB * 1e6)
