"""Grid of a symmetric-Bragg (reflection) solve and segment builders.

``BraggConfig`` keeps the constructor and the sizing rules of DYFOX
``bragg/geometry.py:23-67`` (the returned surface wave lives on this grid):
``dz = dx tan(theta_B)`` (one pixel of lateral walk per depth step),
``Nz = round(t / dz) + 1`` with the thickness snapped to ``(Nz - 1) dz``,
a periodic lateral grid ``Nx = 2 (round(half_x / dx) + 2 Nz + 16)`` padded
past the round-trip walk, and ``ds = dz / sin(theta_B)``.
``bragg_g_vector`` puts g along the surface normal (``geometry.py:18-20``).
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


def edge_segment(sign, cfg, b_mag, depth=None):
    """Edge dislocation along y with b at 45 degrees in the (x, z) plane."""
    depth = cfg.t_crystal * 0.25 if depth is None else depth
    xi = np.array([0.0, 1.0, 0.0])
    bv = sign * b_mag * np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0)
    core = np.array([0.0, 0.0, depth])
    half = 400e-6
    return [(core - half * xi, core + half * xi, bv)]


def threading_segment(kind, sign, b_mag, g_mag, psi=np.pi / 4, y0=0.0,
                      x0=0.0, azimuth_deg=0.0):
    """A dislocation threading the surface at ``psi`` from the normal, with
    g.b = 2 sign for g along the normal (edge or screw)."""
    xi = np.array([0.0, np.sin(psi), np.cos(psi)])
    if azimuth_deg:
        c, s = np.cos(np.radians(azimuth_deg)), np.sin(np.radians(azimuth_deg))
        xi = np.array([c * xi[0] - s * xi[1], s * xi[0] + c * xi[1], xi[2]])
    bz = 2.0 / g_mag
    if kind == "Screw":
        bv = sign * b_mag * xi
    else:
        by = -bz / np.tan(psi)
        bx = np.sqrt(max(b_mag ** 2 - bz ** 2 - by ** 2, 0.0))
        bv = sign * np.array([bx, by, bz])
    core = np.array([x0, y0, 0.0])
    half = 300e-6
    return [(core - half * xi, core + half * xi, bv)]


def darwin_width_urad(xtal):
    """Full width (urad) of the symmetric-Bragg total-reflection domain:
    2 |sqrt(chi_h chi_hbar)| / sin(2 theta_B), with chi = lambda sigma /
    (i pi) (DYFOX bragg/reference.py:59-67)."""
    sh, sb = complex(xtal.sig_h), complex(xtal.sig_hbar)
    chi = np.sqrt(sh * sb) * xtal.lam / (1j * np.pi)
    return float(2.0 * abs(chi) / xtal.sin_2tB * 1e6)
