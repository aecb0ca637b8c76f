"""Sampling of a transmission (Laue) solve.

``LaueGrid(xtal, t_crystal, dx, beam_width, *, beam_thickness, beam_sigma,
Nz, grid_pad)`` keeps the interface and the sizing rules of DYFOX
``laue/grid.py:21-115`` because the grid shape is part of the drop-in
contract (the exit wave is returned on it):

* depth step ``dz = dx / tan(theta_B)`` unless ``Nz`` is forced, so a
  characteristic advances exactly one pixel per step; the thickness snaps to
  ``(Nz - 1) * dz``;
* ``Nx`` covers the sheet, twice the Borrmann fan and ``grid_pad`` pixels of
  margin on each side (at least 128), ``Ny`` the beam width plus margin (at
  least 64); both are rounded up to multiples of 32;
* ``ds = dz / cos(theta_B)``; ``shift_px = tan(theta_B) dz / dx`` snapped to
  the nearest integer when within 1e-9 of it.

Restates DYFOX's LaueGrid sizing rules (MIT licence: see NOTICE).
"""

import numpy as np


class LaueGrid:
    """Grid and beam settings for one Laue solve."""

    def __init__(self, xtal, t_crystal, dx, beam_width, *,
                 beam_thickness=1.0e-6, beam_sigma=0.0, Nz=None,
                 grid_pad=30):
        self.xtal = xtal
        self.beam_thickness = float(beam_thickness)
        self.beam_sigma = float(beam_sigma)
        self.dx = float(dx)
        self.beam_width = float(beam_width)
        self.grid_pad = int(grid_pad)
        if Nz is None:
            step = self.dx / xtal.tan_tB
            self.Nz = int(round(float(t_crystal) / step)) + 1
            self.t_crystal = (self.Nz - 1) * step
            self.exact = True
        else:
            self.Nz = int(Nz)
            self.t_crystal = float(t_crystal)
            step = self.t_crystal / (self.Nz - 1)
            self.exact = abs(xtal.tan_tB * step / self.dx - 1.0) < 1e-9

    def replace(self, **kw):
        """A copy with some settings changed (a forced Nz is kept)."""
        base = dict(xtal=self.xtal, t_crystal=self.t_crystal, dx=self.dx,
                    beam_width=self.beam_width,
                    beam_thickness=self.beam_thickness,
                    beam_sigma=self.beam_sigma, grid_pad=self.grid_pad)
        if "Nz" not in kw and not self.exact:
            base["Nz"] = self.Nz
        base.update(kw)
        return LaueGrid(**base)

    def sheet_arg(self):
        """Beam argument of the march: top-hat half-width, or -sigma for a
        Gaussian amplitude profile."""
        if self.beam_sigma > 0:
            return -self.beam_sigma
        return self.beam_thickness / 2.0

    def geometry(self):
        """``(Nx, Ny, dz, ds, shift_px)``."""
        x = self.xtal
        fan = self.t_crystal * x.tan_tB
        pad = self.grid_pad * self.dx
        sheet = (6.0 * self.beam_sigma if self.beam_sigma > 0
                 else self.beam_thickness)
        nx = max(int(np.ceil((sheet + 2 * fan + 2 * pad) / self.dx)), 128)
        nx = int(np.ceil(nx / 32)) * 32
        ny = max(int(np.ceil((self.beam_width + 2 * pad) / self.dx)), 64)
        ny = int(np.ceil(ny / 32)) * 32
        dz = self.t_crystal / (self.Nz - 1)
        ds = dz / x.cos_tB
        shift = x.tan_tB * dz / self.dx
        if abs(shift - round(shift)) < 1e-9:
            shift = float(round(shift))
        return nx, ny, dz, ds, shift

    @property
    def shape(self):
        """``(Ny, Nx)`` of one exit wave."""
        nx, ny = self.geometry()[:2]
        return ny, nx

    def key(self):
        return dict(beam_thickness=self.beam_thickness,
                    beam_sigma=self.beam_sigma, t_crystal=self.t_crystal,
                    Nz=self.Nz, dx=self.dx, beam_width=self.beam_width,
                    grid_pad=self.grid_pad)

    def __repr__(self):
        nx, ny = self.geometry()[:2]
        return (f"LaueGrid({ny}x{nx}, Nz={self.Nz}, "
                f"t={self.t_crystal * 1e6:.1f}um, dx={self.dx * 1e9:.0f}nm"
                + ("" if self.exact else ", interpolating") + ")")


def grid_arrays(grid):
    """Everything the march needs from a grid object, as plain numbers.

    Accepts this module's ``LaueGrid`` or any object with the same
    ``geometry()``, ``Nz``, ``dx``, ``beam_width`` and ``sheet_arg()``.
    """
    nx, ny, dz, ds, shift = grid.geometry()
    return dict(Nx=int(nx), Ny=int(ny), Nz=int(grid.Nz), dz=float(dz),
                ds=float(ds), shift_px=float(shift), dx=float(grid.dx),
                sheet_hw=float(grid.sheet_arg()),
                fov_hy=float(grid.beam_width / 2.0))
