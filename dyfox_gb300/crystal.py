"""Materials and the two-beam diffraction parameters of one reflection.

This module supplies the scalar inputs of the hot path: wavelength, Bragg
angle, the susceptibility couplings ``sig0``, ``sig_h``, ``sig_hbar``
(``sigma = -i r_e lambda F / V_cell``), the extinction length and the
reciprocal-lattice vector.  Attribute names and the constructor
``CrystalParams.from_reflection(material, hkl, E_keV, ...)`` are those of
DYFOX ``crystal.py:26-165`` so that either object can be handed to the
solvers; the solvers only read attributes.

Conventions (DYFOX ``README.md`` "Conventions" 3-4): atomic form factors
carry ``-i f''``; ``F_0`` uses the forward factor ``Z + f' - i f''``;
``F_{-g} = f * conj(S_g)``.

Restates DYFOX's crystal formulas and material table (MIT licence: see
NOTICE).
"""

from dataclasses import dataclass, replace

import numpy as np

from .units import HC_EV_M, R_E

# Fractional coordinates of the eight atoms of the diamond-cubic cell.
DIAMOND_CUBIC = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5],
                          [0.0, 0.5, 0.5], [0.25, 0.25, 0.25],
                          [0.75, 0.75, 0.25], [0.75, 0.25, 0.75],
                          [0.25, 0.75, 0.75]])


@dataclass(frozen=True)
class Material:
    """A cubic substance: lattice parameter, basis, Z, Poisson ratio, f0.

    ``burgers_mag`` defaults to |(a/2)<110>| and ``core_radius`` (where the
    Volterra field is regularised) to one Burgers vector.
    """

    name: str
    a_lat: float
    basis: np.ndarray
    Z: float
    nu: float
    f0: dict
    burgers_mag: float = None
    core_radius: float = None

    def burgers(self):
        if self.burgers_mag is not None:
            return self.burgers_mag
        return self.a_lat * np.sqrt(2) / 2

    def core(self):
        if self.core_radius is not None:
            return self.core_radius
        return self.burgers()


DIAMOND = Material(name="diamond", a_lat=3.567e-10, basis=DIAMOND_CUBIC,
                   Z=6.0, nu=0.069,
                   f0={(4, 0, 0): 1.589, (2, 2, 0): 1.961})


def lab_frame(normal_hkl, g_hkl):
    """Rows (x, y, z) of a right-handed lab frame: z along the surface
    normal, x along g projected into the surface."""
    z = np.asarray(normal_hkl, float)
    z = z / np.linalg.norm(z)
    g = np.asarray(g_hkl, float)
    x = g - np.dot(g, z) * z
    if np.linalg.norm(x) < 1e-12:
        raise ValueError("g is parallel to the surface normal (a Bragg "
                         "geometry, not symmetric Laue)")
    x = x / np.linalg.norm(x)
    return np.array([x, np.cross(z, x), z])


@dataclass(frozen=True)
class CrystalParams:
    """A material, a reflection and a photon energy, worked through."""

    material: Material
    hkl: tuple
    E_keV: float
    U_lab: np.ndarray
    label: str
    lam: float
    d_hkl: float
    theta_B: float
    F_g: complex
    sig0: complex
    sig_h: complex
    sig_hbar: complex
    xi_g: float
    sin_tB: float
    cos_tB: float
    tan_tB: float
    sin_2tB: float
    a_lat: float
    nu: float
    g_vec: np.ndarray
    b_mag: float
    a_core: float

    @classmethod
    def from_reflection(cls, material, hkl, E_keV, U_lab=None, f0=None,
                        f_prime=0.0, f_dprime=0.0, label=None):
        hkl = tuple(int(h) for h in hkl)
        ghkl = np.array(hkl)
        U = np.eye(3) if U_lab is None else U_lab
        if f0 is None:
            if hkl not in material.f0:
                raise KeyError(f"{material.name} has no f0 for {hkl}; pass "
                               f"f0=... (known: {sorted(material.f0)})")
            f0 = material.f0[hkl]
        a = material.a_lat
        lam = HC_EV_M / (E_keV * 1e3)
        d = a / np.sqrt(np.sum(ghkl ** 2))
        theta = np.arcsin(lam / (2 * d))
        vol = a ** 3
        f_atom = f0 + f_prime - 1j * f_dprime
        structure = np.sum(np.exp(2j * np.pi * material.basis @ ghkl))
        F0 = (material.Z + f_prime - 1j * f_dprime) * len(material.basis)
        Fg = f_atom * structure
        Fmg = f_atom * np.conj(structure)
        # sigma = -i r_e lambda F / V, evaluated left to right.
        sig = [-1j * R_E * lam * F / vol for F in (F0, Fg, Fmg)]
        if label is None:
            label = (f"{material.name.capitalize()}"
                     f"({''.join(str(h) for h in hkl)})")
        return cls(material=material, hkl=hkl, E_keV=float(E_keV), U_lab=U,
                   label=label, lam=lam, d_hkl=d, theta_B=theta, F_g=Fg,
                   sig0=sig[0], sig_h=sig[1], sig_hbar=sig[2],
                   xi_g=np.pi / abs(sig[1]), sin_tB=np.sin(theta),
                   cos_tB=np.cos(theta), tan_tB=np.tan(theta),
                   sin_2tB=np.sin(2 * theta), a_lat=a, nu=material.nu,
                   g_vec=U @ (ghkl / a), b_mag=material.burgers(),
                   a_core=material.core())

    def at_energy(self, E_keV, **kw):
        return CrystalParams.from_reflection(self.material, self.hkl, E_keV,
                                             U_lab=self.U_lab,
                                             label=self.label, **kw)

    def with_frame(self, U_lab):
        U = np.asarray(U_lab, float)
        return replace(self, U_lab=U, g_vec=U @ (np.array(self.hkl)
                                                 / self.a_lat))

    def key(self):
        return {"material": self.material.name, "hkl": list(self.hkl),
                "E_keV": self.E_keV, "label": self.label}

    def __getitem__(self, name):
        return getattr(self, name)


def diamond_400(E_keV=17.0, f_prime=0.003, f_dprime=0.002):
    """Diamond (4,0,0), the crystal of every benchmark configuration."""
    return CrystalParams.from_reflection(DIAMOND, (4, 0, 0), E_keV,
                                         f_prime=f_prime, f_dprime=f_dprime,
                                         label="Diamond(400)")
