"""Physical constants and the rocking-angle <-> deviation-parameter maps.

Interface and constants follow DYFOX ``units.py:13-38``: the deviation
parameter is ``s = phi * sin(2 theta_B) / lambda`` (1/m) for a rocking angle
``phi`` in radians.  Crystal parameters may be given as an object with
attributes or as a mapping.

Restates DYFOX's interface and formulas (MIT licence: see NOTICE).
"""

import numpy as np

R_E = 2.8179403262e-15          # classical electron radius (m)
HC_EV_M = 12398.419e-10         # h*c in eV*m


def param(xtal, key):
    """Crystal parameter ``key`` from a mapping or an attribute holder."""
    try:
        return xtal[key]
    except (TypeError, IndexError, KeyError):
        return getattr(xtal, key)


def deviation_from_rad(phi, xtal):
    """Deviation parameter (1/m) for a rocking angle in radians."""
    return np.asarray(phi) * param(xtal, "sin_2tB") / param(xtal, "lam")


def deviation_from_urad(phi_urad, xtal):
    """Deviation parameter (1/m) for a rocking angle in microradians."""
    return (np.asarray(phi_urad) * 1e-6 * param(xtal, "sin_2tB")
            / param(xtal, "lam"))


def urad_from_deviation(s_dev, xtal):
    """Rocking angle (microradians) for a deviation parameter (1/m)."""
    return (np.asarray(s_dev) * param(xtal, "lam") / param(xtal, "sin_2tB")
            * 1e6)
