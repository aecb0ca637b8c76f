"""ORACLE -- test infrastructure only.  Closed-form perfect-crystal answers.

Restatements of DYFOX's closed forms, pinned by tests/test_oracle_pins.py
against the golden vectors of tests/golden (made from the reference):

    planewave_rocking           analysis/rocking.py:16-34 (two-beam Laue)
    reflectivity_semi_infinite  bragg/reference.py:14-29 (stationary Riccati
                                root with |R| <= 1)
    reflectivity_riccati        bragg/reference.py:32-56 (Riccati ODE
                                integrated from z = t to 0, SciPy DOP853)
    darwin_width_urad           bragg/reference.py:59-67
"""

import numpy as np


def planewave_rocking(s_dev, xtal, t_crystal, absorption=True):
    """|D_g|^2 of a perfect Laue crystal: |sh|^2/gam^2 sin^2(gam s_path)
    exp(2 Re(sig0) s_path), gam^2 = |sh shbar| + alpha^2/4."""
    s_dev = np.asarray(s_dev)
    sh, sb = complex(xtal.sig_h), complex(xtal.sig_hbar)
    alpha = -2 * np.pi * s_dev
    gam = np.sqrt(np.abs(sh * sb) + alpha ** 2 / 4)
    path = t_crystal / xtal.cos_tB
    rc = np.abs(sh) ** 2 / gam ** 2 * np.sin(gam * path) ** 2
    if absorption:
        rc = rc * np.exp(2 * complex(xtal.sig0).real * path)
    return rc


def reflectivity_semi_infinite(s_dev, xtal):
    s_dev = np.atleast_1d(np.asarray(s_dev, float))
    s0, sh, sb = (complex(xtal.sig0), complex(xtal.sig_h),
                  complex(xtal.sig_hbar))
    B = 2.0 * s0 + 1j * (-2.0 * np.pi * s_dev)
    disc = np.sqrt(B ** 2 - 4.0 * sh * sb + 0j)
    r1 = (-B + disc) / (2.0 * sb)
    r2 = (-B - disc) / (2.0 * sb)
    return np.where(np.abs(r1) <= np.abs(r2), r1, r2)


def reflectivity_riccati(s_dev, t_crystal, xtal, rtol=1e-11, atol=1e-14):
    """dR/dz = -(sh + (2 s0 + i alpha) R + sb R^2) / sin(tB), R(t) = 0."""
    from scipy.integrate import solve_ivp
    s0, sh, sb = (complex(xtal.sig0), complex(xtal.sig_h),
                  complex(xtal.sig_hbar))
    out = []
    for sd in np.atleast_1d(np.asarray(s_dev, float)):
        alpha = -2.0 * np.pi * float(sd)

        def rhs(z, R):
            r = R[0] + 1j * R[1]
            d = -(sh + (2.0 * s0 + 1j * alpha) * r + sb * r * r) / xtal.sin_tB
            return [d.real, d.imag]

        with np.errstate(over="ignore", invalid="ignore", divide="ignore"):
            sol = solve_ivp(rhs, [t_crystal, 0.0], [0.0, 0.0], rtol=rtol,
                            atol=atol, method="DOP853")
        out.append(sol.y[0, -1] + 1j * sol.y[1, -1])
    return np.array(out)


def darwin_width_urad(xtal):
    sh, sb = complex(xtal.sig_h), complex(xtal.sig_hbar)
    chi = np.sqrt(sh * sb) * xtal.lam / (1j * np.pi)
    return float(2.0 * abs(chi) / xtal.sin_2tB * 1e6)
