"""What the single-precision march arithmetic costs, on the CPU.

``march_f32_model.c`` restates the compensated FP32 march of the library
with the phase factor taken from a double H (each voxel's e^{iH} correctly
rounded to float).  Against the double-precision oracle its exit-intensity
error is the march's own share of the FP32 error budget (1e-5 relative
L2): a few 1e-7, even over 1434 steps.  Without the compensation the same
arithmetic is an order of magnitude worse.
"""

import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def model(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    so = str(tmp_path_factory.mktemp("model") / "libmarch_f32_model.so")
    subprocess.check_call([cc, "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                           os.path.join(HERE, "march_f32_model.c"), "-o", so,
                           "-lm"])
    L = ctypes.CDLL(so)
    dp = ctypes.POINTER(ctypes.c_double)
    L.march_f32_model.restype = ctypes.c_int
    L.march_f32_model.argtypes = [ctypes.c_int, dp, ctypes.c_double,
                                  ctypes.c_double, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_double, ctypes.c_double, dp, dp]
    return L


def _errors(model, t, dx, n_extra, s_urad, seed=1):
    from oracle import oracle as O
    from dyfox_gb300.crystal import diamond_400
    from dyfox_gb300.dislocations import straight_segment
    from dyfox_gb300.grid import LaueGrid, grid_arrays
    from dyfox_gb300.units import deviation_from_urad
    from dyfox_gb300.workloads import random_110_segments
    O.build()
    x = diamond_400()
    grid = LaueGrid(x, t, dx, 20e-6)
    geo = grid_arrays(grid)
    Nx, Ny, Nz = geo["Nx"], geo["Ny"], geo["Nz"]
    xi = np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0)
    b = x.b_mag * np.array([1.0, 0.0, -1.0]) / np.sqrt(2.0)
    z0 = grid.t_crystal / 2
    seg = straight_segment(xi, b, [-z0 * x.tan_tB, dx / 2, z0], 800e-6)
    seg += random_110_segments(x, grid, n_extra, np.random.default_rng(seed))
    rows = [Ny // 2 - 8, Ny // 2, Ny // 2 + 5]
    H = O.h_rows(seg, x.g_vec, x.nu, x.a_core, Nx, Nz, geo["dx"], geo["dz"],
                 O.grid_y(Ny, geo["dx"], rows))
    sig = np.array([x.sig0.real, x.sig0.imag, x.sig_h.real, x.sig_h.imag,
                    x.sig_hbar.real, x.sig_hbar.imag])
    dp = ctypes.POINTER(ctypes.c_double)
    res = []
    for u in s_urad:
        s = deviation_from_urad([u], x)
        ref = O.laue_march("fullfield", x, s, geo, H_rows=H, rows=rows)[0]
        I_ref = np.abs(ref) ** 2
        errs = []
        for comp in (1, 0):
            got = np.zeros((len(rows), Nx), complex)
            for r in range(len(rows)):
                Hr = np.ascontiguousarray(H[r])
                o = np.zeros(2 * Nx)
                assert model.march_f32_model(
                    comp, sig.ctypes.data_as(dp), float(s[0]), geo["ds"], Nz,
                    Nx, geo["dx"], geo["sheet_hw"], Hr.ctypes.data_as(dp),
                    o.ctypes.data_as(dp)) == 0
                got[r] = o[0::2] + 1j * o[1::2]
            I = np.abs(got) ** 2
            errs.append(np.linalg.norm(I - I_ref) / np.linalg.norm(I_ref))
        res.append(tuple(errs))
    return Nz, res


def test_march_arithmetic_share_of_the_budget(model):
    """README thickness and dx (358 steps), one edge dislocation."""
    Nz, res = _errors(model, 200e-6, 0.25e-6, 0, [0.0, 117.5, -60.0])
    assert Nz == 359
    for comp, plain in res:
        assert comp < 3e-7, res
        assert plain > 3 * comp, res


def test_long_march_stays_within_a_few_1e7(model):
    """t = 400 um at dx = 0.125 um: 1434 steps, 9 segments."""
    Nz, res = _errors(model, 400e-6, 0.125e-6, 8, [0.0, 117.5])
    assert Nz == 1435
    for comp, plain in res:
        assert comp < 5e-7, res
        assert plain > 3 * comp, res
