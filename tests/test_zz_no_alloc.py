"""dyfox_laue_solve_noalloc: the Laue solve for callers that cannot allocate
device memory when they solve (a real-time loop with a fixed memory budget,
a plugin host that forbids allocations after start-up, a C caller without a
device allocator).  Its scratch is a fixed 32 MiB array inside the library.

The test calls it through the C ABI, twice in a row (the array keeps the
previous call's contents), and compares each result with the workspace entry
point dyfox_laue_solve on the same inputs, within the tolerances of the Laue
tests: 1e-12 relative L2 in FP64, 1e-5 on the exit intensity in FP32.
This file is collected last, so a failure here stops a -x run only after
every other test has run.
"""

import ctypes

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def _problem(diamond400):
    from dyfox_gb300.grid import LaueGrid
    from dyfox_gb300.dislocations import burgers_vector, straight_segment
    from dyfox_gb300.units import deviation_from_urad
    grid = LaueGrid(diamond400, 200e-6, 0.25e-6, 120e-6)
    z0 = grid.t_crystal / 2
    b = burgers_vector(np.eye(3), [1, 0, -1], diamond400.b_mag, +1)
    seg = straight_segment(np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0), b,
                           [-z0 * diamond400.tan_tB, grid.dx / 2, z0],
                           800e-6)
    return grid, seg, deviation_from_urad([0.0, 117.5], diamond400)


def _bind(L):
    f = L.dyfox_laue_solve_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 6
    return f


@pytest.mark.parametrize("prec", ["fp64", "fp32"])
def test_noalloc_matches_the_workspace_entry_point(gpu, diamond400, prec):
    from dyfox_gb300 import _lib
    from dyfox_gb300.backend import precision
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import _desc
    torch = gpu
    P = precision(prec)
    grid, seg, s = _problem(diamond400)
    geo = grid_arrays(grid)
    L = _lib.lib()
    noalloc = _bind(L)
    table = _lib.segment_table(seg, diamond400.g_vec, diamond400.nu,
                               diamond400.a_core, geo["dx"])
    tdev = _lib.device_table(table)
    s_dev = torch.from_numpy(np.asarray(s, float)).cuda()
    d = _desc(diamond400, geo, len(s), P, _lib.H_SEGMENTS, len(table))
    need = L.dyfox_laue_workspace_bytes(d)
    assert 0 < need <= 32 << 20
    shape = (len(s), geo["Ny"], geo["Nx"])
    ref = torch.empty(shape, dtype=P.torch_complex, device="cuda")
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    _lib.check(L.dyfox_laue_solve(
        d, _lib.ptr(s_dev), None, _lib.ptr(tdev), _lib.ptr(ref),
        _lib.ptr(ws), ws.numel(), _lib.c_void_p(stream)), "dyfox_laue_solve")
    want = ref.cpu().numpy()
    for _ in range(2):                    # two calls in a row
        out = torch.full(shape, float("nan"), dtype=P.torch_complex,
                         device="cuda")
        st = noalloc(ctypes.addressof(d), s_dev.data_ptr(), None,
                     tdev.data_ptr(), out.data_ptr(), stream)
        _lib.check(st, "dyfox_laue_solve_noalloc")
        got = out.cpu().numpy()
        if prec == "fp64":
            assert rel_l2(got, want) < 1e-12
        else:
            assert rel_l2(np.abs(got) ** 2, np.abs(want) ** 2) < 1e-5


def test_noalloc_rejects_problems_beyond_its_array(gpu, diamond400):
    """A 256-angle scan of 64 segments needs a staged phase grid of about
    2 GB: far beyond the fixed 32 MiB, so the call must refuse it."""
    from dyfox_gb300 import _lib
    from dyfox_gb300.backend import FP32
    from dyfox_gb300.grid import LaueGrid, grid_arrays
    from dyfox_gb300.laue import _desc
    grid = LaueGrid(diamond400, 273e-6, 0.25e-6, 120e-6)
    d = _desc(diamond400, grid_arrays(grid), 256, FP32, _lib.H_SEGMENTS, 64)
    L = _lib.lib()
    assert L.dyfox_laue_workspace_bytes(d) > 32 << 20
    st = _bind(L)(ctypes.addressof(d), 8, None, 8, 8, None)
    assert st == _lib.DYFOX_ENOMEM
    assert b"32" in L.dyfox_last_error() or b"holds" in L.dyfox_last_error()
