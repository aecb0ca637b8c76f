"""dyfox_laue_solve_noalloc: the Laue solve for callers that cannot allocate
device memory when they solve (a real-time loop with a fixed memory budget,
a plugin host that forbids allocations after start-up, a C caller without a
device allocator).  Its scratch is a fixed 32 MiB array inside the library,
shared by every call and keeping the previous call's contents.

The test calls it through the C ABI.  Before each solve that it checks, a
DIFFERENT problem (another grid, another precision, another number of
angles) runs through the same entry point, so the array holds that
problem's tables; the checked solve must still equal the workspace entry
point dyfox_laue_solve on the same inputs byte for byte (the same kernels,
so the same bits), in FP64 and in FP32, on two calls in a row.  A repeat
call must leave the device's free memory (cudaMemGetInfo) unchanged.
This file is collected last, so a failure here stops a -x run only after
every other test has run.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _readme_problem(x):
    """README size: 544 x 800, Nz 359, one edge dislocation, 2 angles."""
    from dyfox_gb300.dislocations import burgers_vector, straight_segment
    from dyfox_gb300.grid import LaueGrid
    from dyfox_gb300.units import deviation_from_urad
    grid = LaueGrid(x, 200e-6, 0.25e-6, 120e-6)
    z0 = grid.t_crystal / 2
    b = burgers_vector(np.eye(3), [1, 0, -1], x.b_mag, +1)
    seg = straight_segment(np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0), b,
                           [-z0 * x.tan_tB, grid.dx / 2, z0], 800e-6)
    return grid, seg, deviation_from_urad([0.0, 117.5], x)


def _other_problem(x):
    """A different problem to leave other contents in the array: 40 um
    crystal (a smaller grid), three segments, 5 angles."""
    from dyfox_gb300.dislocations import burgers_vector, straight_segment
    from dyfox_gb300.grid import LaueGrid
    grid = LaueGrid(x, 40e-6, 0.25e-6, 8e-6, beam_thickness=1e-6)
    segs = []
    for k, (d, bv) in enumerate((([1, 0, 1], [1, 0, -1]),
                                 ([1, 1, 0], [0, 1, 1]),
                                 ([0, 1, 1], [1, 1, 0]))):
        xi = np.asarray(d, float) / np.linalg.norm(d)
        b = burgers_vector(np.eye(3), bv, x.b_mag, +1)
        segs += straight_segment(xi, b, [0.3e-6 * k, grid.dx / 2 + 0.7e-6 * k,
                                         (10 + 9 * k) * 1e-6], 300e-6)
    return grid, segs, np.linspace(-2.0e5, 1.5e5, 5)


class _Case:
    """Device inputs, descriptor and a workspace-entry-point answer."""

    def __init__(self, torch, x, problem, prec):
        from dyfox_gb300 import _lib
        from dyfox_gb300.backend import precision
        from dyfox_gb300.grid import grid_arrays
        from dyfox_gb300.laue import _desc
        grid, segs, s = problem
        P = precision(prec)
        geo = grid_arrays(grid)
        table = _lib.segment_table(segs, x.g_vec, x.nu, x.a_core, geo["dx"])
        self.torch = torch
        self.tdev = _lib.device_table(table)
        self.s_dev = torch.from_numpy(np.asarray(s, float)).cuda()
        self.d = _desc(x, geo, len(s), P, _lib.H_SEGMENTS, len(table))
        self.shape = (len(s), geo["Ny"], geo["Nx"])
        self.ctype = P.torch_complex
        self.need = _lib.lib().dyfox_laue_workspace_bytes(self.d)

    def workspace_answer(self):
        from dyfox_gb300 import _lib
        torch = self.torch
        out = torch.empty(self.shape, dtype=self.ctype, device="cuda")
        ws = torch.empty(self.need, dtype=torch.uint8, device="cuda")
        _lib.check(_lib.lib().dyfox_laue_solve(
            self.d, _lib.ptr(self.s_dev), None, _lib.ptr(self.tdev),
            _lib.ptr(out), _lib.ptr(ws), ws.numel(),
            _lib.c_void_p(torch.cuda.current_stream().cuda_stream)),
            "dyfox_laue_solve")
        return out.cpu().numpy()

    def noalloc(self, fn, out):
        from dyfox_gb300 import _lib
        st = fn(ctypes.addressof(self.d), self.s_dev.data_ptr(), None,
                self.tdev.data_ptr(), out.data_ptr(),
                self.torch.cuda.current_stream().cuda_stream)
        _lib.check(st, "dyfox_laue_solve_noalloc")

    def nan_output(self):
        return self.torch.full(self.shape, float("nan"), dtype=self.ctype,
                               device="cuda")


def _bind(L):
    f = L.dyfox_laue_solve_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p] * 6
    return f


@pytest.mark.parametrize("prec,other", [("fp64", "fp32"), ("fp32", "fp64")])
def test_noalloc_equals_the_workspace_entry_point(gpu, diamond400, prec,
                                                  other):
    from dyfox_gb300 import _lib
    torch = gpu
    fn = _bind(_lib.lib())
    case = _Case(torch, diamond400, _readme_problem(diamond400), prec)
    dirt = _Case(torch, diamond400, _other_problem(diamond400), other)
    assert 0 < case.need <= 32 << 20 and 0 < dirt.need <= 32 << 20
    want = case.workspace_answer()
    dirt_out = dirt.nan_output()
    for call in range(2):                         # two calls in a row
        dirt.noalloc(fn, dirt_out)                # other contents first
        out = case.nan_output()
        case.noalloc(fn, out)
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        assert got.tobytes() == want.tobytes(), f"call {call}"
    # The other problem's answer is also the workspace entry point's.
    assert dirt_out.cpu().numpy().tobytes() == \
        dirt.workspace_answer().tobytes()
    # A repeat call reserves no device memory.
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    case.noalloc(fn, out)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert out.cpu().numpy().tobytes() == want.tobytes()


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
    assert b"holds" in L.dyfox_last_error()
