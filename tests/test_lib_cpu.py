"""The C-ABI library on the CPU: it loads, exports every entry point the
header declares, and its host-only entry points and argument checks work
without a GPU (no compute call is made here)."""

import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, golden

HEADER = os.path.join(ROOT, "include", "dyfox_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"\b(dyfox_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    from dyfox_gb300 import _lib, build
    import shutil
    if not os.path.exists(build.LIB):
        if not shutil.which("nvcc") and not os.path.exists(
                "/usr/local/cuda/bin/nvcc"):
            pytest.skip("library not built and no nvcc")
        build.build()
    return _lib.lib()


def test_header_declares_the_entry_points():
    syms = declared_symbols()
    for name in ("dyfox_laue_solve", "dyfox_h_grid", "dyfox_h_rows",
                 "dyfox_segment_table", "dyfox_laue_workspace_bytes"):
        assert name in syms


def test_every_declared_symbol_is_exported(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_status_strings(lib):
    from dyfox_gb300 import _lib
    assert lib.dyfox_abi_version() == 1
    assert lib.dyfox_status_string(_lib.DYFOX_EINVAL) == b"invalid argument"
    assert lib.dyfox_status_string(99) == b"unknown status"


def test_segment_table_matches_the_oracle_frames(lib, diamond400):
    """dyfox_segment_table is host code: the frame equals the oracle's."""
    from dyfox_gb300 import _lib
    from oracle import oracle as O
    v = golden("volterra")
    for name in ("n", "x", "r", "screw", "zero"):
        segs = [(s[:3], s[3:6], s[6:]) for s in v[f"segs_{name}"]]
        t = _lib.segment_table(segs, diamond400.g_vec, diamond400.nu,
                               diamond400.a_core, 0.25e-6)
        f = O.segment_frames(segs, diamond400.g_vec)
        np.testing.assert_allclose(t[:, :16], f, rtol=1e-15, atol=1e-30)


def test_degenerate_segments_are_dropped(lib, diamond400):
    from dyfox_gb300 import _lib
    p = np.array([1e-6, 2e-6, 3e-6])
    t = _lib.segment_table([(p, p, np.array([1e-10, 0, 0]))],
                           diamond400.g_vec, diamond400.nu,
                           diamond400.a_core, 0.25e-6)
    assert len(t) == 0


def test_non_finite_segment_is_rejected(lib, diamond400):
    from dyfox_gb300 import _lib
    bad = [(np.array([np.nan, 0, 0]), np.ones(3), np.ones(3))]
    with pytest.raises(ValueError):
        _lib.segment_table(bad, diamond400.g_vec, diamond400.nu,
                           diamond400.a_core, 0.25e-6)


def _desc(diamond400, small_grid, **kw):
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import _desc
    from dyfox_gb300.backend import FP64
    d = _desc(diamond400, grid_arrays(small_grid), 3, FP64, 0)
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def test_workspace_query_without_a_gpu(lib, diamond400, small_grid):
    d = _desc(diamond400, small_grid)
    n = lib.dyfox_laue_workspace_bytes(d)
    assert n >= 3 * (small_grid.Nz - 1) * 32
    assert lib.dyfox_laue_workspace_bytes(
        _desc(diamond400, small_grid, Nz=1)) == 0
    assert lib.dyfox_laue_workspace_bytes(
        _desc(diamond400, small_grid, precision=7)) == 0


@pytest.mark.parametrize("field,value,status", [
    ("Nx", 0, 1), ("n_e", 0, 1), ("precision", 5, 1), ("h_source", 9, 1),
    ("shift_px", -1.0, 1)])
def test_bad_descriptors_fail_before_any_cuda_call(lib, diamond400,
                                                   small_grid, field, value,
                                                   status):
    d = _desc(diamond400, small_grid, **{field: value})
    st = lib.dyfox_laue_solve(d, ctypes.c_void_p(8), None, None,
                              ctypes.c_void_p(8), None, 0, None)
    assert st == status
    assert lib.dyfox_last_error() != b""


def test_null_pointers_are_rejected(lib, diamond400, small_grid):
    d = _desc(diamond400, small_grid)
    assert lib.dyfox_laue_solve(d, None, None, None, None, None, 0,
                                None) == 1
    st = lib.dyfox_laue_solve(d, ctypes.c_void_p(8), None, None,
                              ctypes.c_void_p(8), None, 0, None)
    assert st == 2          # workspace too small


def test_solvers_fail_loudly_without_a_gpu(diamond400, small_grid):
    from conftest import has_gpu
    if has_gpu():
        pytest.skip("a GPU is visible")
    from dyfox_gb300.laue import solve_pristine
    with pytest.raises(RuntimeError, match="CUDA"):
        solve_pristine([0.0], small_grid, diamond400)


def test_ctypes_structs_match_the_header(tmp_path):
    """The ctypes mirrors of the header's structs have the C compiler's
    sizes and field offsets (a C program built from the header prints
    them)."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    from dyfox_gb300 import _lib
    from dyfox_gb300.batch import BatchItem, BatchOpts
    from dyfox_gb300.bragg import BraggDesc
    structs = {"dyfox_laue_desc": _lib.LaueDesc,
               "dyfox_bragg_desc": BraggDesc,
               "dyfox_batch_item": BatchItem,
               "dyfox_batch_opts": BatchOpts}
    lines = ['#include <stdio.h>', '#include <stddef.h>',
             '#include "dyfox_gb300.h"', 'int main(void) {']
    for cname, py in structs.items():
        lines.append(f'printf("{cname} size %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'printf("{cname} {f[0]} %zu\\n", '
                         f'offsetof({cname}, {f[0]}));')
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call([cc, "-I", os.path.join(ROOT, "include"),
                           str(src), "-o", str(exe)])
    got = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        cname, field, v = line.split()
        got[(cname, field)] = int(v)
    for cname, py in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f in py._fields_:
            assert got[(cname, f[0])] == getattr(py, f[0]).offset, \
                (cname, f[0])


def _bragg_desc(diamond400, mixed=False, **kw):
    from dyfox_gb300.bragg import BraggConfig, _desc
    from dyfox_gb300.backend import FP32, FP64
    cfg = BraggConfig(diamond400, t_crystal=10e-6, dx=0.5e-6, half_x=8e-6)
    d = _desc(cfg, diamond400, n_y=3, n_s=5, n_seg=1, tol=1e-10, restart=20,
              maxiter=10, prec=FP32 if mixed else FP64)
    for k, v in kw.items():
        setattr(d, k, v)
    return d


def test_bragg_workspace_query_without_a_gpu(lib, diamond400):
    """The workspace holds the couplings of every plane, the Krylov basis of
    every (plane, s) system and, for the mixed form, the single-precision
    and low-word copies of the couplings."""
    from dyfox_gb300 import bragg
    L = bragg._L()
    d64, d32 = _bragg_desc(diamond400), _bragg_desc(diamond400, mixed=True)
    n64, n32 = (L.dyfox_bragg_workspace_bytes(d64),
                L.dyfox_bragg_workspace_bytes(d32))
    plane = d64.Nz * d64.Nx
    assert n64 >= (2 * d64.n_y * plane * 16
                   + d64.n_y * d64.n_s * (d64.restart + 1) * d64.Nx * 16)
    assert n32 - n64 >= 4 * d64.n_y * plane * 8
    assert n64 % 256 == 0 and n32 % 256 == 0
    for bad in (dict(Nx=1), dict(n_s=0), dict(tol=0.0), dict(restart=0),
                dict(restart=2000), dict(precision=3), dict(flags=8)):
        assert L.dyfox_bragg_workspace_bytes(
            _bragg_desc(diamond400, **bad)) == 0, bad


@pytest.mark.parametrize("field,value,status", [
    ("Nx", 1, 1), ("n_y", 0, 1), ("ds", -1.0, 1), ("maxiter", 0, 1),
    ("precision", 4, 1), ("flags", 2, 1), ("Nx", 8192, 7)])
def test_bragg_bad_descriptors_fail_before_any_cuda_call(lib, diamond400,
                                                         field, value, status):
    from dyfox_gb300 import bragg
    L = bragg._L()
    d = _bragg_desc(diamond400, **{field: value})
    p = ctypes.c_void_p(8)
    st = L.dyfox_bragg_solve(d, p, p, p, None, p, None, p, 1 << 40, None)
    assert st == status
    assert lib.dyfox_last_error() != b""
    assert L.dyfox_bragg_symbol(d, p, p, None, None) == status


def test_bragg_null_pointers_modes_and_workspace(lib, diamond400):
    from dyfox_gb300 import bragg
    L = bragg._L()
    p = ctypes.c_void_p(8)
    d64, d32 = _bragg_desc(diamond400), _bragg_desc(diamond400, mixed=True)
    n = L.dyfox_bragg_workspace_bytes(d64)
    # NULL planes, s values, output or segment table (n_seg = 1)
    for args in ((None, p, p, p), (p, None, p, p), (p, p, None, p),
                 (p, p, p, None)):
        seg, y, s, out = args
        assert L.dyfox_bragg_solve(d64, seg, y, s, None, out, None, p, n,
                                   None) == 1
    assert L.dyfox_bragg_solve(d64, p, p, p, None, p, None, p, n - 1,
                               None) == 2
    assert L.dyfox_bragg_solve(d64, p, p, p, None, p, None, None, n,
                               None) == 2
    # apply: modes 0..2, the float-float march (2) only for the mixed form,
    # the preconditioner (1) needs its input
    for d, mode in ((d64, 3), (d64, -1), (d64, 2), (d32, 3)):
        assert L.dyfox_bragg_apply(d, mode, p, p, p, p, p, p, p, 1 << 40,
                                   None) == 1, (d.precision, mode)
    assert L.dyfox_bragg_apply(d64, 1, p, p, p, None, None, p, p, 1 << 40,
                               None) == 1
    assert L.dyfox_bragg_symbol(d64, None, p, p, None) == 1
    assert L.dyfox_bragg_symbol(d64, p, None, None, None) == 1



def test_batch_plan_without_a_gpu(lib, diamond400, small_grid):
    """A batch of Bragg items is planned on the host alone: its workspace
    holds every instance's own workspace and grows with each instance.
    Bad options, NULL inputs, unknown kinds and unsupported Laue items are
    refused before any device query."""
    from dyfox_gb300 import batch, bragg
    L, LB = batch._L(), bragg._L()
    p = ctypes.c_void_p(8)
    y = (ctypes.c_double * 3)(0.0, 1e-7, 2e-7)

    def item(**kw):
        it = batch.BatchItem()
        it.kind = 1
        it.bragg = _bragg_desc(diamond400, **kw)
        it.s_dev, it.seg_table, it.out = p, p, p
        it.y_values = ctypes.cast(y, ctypes.c_void_p)
        return it

    def plan(items, opts=None):
        arr = (batch.BatchItem * max(len(items), 1))(*items)
        n = ctypes.c_size_t(1)
        st = L.dyfox_batch_workspace_bytes(arr, len(items), opts,
                                           ctypes.byref(n))
        return st, n.value

    assert plan([]) == (0, 256)
    one = [item()]
    two = one + [item(mixed=True, Nz=7)]
    st1, n1 = plan(one)
    st2, n2 = plan(two)
    assert st1 == 0 and st2 == 0
    assert n1 >= LB.dyfox_bragg_workspace_bytes(one[0].bragg)
    assert n2 - n1 >= LB.dyfox_bragg_workspace_bytes(two[1].bragg)
    for opts in (dict(laue_cols_per_lane=6), dict(laue_warps=32),
                 dict(laue_ctas_per_sm=-1), dict(flags=1)):
        o = batch.BatchOpts(**opts)
        assert plan(one, ctypes.byref(o)) == (1, 0), opts
    no_y = item()
    no_y.y_values = None
    assert plan([no_y])[0] == 1
    assert plan([item(restart=0)])[0] == 1
    unknown = item()
    unknown.kind = 5
    assert plan([unknown])[0] == 1
    # batched Laue items are single precision (here FP64: refused)
    laue = batch.BatchItem()
    laue.kind = 0
    laue.laue = _desc(diamond400, small_grid)
    laue.s_dev, laue.out = p, p
    assert plan([laue])[0] == 7
    assert b"DYFOX_FP32" in lib.dyfox_last_error()


@pytest.mark.parametrize("n,Ny,Nx,prec", [
    (0, 8, 8, 0), (1, 7, 8, 0), (1, 8, 9, 1), (1, 8, 8, 2), (2, 0, 8, 1)])
def test_imaging_sizes_are_checked_before_any_cuda_call(lib, n, Ny, Nx,
                                                        prec):
    """Imaging takes even grids (the unshifted composition is exact only
    there) and one of the two precisions."""
    from dyfox_gb300 import optics
    L = optics._L()
    b = ctypes.c_size_t(1)
    assert L.dyfox_image_workspace_bytes(n, Ny, Nx, prec,
                                         ctypes.byref(b)) == 1
    assert b.value == 0
    p = ctypes.c_void_p(8)
    assert L.dyfox_image(p, n, Ny, Nx, prec, p, p, None, None, None, None,
                         p, 1 << 40, None) == 1
    assert b"even" in lib.dyfox_last_error() or \
        b"precision" in lib.dyfox_last_error()


def test_pupil_arguments_are_checked_before_any_cuda_call(lib):
    from dyfox_gb300 import optics
    L = optics._L()
    p = ctypes.c_void_p(8)
    good = dict(Nx=8, Ny=8, dx=1e-7, f=1e-4, levels=0, prec=0, out=p)
    for bad in (dict(Nx=0), dict(dx=0.0), dict(f=-1.0), dict(levels=-1),
                dict(prec=3), dict(out=None)):
        a = {**good, **bad}
        assert L.dyfox_pupil(a["Nx"], a["Ny"], a["dx"], a["f"], 2, 0.0, 0.0,
                             0.0, 0.0, 1, a["levels"], a["prec"], a["out"],
                             None) == 1, bad


def test_integration_stub_struct_matches_the_binding():
    """The ctypes stub shown to maintainers declares dyfox_laue_desc with
    the same fields, types and layout as the library's own binding."""
    import re
    from dyfox_gb300 import _lib
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    m = re.search(r"class Desc\(ctypes\.Structure\):.*?\n(\s+_fields_ = "
                  r"\[.*?\])\n", text, re.S)
    assert m, "no Desc struct in the stub"
    ns = {"ctypes": ctypes, "_D": ctypes.c_double}
    exec("class Desc(ctypes.Structure):\n" + m.group(1), ns)
    stub = ns["Desc"]
    assert [f[0] for f in stub._fields_] == \
        [f[0] for f in _lib.LaueDesc._fields_]
    assert ctypes.sizeof(stub) == ctypes.sizeof(_lib.LaueDesc)
    for name, _ in stub._fields_:
        assert getattr(stub, name).offset == \
            getattr(_lib.LaueDesc, name).offset, name


def test_diagnostics_refuse_bad_use_before_any_cuda_call(lib):
    """The kernel-time read needs a timed solve on the thread first; the
    arithmetic probe checks its operation code and pointers."""
    import ctypes
    from dyfox_gb300 import _lib
    ms = (ctypes.c_float * 3)()
    assert lib.dyfox_laue_kernel_ms(ms) == _lib.DYFOX_EINVAL
    assert b"dyfox_kernel_timing" in lib.dyfox_last_error()
    f = lib.dyfox_arith_probe
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    assert f(9, 8, 8, 8, 4, None) == _lib.DYFOX_EINVAL
    assert f(2, 8, None, 8, 4, None) == _lib.DYFOX_EINVAL
    assert f(0, None, None, 8, 4, None) == _lib.DYFOX_EINVAL
    assert f(0, None, None, None, 0, None) == _lib.DYFOX_OK
