"""The transmission (Laue) solver: drop-ins for DYFOX ``laue``.

    stack = solve_dislocation(segs, s_dev, grid, xtal)
    stack = solve_pristine(s_dev, grid, xtal)

Signatures, defaults and results follow DYFOX ``laue/solver.py:34-118``: the
exit waves D_g(z = t) on the (Ny, Nx) grid for each deviation parameter, as
an (n_angles, Ny, Nx) complex CUDA tensor (complex128 for FP64, complex64
for FP32); ``backend.to_numpy`` copies it to the host.  Rows outside the
beam are zero.  The displacement phase comes from, in order of preference:
``H_gpu`` (a caller's (Ny, Nz, Nx) grid, float64 or float32, torch or any
DLPack array), the closed form of a single line along x_lab, or the Volterra
field of the segments evaluated inside the march (no H grid is stored).
"""

import numpy as np

from . import _lib
from .backend import FP64, precision as as_precision
from .dislocations import analytic_line_params, analytic_vector
from .grid import LaueGrid, grid_arrays  # noqa: F401  (re-export)

_workspace = {}


def _workspace_tensor(nbytes):
    torch = _lib.torch_cuda()
    dev = torch.cuda.current_device()
    buf = _workspace.get(dev)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8,
                          device="cuda")
        _workspace[dev] = buf
    return buf


def release_workspace():
    """Drop the cached march workspace (see ``backend.free_gpu``)."""
    _workspace.clear()


def _as_device_grid(H, Ny, Nz, Nx):
    torch = _lib.torch_cuda()
    if not isinstance(H, torch.Tensor):
        H = torch.from_dlpack(H)
    if H.device.type != "cuda":
        raise ValueError("H_gpu must live on the GPU")
    if tuple(H.shape) != (Ny, Nz, Nx):
        raise ValueError(f"H_gpu has shape {tuple(H.shape)}, the grid needs "
                         f"{(Ny, Nz, Nx)}")
    if H.dtype not in (torch.float64, torch.float32):
        raise ValueError(f"H_gpu must be float64 or float32, not {H.dtype}")
    return H.contiguous()


def _check_angles(s, xtal, geo):
    if not np.all(np.isfinite(s)):
        raise ValueError("s_dev must be finite")
    # The interaction picture divides by |P22|; it vanishes only when
    # cos(gamma ds) = 0 at alpha = 0, i.e. a depth step near a quarter
    # Pendelloesung period, far outside any exact-advection grid.
    sh = complex(xtal.sig_h)
    alpha = -2.0 * np.pi * s
    gam = np.sqrt(abs(sh) ** 2 + alpha ** 2 / 4)
    ds = geo["ds"]
    sg = np.where(gam > 1e-30, np.sin(gam * ds) / np.maximum(gam, 1e-300), ds)
    rho = np.hypot(np.where(gam > 1e-30, np.cos(gam * ds), 1.0),
                   alpha * 0.5 * sg)
    if np.any(rho < 1e-6):
        raise ValueError("depth step too coarse for this deviation "
                         "parameter (|P22| < 1e-6)")


def _desc(xtal, geo, n_e, prec, h_source, n_seg=0, analytic=None, flags=0,
          angles_per_cta=0, cols_per_lane=0):
    d = _lib.LaueDesc()
    for name in ("sig0", "sig_h", "sig_hbar"):
        v = complex(getattr(xtal, name))
        getattr(d, name)[0] = v.real
        getattr(d, name)[1] = v.imag
    d.Nx, d.Ny, d.Nz = geo["Nx"], geo["Ny"], geo["Nz"]
    d.dx, d.dz, d.ds = geo["dx"], geo["dz"], geo["ds"]
    d.shift_px, d.sheet_hw, d.fov_hy = (geo["shift_px"], geo["sheet_hw"],
                                        geo["fov_hy"])
    d.n_e = n_e
    d.precision = prec.code
    d.h_source = h_source
    d.n_seg = n_seg
    d.nu = float(getattr(xtal, "nu", 0.0))
    d.a_core = float(getattr(xtal, "a_core", 1.0))
    if analytic is not None:
        for i, v in enumerate(analytic_vector(analytic)):
            d.analytic[i] = v
    d.flags = flags
    d.angles_per_cta = angles_per_cta
    d.cols_per_lane = cols_per_lane
    return d


_MODES = {"auto": 0, "fused": _lib.FLAG_FUSED, "staged": _lib.FLAG_STAGED}


def _h_source_of(seg_list, xtal, H_gpu, pristine=False):
    """The C ABI's H source for these inputs (no device work)."""
    if pristine:
        return _lib.H_NONE
    if H_gpu is not None:
        torch = _lib.torch_cuda()
        dt = H_gpu.dtype if isinstance(H_gpu, torch.Tensor) else None
        return _lib.H_GRID_F32 if dt == torch.float32 else _lib.H_GRID_F64
    if analytic_line_params(seg_list, xtal) is not None:
        return _lib.H_ANALYTIC
    return _lib.H_SEGMENTS


def _flags(prec, h_mode, compensated, general, h_sum, pairs="auto"):
    if h_mode not in _MODES:
        raise ValueError(f"h_mode is one of {sorted(_MODES)}, not {h_mode!r}")
    flags = _MODES[h_mode]
    if prec.is_fp32 and not compensated:
        flags |= _lib.FLAG_NO_COMP
    if general:
        flags |= _lib.FLAG_GENERAL
    if h_sum not in ("ff", "fp64"):
        raise ValueError(f"h_sum is 'ff' or 'fp64', not {h_sum!r}")
    if h_sum == "fp64":
        flags |= _lib.FLAG_H_FP64
    if pairs not in ("auto", True, False):
        raise ValueError(f"pairs is 'auto', True or False, not {pairs!r}")
    if pairs is True:
        flags |= _lib.FLAG_PAIRS
    elif pairs is False:
        flags |= _lib.FLAG_SCALAR
    return flags


def _solve(seg_list, s_dev_arr, grid, xtal, H_gpu, batch, precision,
           pristine, h_mode="auto", compensated=True, general=False,
           angles_per_cta=0, cols_per_lane=0, out=None, h_sum="ff",
           tuned=True, pairs="auto", host_out=None):
    torch = _lib.torch_cuda()
    prec = as_precision(precision)
    s = np.atleast_1d(np.asarray(s_dev_arr, dtype=float))
    geo = grid_arrays(grid)
    _check_angles(s, xtal, geo)
    Nx, Ny, Nz = geo["Nx"], geo["Ny"], geo["Nz"]
    n_e = len(s)
    flags = _flags(prec, h_mode, compensated, general, h_sum, pairs)
    table_dev, n_seg, ap, H = None, 0, None, None
    h_source = _h_source_of(seg_list, xtal, H_gpu, pristine)
    if h_source in (_lib.H_GRID_F64, _lib.H_GRID_F32):
        H = _as_device_grid(H_gpu, Ny, Nz, Nx)
        h_source = (_lib.H_GRID_F64 if H.dtype == torch.float64
                    else _lib.H_GRID_F32)
    elif h_source == _lib.H_ANALYTIC:
        ap = analytic_line_params(seg_list, xtal)
    elif h_source == _lib.H_SEGMENTS:
        table = _lib.segment_table(seg_list, xtal.g_vec, xtal.nu,
                                   xtal.a_core, geo["dx"])
        n_seg = len(table)
        table_dev = _lib.device_table(table)
    if out is None:
        out = torch.empty((n_e, Ny, Nx), dtype=prec.torch_complex,
                          device="cuda")
    batch = max(1, int(batch)) if batch else n_e
    s_dev = torch.from_numpy(s).to("cuda")
    stream = _lib.stream_ptr()
    copy_stream = None
    if host_out is not None:
        if (host_out.device.type != "cpu" or host_out.dtype != out.dtype or
                tuple(host_out.shape) != tuple(out.shape) or
                not host_out.is_contiguous()):
            raise ValueError(f"host_out must be a contiguous CPU tensor of "
                             f"shape {tuple(out.shape)} and dtype {out.dtype}")
        copy_stream = torch.cuda.Stream()
    for bs in range(0, n_e, batch):
        be = min(bs + batch, n_e)
        d = _desc(xtal, geo, be - bs, prec, h_source, n_seg, ap, flags,
                  angles_per_cta, cols_per_lane)
        if tuned and not angles_per_cta and not cols_per_lane:
            from .autotune import lookup
            shape = lookup(d)
            if shape is not None:
                d.cols_per_lane, d.angles_per_cta, use_pairs = shape
                if pairs == "auto" and use_pairs:
                    d.flags |= _lib.FLAG_PAIRS
        nbytes = _lib.lib().dyfox_laue_workspace_bytes(d)
        if nbytes == 0:
            _lib.check(_lib.DYFOX_EINVAL, "dyfox_laue_workspace_bytes")
        ws = _workspace_tensor(nbytes)
        if host_out is None:
            _lib.check(_lib.lib().dyfox_laue_solve(
                d, _lib.c_void_p(s_dev.data_ptr() + 8 * bs), _lib.ptr(H),
                _lib.ptr(table_dev), _lib.c_void_p(out[bs].data_ptr()),
                _lib.ptr(ws), ws.numel(), stream), "dyfox_laue_solve")
        else:
            # eight row chunks, each chunk's rows copied while the next
            # marches
            _lib.check(_lib.lib().dyfox_laue_solve_to_host(
                d, _lib.c_void_p(s_dev.data_ptr() + 8 * bs), _lib.ptr(H),
                _lib.ptr(table_dev), _lib.c_void_p(out[bs].data_ptr()),
                _lib.c_void_p(host_out[bs].data_ptr()), _lib.ptr(ws),
                ws.numel(), 0, stream,
                _lib.c_void_p(copy_stream.cuda_stream)),
                "dyfox_laue_solve_to_host")
    if host_out is not None:
        copy_stream.synchronize()
        return host_out
    return out


def describe(seg_list, s_dev_arr, grid, xtal, *, H_gpu=None,
             precision=FP64, h_mode="auto", compensated=True, h_sum="ff",
             pairs="auto"):
    """The C-ABI descriptor one solve_dislocation call would use (host only;
    the autotuner keys its cache on it)."""
    prec = as_precision(precision)
    s = np.atleast_1d(np.asarray(s_dev_arr, dtype=float))
    h_source = _h_source_of(seg_list, xtal, H_gpu)
    n_seg = 0
    if h_source == _lib.H_SEGMENTS:
        n_seg = len(_lib.segment_table(seg_list, xtal.g_vec, xtal.nu,
                                       xtal.a_core, grid.dx))
    ap = analytic_line_params(seg_list, xtal) \
        if h_source == _lib.H_ANALYTIC else None
    return _desc(xtal, grid_arrays(grid), len(s), prec, h_source, n_seg, ap,
                 _flags(prec, h_mode, compensated, False, h_sum, pairs))


def solve_dislocation(seg_list, s_dev_arr, grid, xtal, *, H_gpu=None,
                      batch=64, precision=FP64, h_mode="auto",
                      compensated=True, h_sum="ff", pairs="auto",
                      host_out=None):
    """Exit wave of a dislocation field at each deviation parameter.

    ``batch`` caps the angles per launch (results do not depend on it).
    Keyword-only extensions: ``h_mode`` ("auto", "fused": H evaluated inside
    the march, "staged": e^{iH} computed once into the workspace and read by
    every angle group), ``compensated`` (FP32 compensated updates, default
    on), ``h_sum`` (FP32: segment sum and 2 pi reduction in float-float
    "ff", default, or in double "fp64"), ``pairs`` (FP32 compensated: march
    two deviation parameters per thread in packed f32x2 arithmetic; "auto"
    follows the autotuner and is the scalar march without a tuned shape;
    the results are the same bits either way), ``host_out`` (a contiguous
    CPU tensor, pinned for speed, of the result's shape and dtype: the exit
    waves are copied into it while the march proceeds, in about eight
    batches of angles a call, and it is returned once complete).
    """
    return _solve(seg_list, s_dev_arr, grid, xtal, H_gpu, batch, precision,
                  False, h_mode, compensated, h_sum=h_sum, pairs=pairs,
                  host_out=host_out)


def solve_pristine(s_dev_arr, grid, xtal, *, precision=FP64):
    """Exit wave of a perfect crystal at each deviation parameter."""
    return _solve([], s_dev_arr, grid, xtal, None, 0, precision, True)
