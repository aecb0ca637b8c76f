"""ctypes binding of libdyfox_gb300.so (the C ABI of ``include/dyfox_gb300.h``).

The shims pass raw device pointers of torch CUDA tensors and torch's current
CUDA stream.  There is no CPU fallback: without a CUDA device, or without the
compiled library, every solver raises.
"""

import ctypes
import os

import numpy as np

from .build import LIB

DYFOX_OK, DYFOX_EINVAL, DYFOX_ENOMEM, DYFOX_ESMEM = 0, 1, 2, 3
DYFOX_EMAXITER, DYFOX_ENAN, DYFOX_ECUDA, DYFOX_ENOSYS = 4, 5, 6, 7
DYFOX_ETIMEOUT = 8
DYFOX_FP64, DYFOX_FP32 = 0, 1
H_NONE, H_GRID_F64, H_GRID_F32, H_SEGMENTS, H_ANALYTIC = 0, 1, 2, 3, 4
FLAG_FUSED, FLAG_STAGED, FLAG_NO_COMP, FLAG_GENERAL = 1, 2, 4, 8
FLAG_H_FP64 = 16
FLAG_PAIRS, FLAG_SCALAR = 32, 64
SEG_STRIDE = 24


class DyfoxError(RuntimeError):
    """A CUDA-side failure reported by the library."""


_EXC = {DYFOX_EINVAL: ValueError, DYFOX_ENOMEM: MemoryError,
        DYFOX_ESMEM: MemoryError, DYFOX_EMAXITER: DyfoxError,
        DYFOX_ENAN: ValueError, DYFOX_ECUDA: DyfoxError,
        DYFOX_ENOSYS: NotImplementedError, DYFOX_ETIMEOUT: DyfoxError}

c_int, c_uint, c_double, c_size_t, c_void_p = (
    ctypes.c_int, ctypes.c_uint, ctypes.c_double, ctypes.c_size_t,
    ctypes.c_void_p)
_dp = ctypes.POINTER(c_double)


class LaueDesc(ctypes.Structure):
    """``dyfox_laue_desc``."""
    _fields_ = [("sig0", c_double * 2), ("sig_h", c_double * 2),
                ("sig_hbar", c_double * 2), ("Nx", c_int), ("Ny", c_int),
                ("Nz", c_int), ("dx", c_double), ("dz", c_double),
                ("ds", c_double), ("shift_px", c_double),
                ("sheet_hw", c_double), ("fov_hy", c_double),
                ("n_e", c_int), ("precision", c_int), ("h_source", c_int),
                ("n_seg", c_int), ("nu", c_double), ("a_core", c_double),
                ("analytic", c_double * 12), ("flags", c_uint),
                ("angles_per_cta", c_int), ("cols_per_lane", c_int)]


_SIGNATURES = {
    "dyfox_abi_version": (c_int, []),
    "dyfox_status_string": (ctypes.c_char_p, [c_int]),
    "dyfox_last_error": (ctypes.c_char_p, []),
    "dyfox_segment_table": (c_int, [_dp, c_int, _dp, c_double, c_double,
                                    c_double, _dp,
                                    ctypes.POINTER(c_int)]),
    "dyfox_h_grid": (c_int, [c_void_p, c_int, c_int, c_int, c_int, c_double,
                             c_double, c_double, c_double, c_int, c_void_p,
                             c_void_p]),
    "dyfox_h_rows": (c_int, [c_void_p, c_int, c_int, c_int, c_double,
                             c_double, c_double, c_double, c_void_p, c_int,
                             c_void_p, c_void_p]),
    "dyfox_laue_workspace_bytes": (c_size_t, [ctypes.POINTER(LaueDesc)]),
    "dyfox_pipe_peak": (c_int, [c_int, c_int, _dp, c_void_p]),
    "dyfox_launch_count": (ctypes.c_ulonglong, []),
    "dyfox_kernel_timing": (c_int, [c_int]),
    "dyfox_laue_kernel_ms": (c_int, [ctypes.POINTER(ctypes.c_float)]),
    "dyfox_laue_solve": (c_int, [ctypes.POINTER(LaueDesc), c_void_p,
                                 c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_size_t, c_void_p]),
    "dyfox_laue_solve_to_host": (c_int, [ctypes.POINTER(LaueDesc), c_void_p,
                                         c_void_p, c_void_p, c_void_p,
                                         c_void_p, c_void_p, c_size_t,
                                         c_int, c_void_p, c_void_p]),
    "dyfox_laue_solve_status": (c_int, [ctypes.POINTER(LaueDesc), c_void_p,
                                        c_size_t, c_void_p]),
}

_lib = None


def lib():
    """The loaded library; raises if it was never built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise ImportError(
                f"{LIB} is missing: run `python -m dyfox_gb300.build` (needs "
                "nvcc) before using the solvers")
        L = ctypes.CDLL(LIB)
        for name, (res, args) in _SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def laue_kernel_ms():
    """Durations (ms) of the prologue, staging and march kernels of the last
    dyfox_laue_solve on this thread after ``lib().dyfox_kernel_timing(1)``."""
    ms = (ctypes.c_float * 3)()
    check(lib().dyfox_laue_kernel_ms(ms), "dyfox_laue_kernel_ms")
    return [float(v) for v in ms]


def check(status, what):
    if status != DYFOX_OK:
        msg = lib().dyfox_last_error().decode() or \
            lib().dyfox_status_string(status).decode()
        raise _EXC.get(status, DyfoxError)(f"{what}: {msg}")


def torch_cuda():
    """torch, with a CUDA device required."""
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("dyfox_gb300 runs on a CUDA GPU and none is "
                           "visible; there is no CPU fallback")
    return torch


def stream_ptr():
    torch = torch_cuda()
    return c_void_p(torch.cuda.current_stream().cuda_stream)


def ptr(t):
    return c_void_p(t.data_ptr()) if t is not None else c_void_p(0)


def segment_table(seg_list, g_vec, nu, a_core, dx):
    """Host table of ``dyfox_segment_table``: (n_valid, 24) float64."""
    n = len(seg_list)
    segs = np.zeros((max(n, 1), 9))
    for i, s in enumerate(seg_list):
        segs[i] = np.concatenate([np.asarray(v, float).ravel() for v in s])
    segs = np.ascontiguousarray(segs)
    table = np.zeros((max(n, 1), SEG_STRIDE))
    g = np.ascontiguousarray(np.asarray(g_vec, float).ravel()[:3])
    nv = c_int(0)
    check(lib().dyfox_segment_table(
        segs.ctypes.data_as(_dp), c_int(n), g.ctypes.data_as(_dp),
        c_double(nu), c_double(a_core), c_double(dx),
        table.ctypes.data_as(_dp), ctypes.byref(nv)), "dyfox_segment_table")
    return table[:nv.value]


def device_table(table):
    """The segment table as a float64 CUDA tensor (None when empty)."""
    torch = torch_cuda()
    if len(table) == 0:
        return None
    return torch.from_numpy(np.ascontiguousarray(table)).to("cuda")
