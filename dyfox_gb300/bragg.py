"""The reflection (Bragg) solver: drop-ins for DYFOX ``bragg``.

    surface, info = solve_surface_batch(segs, s_dev, cfg, ys, xtal, g)
    wave, info = solve_bragg_stable(segs, s_dev, cfg, xtal, g)
    T21, T22 = perfect_symbol(e0, eg, ds, Nz, Nx, xtal)

Signatures and results follow DYFOX ``bragg/solver.py:38-379``.  Every
y-plane is an independent shooting problem (transport stays in the plane of
incidence), so each plane gets its own Krylov space on the GPU: one CTA per
(plane, deviation parameter) runs restarted, left-preconditioned GMRES to a
true relative residual <= ``tol`` entirely on the device.  Planes therefore
never need the reference's chunk splitting; ``chunk``, ``chunk_cap``,
``max_depth``, ``per_plane``, ``gpu_gmres``, ``xp`` and ``verbose`` are
accepted for signature compatibility.  A plane whose true residual is above
``accept`` is solved again, warm started, with a Krylov space ``grow`` times
larger (up to ``restart_cap``), at most ``tries`` times.

``solve_scan`` is the batched form: many deviation parameters over the same
planes in one launch.

``precision=FP32`` (keyword-only) selects the mixed-precision solve: the
Krylov products (march and preconditioner) run in single precision, while
the right-hand side, every true residual, the orthogonalisation, the
rotations and the solution stay in double, each restart being one step of
iterative refinement.  It stops on the same true relative residual
``tol`` as the FP64 solve, so its answers agree with FP64 to about ``tol``.
"""

import numpy as np

from . import _lib
from .backend import FP64, precision as as_precision
from .bragg_geometry import (BraggConfig, bragg_g_vector,  # noqa: F401
                             edge_segment, threading_segment)


class BraggDesc(_lib.ctypes.Structure):
    """``dyfox_bragg_desc``."""
    c_double, c_int = _lib.c_double, _lib.c_int
    _fields_ = [("sig0", c_double * 2), ("sig_h", c_double * 2),
                ("sig_hbar", c_double * 2), ("Nx", c_int), ("Nz", c_int),
                ("dx", c_double), ("dz", c_double), ("ds", c_double),
                ("n_y", c_int), ("n_s", c_int), ("n_seg", c_int),
                ("nu", c_double), ("a_core", c_double), ("beam", c_int),
                ("beam_thickness", c_double), ("beam_centre", c_double),
                ("tol", c_double), ("restart", c_int), ("maxiter", c_int),
                ("precision", c_int), ("flags", _lib.c_uint)]


_SIG = {
    "dyfox_bragg_workspace_bytes": (_lib.c_size_t,
                                    [_lib.ctypes.POINTER(BraggDesc)]),
    "dyfox_bragg_solve": (_lib.c_int, [_lib.ctypes.POINTER(BraggDesc)]
                          + [_lib.c_void_p] * 7 + [_lib.c_size_t,
                                                   _lib.c_void_p]),
    "dyfox_bragg_apply": (_lib.c_int, [_lib.ctypes.POINTER(BraggDesc),
                                       _lib.c_int] + [_lib.c_void_p] * 7
                          + [_lib.c_size_t, _lib.c_void_p]),
    "dyfox_bragg_symbol": (_lib.c_int, [_lib.ctypes.POINTER(BraggDesc)]
                           + [_lib.c_void_p] * 4),
}
_bound = False


def _L():
    global _bound
    L = _lib.lib()
    if not _bound:
        for name, (res, args) in _SIG.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _bound = True
    return L


FORCE_RESUME = 1


def _desc(cfg, xtal, n_y, n_s, n_seg, tol, restart, maxiter, prec=FP64,
          flags=0):
    d = BraggDesc()
    for name in ("sig0", "sig_h", "sig_hbar"):
        v = complex(getattr(xtal, name))
        getattr(d, name)[0] = v.real
        getattr(d, name)[1] = v.imag
    d.Nx, d.Nz = int(cfg.Nx), int(cfg.Nz)
    d.dx, d.dz, d.ds = float(cfg.dx), float(cfg.dz), float(cfg.ds)
    d.n_y, d.n_s, d.n_seg = int(n_y), int(n_s), int(n_seg)
    d.nu, d.a_core = float(xtal.nu), float(xtal.a_core)
    bt = getattr(cfg, "beam_thickness", None)
    d.beam = 0 if bt is None else 1
    d.beam_thickness = 0.0 if bt is None else float(bt)
    d.beam_centre = float(getattr(cfg, "beam_centre", 0.0))
    d.tol, d.restart, d.maxiter = float(tol), int(restart), int(maxiter)
    d.precision = as_precision(prec).code
    d.flags = int(flags)
    return d


class _Problem:
    """Device-side inputs of one call: segment table, planes, s values."""

    def __init__(self, seg_list, s_values, cfg, y_values, xtal, g_vec,
                 precision=FP64, flags=0):
        torch = _lib.torch_cuda()
        self.prec = as_precision(precision)
        self.flags = flags
        self.torch = torch
        self.cfg, self.xtal = cfg, xtal
        self.seg_list, self.g_vec = seg_list or [], g_vec
        self.y = np.ascontiguousarray(np.atleast_1d(
            np.asarray(y_values, float)))
        self.s = np.atleast_1d(np.asarray(s_values, float))
        if not np.all(np.isfinite(self.s)):
            raise ValueError("s_dev must be finite")
        table = _lib.segment_table(seg_list or [], g_vec, xtal.nu,
                                   xtal.a_core, cfg.dx)
        self.n_seg = len(table)
        self.table = _lib.device_table(table)
        self.s_dev = torch.from_numpy(self.s).to("cuda")

    def desc(self, tol=1e-10, restart=40, maxiter=25, n_s=None):
        return _desc(self.cfg, self.xtal, len(self.y),
                     len(self.s) if n_s is None else n_s, self.n_seg, tol,
                     restart, maxiter, self.prec, self.flags)

    def workspace(self, d):
        n = _L().dyfox_bragg_workspace_bytes(d)
        if n == 0:
            _lib.check(_lib.DYFOX_EINVAL, "dyfox_bragg_workspace_bytes")
        return self.torch.empty(n, dtype=self.torch.uint8, device="cuda")


def _yp(prob):
    return prob.y.ctypes.data_as(_lib.c_void_p)


def solve_scan(seg_list, s_values, cfg, y_values, xtal, g_vec, tol=1e-10,
               restart=40, maxiter=25, x0=None, *, precision=FP64,
               _flags=0):
    """All deviation parameters x all planes in one launch.

    Returns (out, info): out is a (n_s, n_y, Nx) complex128 CUDA tensor of
    physical exit waves; info a (n_s * n_y, 4) CUDA tensor of (true relative
    residual, inner iterations, code, |b|) per system.
    """
    prob = _Problem(seg_list, s_values, cfg, y_values, xtal, g_vec,
                    precision, _flags)
    return _run(prob, tol, restart, maxiter, x0)


def _run(prob, tol, restart, maxiter, x0=None):
    torch = prob.torch
    d = prob.desc(tol, restart, maxiter)
    ws = prob.workspace(d)
    n_s, n_y, Nx = len(prob.s), len(prob.y), int(prob.cfg.Nx)
    out = torch.empty((n_s, n_y, Nx), dtype=torch.complex128, device="cuda")
    info = torch.empty((n_s * n_y, 4), dtype=torch.float64, device="cuda")
    _lib.check(_L().dyfox_bragg_solve(
        d, _lib.ptr(prob.table), _yp(prob), _lib.ptr(prob.s_dev),
        _lib.ptr(x0), _lib.ptr(out), _lib.ptr(info), _lib.ptr(ws),
        ws.numel(), _lib.stream_ptr()), "dyfox_bragg_solve")
    return out, info


def solve_surface_batch(seg_list, s_dev, cfg, y_values, xtal, g_vec,
                        xp=None, chunk=32, tol=1e-10, restart=40, maxiter=25,
                        verbose=False, gpu_gmres=True, accept=1e-7, grow=4,
                        tries=3, restart_cap=256, max_depth=6, per_plane=6,
                        chunk_cap=32, *, precision=FP64):
    """Exit wave on the (ny, Nx) surface grid for one deviation parameter.

    Returns (NumPy complex128 (ny, Nx), info) with info keys ``residual``
    (worst true relative residual), ``iterations`` (most inner iterations of
    any plane), ``retries``, ``splits`` (always 0: planes are independent),
    ``unconverged_chunks`` (planes above ``accept``) and ``converged``.
    """
    torch = _lib.torch_cuda()
    prob = _Problem(seg_list, [float(s_dev)], cfg, y_values, xtal, g_vec,
                    precision)
    out, info = _run(prob, tol, restart, maxiter)
    res = info[:, 0].cpu().numpy()
    its = int(info[:, 1].max().item()) if len(res) else 0
    retries, r = 0, restart
    for _ in range(max(tries - 1, 0)):
        bad = np.nonzero(res > accept)[0]
        if len(bad) == 0 or r >= restart_cap:
            break
        r = min(r * grow, restart_cap)
        retries += 1
        sub = _Problem(seg_list, [float(s_dev)], cfg, prob.y[bad], xtal,
                       g_vec, precision)
        # warm start from the previous solution (undo the phase restoration)
        e0h = torch.exp(-1j * _plane_H0(sub))
        x0 = (out[0, torch.as_tensor(bad, device="cuda")] / e0h)[None]
        o2, i2 = _run(sub, tol, r, maxiter, x0.contiguous())
        out[0, torch.as_tensor(bad, device="cuda")] = o2[0]
        res[bad] = i2[:, 0].cpu().numpy()
        its = max(its, int(i2[:, 1].max().item()))
    unconverged = int(np.sum(res > accept))
    surface = out[0].cpu().numpy()
    return surface, {"residual": float(res.max()) if len(res) else 0.0,
                     "iterations": its, "retries": retries, "splits": 0,
                     "unconverged_chunks": unconverged,
                     "converged": unconverged == 0}


def _plane_H0(prob):
    """H at z = 0 on each plane of a problem, (n_y, Nx) CUDA tensor (undoes
    the phase restoration of a previous solution for a warm start)."""
    from .dislocations import H_rows
    cfg = prob.cfg
    if prob.n_seg == 0:
        return prob.torch.zeros((len(prob.y), int(cfg.Nx)),
                                dtype=prob.torch.float64, device="cuda")
    return H_rows(prob.seg_list, cfg.Nx, 1, cfg.dx, cfg.dz, prob.g_vec,
                  prob.xtal.nu, prob.xtal.a_core, prob.y)[:, 0, :]


def solve_bragg_stable(seg_list, s_dev, cfg, xtal, g_vec, xp=None,
                       tol=1e-10, y_plane=0.0, restart=40, maxiter=20, *,
                       precision=FP64):
    """One plane: (exit wave, {gmres_code, iterations, residual}).  The wave
    is a NumPy array when ``xp`` is None or NumPy, else a CUDA tensor."""
    prob = _Problem(seg_list, [float(s_dev)], cfg, [y_plane], xtal, g_vec,
                    precision)
    out, info = _run(prob, tol, restart, maxiter)
    inf = info[0].cpu().numpy()
    wave = out[0, 0]
    if xp is None or xp is np:
        wave = wave.cpu().numpy()
    return wave, {"gmres_code": int(inf[2]), "iterations": int(inf[1]),
                  "residual": float(inf[0])}


def apply_operator(seg_list, s_values, cfg, y_values, xtal, g_vec, mode,
                   in0=None, in1=None, *, precision=FP64):
    """The down-march (mode "march": D_g(t) of (D0(0), Dg(0)) = (in0, in1))
    or the preconditioner (mode "precond": M in0) for every (s, plane);
    inputs and output are (n_s, n_y, Nx) complex128 CUDA tensors.
    precision=FP32: the single-precision operators of the mixed solve, and
    mode "march_ff": its float-float march (right-hand side, residuals)."""
    modes = {"march": 0, "precond": 1, "march_ff": 2}
    if mode not in modes:
        raise ValueError(f"mode is one of {sorted(modes)}, not {mode!r}")
    prob = _Problem(seg_list, s_values, cfg, y_values, xtal, g_vec,
                    precision)
    torch = prob.torch
    d = prob.desc()
    ws = prob.workspace(d)
    out = torch.empty((len(prob.s), len(prob.y), int(cfg.Nx)),
                      dtype=torch.complex128, device="cuda")
    _lib.check(_L().dyfox_bragg_apply(
        d, modes[mode], _lib.ptr(prob.table), _yp(prob),
        _lib.ptr(prob.s_dev), _lib.ptr(in0), _lib.ptr(in1), _lib.ptr(out),
        _lib.ptr(ws), ws.numel(), _lib.stream_ptr()), "dyfox_bragg_apply")
    return out


def perfect_symbol(e0, eg, ds, Nz, Nx, xtal):
    """Fourier symbol (T21, T22) of the perfect-crystal shooting operator
    (NumPy, length Nx).  e0 = exp(sig0 ds) and eg = exp((sig0 + i alpha) ds)
    as in the reference; alpha is recovered from eg / e0 (only e^{i alpha
    ds} enters the symbol)."""
    torch = _lib.torch_cuda()
    alpha = np.angle(complex(eg) / complex(e0)) / ds
    s = torch.tensor([-alpha / (2.0 * np.pi)], dtype=torch.float64,
                     device="cuda")

    class _Cfg:
        pass
    cfg = _Cfg()
    cfg.Nx, cfg.Nz, cfg.dx, cfg.dz, cfg.ds = int(Nx), int(Nz), 1.0, 1.0, ds
    d = _desc(cfg, xtal, 1, 1, 0, 1e-10, 1, 1)
    T21 = torch.empty(Nx, dtype=torch.complex128, device="cuda")
    T22 = torch.empty_like(T21)
    _lib.check(_L().dyfox_bragg_symbol(d, _lib.ptr(s), _lib.ptr(T21),
                                       _lib.ptr(T22), _lib.stream_ptr()),
               "dyfox_bragg_symbol")
    return T21.cpu().numpy(), T22.cpu().numpy()
