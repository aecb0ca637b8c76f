"""Batched uneven instances: many Laue and Bragg solves in one CUDA graph.

    batch = Batch([LaueInstance(segs, s, grid, xtal), ...,
                   BraggInstance(segs, s, cfg, ys, xtal, g), ...])
    batch.run()                 # one graph replay (asynchronous)
    waves = batch.outputs       # per instance, on the GPU

No single DYFOX counterpart: DYFOX solves such a set with one
``laue.solve_dislocation`` (laue/solver.py:34-91) or
``bragg.solve_surface_batch`` (bragg/solver.py:182-379) call per instance.
Here the set is planned once (``dyfox_batch_create``): every instance's
set-up, one persistent march launch over all Laue rows (longest first; the
Volterra phase of each row evaluated once by the CTA that marches it) and
one launch over all Bragg systems are captured into a CUDA graph that
``run`` replays.  Laue instances run the compensated FP32 march (complex64
output) with the segment sum and 2 pi reduction in float-float, or in
double with ``h_sum="fp64"``; Bragg instances run the FP64 or the
mixed-precision solve (complex128 output).  ``cols_per_lane`` and
``warps`` shape the Laue march; ``autotune`` picks them by timing.
"""

import ctypes

import numpy as np

from . import _lib
from .backend import FP32, precision as as_precision
from .bragg import BraggDesc, _desc as _bragg_desc
from .grid import grid_arrays
from .laue import _check_angles, _desc as _laue_desc

BATCH_LAUE, BATCH_BRAGG = 0, 1


class BatchItem(ctypes.Structure):
    """``dyfox_batch_item``."""
    _fields_ = [("kind", _lib.c_int), ("laue", _lib.LaueDesc),
                ("bragg", BraggDesc), ("s_dev", _lib.c_void_p),
                ("seg_table", _lib.c_void_p), ("y_values", _lib.c_void_p),
                ("out", _lib.c_void_p), ("info", _lib.c_void_p)]


class BatchOpts(ctypes.Structure):
    """``dyfox_batch_opts``."""
    _fields_ = [("laue_cols_per_lane", _lib.c_int), ("laue_warps", _lib.c_int),
                ("laue_ctas_per_sm", _lib.c_int), ("flags", _lib.c_uint)]


_SIG = {
    "dyfox_batch_workspace_bytes": (_lib.c_int, [
        ctypes.POINTER(BatchItem), _lib.c_int, ctypes.POINTER(BatchOpts),
        ctypes.POINTER(_lib.c_size_t)]),
    "dyfox_batch_create": (_lib.c_int, [
        ctypes.POINTER(BatchItem), _lib.c_int, ctypes.POINTER(BatchOpts),
        _lib.c_void_p, _lib.c_size_t, _lib.c_void_p,
        ctypes.POINTER(_lib.c_void_p)]),
    "dyfox_batch_launch": (_lib.c_int, [_lib.c_void_p, _lib.c_void_p]),
    "dyfox_batch_kernel_count": (_lib.c_int, [_lib.c_void_p]),
    "dyfox_batch_status": (_lib.c_int, [_lib.c_void_p, _lib.c_void_p]),
    "dyfox_batch_destroy": (_lib.c_int, [_lib.c_void_p]),
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


class LaueInstance:
    """One Laue solve: ``solve_dislocation(segs, s, grid, xtal,
    precision=FP32)`` (an exact-advection grid, even Nx)."""

    kind = "laue"

    def __init__(self, segs, s_dev, grid, xtal):
        self.segs, self.grid, self.xtal = list(segs or []), grid, xtal
        self.s = np.atleast_1d(np.asarray(s_dev, float))


class BraggInstance:
    """One Bragg scan: ``solve_scan(segs, s, cfg, ys, xtal, g,
    precision=...)`` with x0 = 0."""

    kind = "bragg"

    def __init__(self, segs, s_dev, cfg, y_values, xtal, g_vec, *,
                 precision=FP32, tol=1e-10, restart=40, maxiter=25):
        self.segs, self.cfg, self.xtal = list(segs or []), cfg, xtal
        self.g_vec = np.asarray(g_vec, float)
        self.s = np.atleast_1d(np.asarray(s_dev, float))
        self.ys = np.ascontiguousarray(np.atleast_1d(np.asarray(y_values,
                                                                float)))
        self.prec = as_precision(precision)
        self.tol, self.restart, self.maxiter = tol, restart, maxiter


def from_workload(instances, bragg_precision=FP32):
    """Batch instances from the dicts of ``workloads.batched_uneven``."""
    out = []
    for w in instances:
        if w["kind"] == "laue":
            out.append(LaueInstance(w["segs"], w["s"], w["grid"], w["xtal"]))
        else:
            out.append(BraggInstance(w["segs"], w["s"], w["cfg"], w["ys"],
                                     w["xtal"], w["g"],
                                     precision=bragg_precision))
    return out


class Batch:
    """A planned batch: inputs uploaded, outputs allocated, graph ready.

    ``outputs[i]``: (n_e, Ny, Nx) complex64 for a Laue instance, (n_s, n_y,
    Nx) complex128 for a Bragg one; ``infos[i]``: the Bragg instance's
    (n_s * n_y, 4) per-system info (true relative residual, inner
    iterations, code, |b|), None for Laue.
    """

    def __init__(self, instances, *, cols_per_lane=0, warps=0, ctas_per_sm=0,
                 h_sum="ff"):
        torch = _lib.torch_cuda()
        if h_sum not in ("ff", "fp64"):
            raise ValueError(f"h_sum is 'ff' or 'fp64', not {h_sum!r}")
        self.instances = list(instances)
        n = len(self.instances)
        self._items = (BatchItem * max(n, 1))()
        self._keep = []
        self.outputs, self.infos = [], []
        for i, inst in enumerate(self.instances):
            it = self._items[i]
            if inst.kind == "laue":
                self._laue_item(inst, it, h_sum)
            elif inst.kind == "bragg":
                self._bragg_item(inst, it)
            else:
                raise ValueError(f"unknown instance kind {inst.kind!r}")
        self._opts = BatchOpts(int(cols_per_lane), int(warps),
                               int(ctas_per_sm),
                               _lib.FLAG_H_FP64 if h_sum == "fp64" else 0)
        L = _L()
        nb = _lib.c_size_t(0)
        _lib.check(L.dyfox_batch_workspace_bytes(self._items, n, self._opts,
                                                 ctypes.byref(nb)),
                   "dyfox_batch_workspace_bytes")
        self.workspace = torch.empty(int(nb.value), dtype=torch.uint8,
                                     device="cuda")
        handle = _lib.c_void_p()
        _lib.check(L.dyfox_batch_create(
            self._items, n, self._opts, _lib.ptr(self.workspace),
            self.workspace.numel(), _lib.stream_ptr(), ctypes.byref(handle)),
            "dyfox_batch_create")
        self._handle = handle

    def _laue_item(self, inst, it, h_sum):
        torch = _lib.torch_cuda()
        geo = grid_arrays(inst.grid)
        _check_angles(inst.s, inst.xtal, geo)
        x = inst.xtal
        n_seg, h_source, table = 0, _lib.H_NONE, None
        if inst.segs:
            tab = _lib.segment_table(inst.segs, x.g_vec, x.nu, x.a_core,
                                     geo["dx"])
            if len(tab):
                table = _lib.device_table(tab)
                n_seg, h_source = len(tab), _lib.H_SEGMENTS
        flags = _lib.FLAG_H_FP64 if h_sum == "fp64" else 0
        it.kind = BATCH_LAUE
        it.laue = _laue_desc(x, geo, len(inst.s), FP32, h_source, n_seg,
                             None, flags)
        s_dev = torch.from_numpy(inst.s).to("cuda")
        out = torch.empty((len(inst.s), geo["Ny"], geo["Nx"]),
                          dtype=torch.complex64, device="cuda")
        it.s_dev, it.seg_table = _lib.ptr(s_dev), _lib.ptr(table)
        it.out = _lib.ptr(out)
        self._keep += [s_dev, table]
        self.outputs.append(out)
        self.infos.append(None)

    def _bragg_item(self, inst, it):
        torch = _lib.torch_cuda()
        if not np.all(np.isfinite(inst.s)):
            raise ValueError("s_dev must be finite")
        x = inst.xtal
        tab = _lib.segment_table(inst.segs, inst.g_vec, x.nu, x.a_core,
                                 inst.cfg.dx)
        table = _lib.device_table(tab)
        it.kind = BATCH_BRAGG
        it.bragg = _bragg_desc(inst.cfg, x, len(inst.ys), len(inst.s),
                               len(tab), inst.tol, inst.restart, inst.maxiter,
                               inst.prec)
        s_dev = torch.from_numpy(inst.s).to("cuda")
        out = torch.empty((len(inst.s), len(inst.ys), int(inst.cfg.Nx)),
                          dtype=torch.complex128, device="cuda")
        info = torch.empty((len(inst.s) * len(inst.ys), 4),
                           dtype=torch.float64, device="cuda")
        it.s_dev, it.seg_table = _lib.ptr(s_dev), _lib.ptr(table)
        it.y_values = inst.ys.ctypes.data_as(_lib.c_void_p)
        it.out, it.info = _lib.ptr(out), _lib.ptr(info)
        self._keep += [s_dev, table, inst.ys]
        self.outputs.append(out)
        self.infos.append(info)

    @property
    def kernel_count(self):
        """Kernel launches one ``run`` makes."""
        return int(_L().dyfox_batch_kernel_count(self._handle))

    def run(self):
        """Replays the batch on torch's current stream (asynchronous)."""
        if self._handle is None:
            raise ValueError("batch is closed")
        _lib.check(_L().dyfox_batch_launch(self._handle, _lib.stream_ptr()),
                   "dyfox_batch_launch")
        return self.outputs

    def check(self):
        """Waits for the last run on torch's current stream and raises
        DyfoxError if one of its bounded device waits ran out."""
        if self._handle is None:
            raise ValueError("batch is closed")
        _lib.check(_L().dyfox_batch_status(self._handle, _lib.stream_ptr()),
                   "dyfox_batch_status")

    def close(self):
        if getattr(self, "_handle", None) is not None:
            _L().dyfox_batch_destroy(self._handle)
            self._handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def solve_batch(instances, **kw):
    """Plans, runs once and returns (outputs, infos)."""
    b = Batch(instances, **kw)
    b.run()
    return b.outputs, b.infos


CANDIDATES = ((5, 8), (7, 8), (9, 8), (11, 8), (5, 16), (7, 16), (5, 4))


def pick_shape(times, tie=0.01):
    """The (cols_per_lane, warps) of ``times`` {shape: ms} to use: shapes
    within ``tie`` of the fastest are a tie, won by the fewest warps a CTA
    (smaller CTAs balance the persistent queue better on the whole set:
    3.22 against 3.41 s for 4 against 8 warps on the 512-instance set,
    0.03% apart on its tuning sample), then by time."""
    fastest = min(times.values())
    return min((k for k, t in times.items() if t <= (1.0 + tie) * fastest),
               key=lambda k: (k[1], times[k]))


def autotune(instances, candidates=CANDIDATES, sample=48, repeats=2,
             h_sum="ff", seed=0, verbose=False):
    """Launch shape of the batched Laue march: times a batch of ``sample``
    Laue instances (drawn with ``seed``) under each (cols_per_lane, warps)
    candidate, ``repeats`` replays after one warm-up, and returns
    {"cols_per_lane", "warps", "ms": {candidate: ms}}.  Candidates that
    cannot hold an instance are skipped."""
    torch = _lib.torch_cuda()
    laue = [i for i in instances if i.kind == "laue"]
    rng = np.random.default_rng(seed)
    if len(laue) > sample:
        laue = [laue[j] for j in sorted(rng.choice(len(laue), sample,
                                                   replace=False))]
    times = {}
    for cpl, warps in candidates:
        try:
            b = Batch(laue, cols_per_lane=cpl, warps=warps, h_sum=h_sum)
        except (NotImplementedError, MemoryError, ValueError):
            continue
        b.run()
        torch.cuda.synchronize()
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(2)]
        ev[0].record()
        for _ in range(repeats):
            b.run()
        ev[1].record()
        torch.cuda.synchronize()
        times[(cpl, warps)] = ev[0].elapsed_time(ev[1]) / repeats
        if verbose:
            print(f"cpl={cpl} warps={warps}: {times[(cpl, warps)]:.2f} ms")
        b.close()
        del b
    if not times:
        raise NotImplementedError("no launch shape holds these instances")
    best = pick_shape(times)
    return {"cols_per_lane": best[0], "warps": best[1],
            "ms": {f"{c}x{w}": t for (c, w), t in times.items()}}
