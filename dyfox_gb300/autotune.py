"""Launch-shape autotuner of the Laue march.

The register-resident march has two free shape parameters: columns per lane
(CPL, the register tile of one thread: 4-8 in FP64, 5-13 in FP32, 3-7 in
the packed-pair FP32 march) and angles per CTA (how many deviation
parameters share one e^{iH} row, each with WA = ceil(Nx / (32 CPL)) warps,
or each pair of them in the pair march).  The best shape depends on Nx, on
the number of angles, on the H source and on the precision.  The pair march
is timed only when asked (``pairs=True``): on GB300 it has run about 10%
behind the scalar march on the README and rocking-scan workloads, since a
packed FFMA2 issues once but occupies the FP32 pipe for two operations.
``tune`` times the
candidates on a copy of the grid cut down in rows (same Nx and Nz, so the
per-row work is unchanged) but with about 2048 CTAs per candidate, enough to
fill the GPU as the full problem does, compares time per row, keeps the
fastest, and caches it per GPU
model and problem signature in a JSON file (``DYFOX_TUNE_CACHE``, default
``~/.cache/dyfox_gb300/laue_tune.json``).  ``solve_dislocation`` and
``solve_pristine`` read the cache for every solve whose shape is not given
explicitly.
"""

import json
import os
import threading

import numpy as np

from . import _lib

CPL = {"fp64": (4, 5, 6, 7, 8), "fp32": (5, 7, 9, 11, 13)}
ANGLES = (1, 2, 3, 4, 6, 8)
CPL_PAIRS = (3, 5, 7)
ANGLES_PAIRS = (2, 4, 6, 8)
_lock = threading.Lock()
_cache = None


def cache_path():
    return os.environ.get("DYFOX_TUNE_CACHE", os.path.join(
        os.path.expanduser("~"), ".cache", "dyfox_gb300", "laue_tune.json"))


def _load():
    global _cache
    if _cache is None:
        try:
            with open(cache_path()) as f:
                _cache = json.load(f)
        except (OSError, ValueError):
            _cache = {}
    return _cache


def _save():
    path = cache_path()
    os.makedirs(os.path.dirname(path), exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(_cache, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def _bucket(n):
    """Angle counts are bucketed by powers of two above 8 (the shape that
    is best for 200 angles is best for 256)."""
    if n <= 8:
        return n
    return 1 << int(np.ceil(np.log2(n)))


def signature(desc):
    torch = _lib.torch_cuda()
    name = torch.cuda.get_device_name()
    flags = desc.flags & ~(_lib.FLAG_GENERAL | _lib.FLAG_PAIRS |
                           _lib.FLAG_SCALAR)
    return "|".join(str(v) for v in (
        name, desc.precision, desc.h_source, flags,
        desc.Nx, desc.Nz, _bucket(desc.n_e), _bucket(desc.n_seg)))


def lookup(desc):
    """(cols_per_lane, angles_per_cta, pairs) cached for this signature,
    or None."""
    with _lock:
        e = _load().get(signature(desc))
    return None if e is None else (e["cols_per_lane"], e["angles_per_cta"],
                                   bool(e.get("pairs", False)))


def tune(seg_list, s_dev_arr, grid, xtal, *, precision="fp32",
         h_mode="auto", H_gpu=None, compensated=True, h_sum="ff", ctas=2048,
         repeats=3, verbose=False, pairs=False):
    """Time every (CPL, angles per CTA, pair march) candidate for this
    problem and cache the fastest.  Returns {"cols_per_lane",
    "angles_per_cta", "pairs", "ms", "candidates": [(cpl, A, pairs, ms),
    ...]}."""
    from .backend import precision as as_precision
    from .grid import grid_arrays
    from .laue import _solve
    torch = _lib.torch_cuda()
    prec = as_precision(precision)
    s = np.atleast_1d(np.asarray(s_dev_arr, float))
    full = grid_arrays(grid)
    full_rows = int(np.sum(np.abs((np.arange(full["Ny"]) - full["Ny"] // 2)
                                  * full["dx"]) < full["fov_hy"]))
    results = []
    ev0, ev1 = torch.cuda.Event(enable_timing=True), \
        torch.cuda.Event(enable_timing=True)
    shapes = [(cpl, A, False) for cpl in CPL[prec.name] for A in ANGLES]
    if pairs and prec.is_fp32 and compensated and len(s) >= 2:
        shapes += [(cpl, A, True) for cpl in CPL_PAIRS for A in ANGLES_PAIRS]
    for cpl, A, pairs in shapes:
        if -(-full["Nx"] // (32 * cpl)) > 32:
            continue
        if A > len(s) + (1 if pairs else 0):
            continue
        groups = -(-len(s) // A)
        rows = min(full_rows, max(32, -(-ctas // groups)))
        small = grid if (H_gpu is not None or rows >= full_rows) else \
            grid.replace(beam_width=rows * grid.dx)
        geo = grid_arrays(small)
        n_rows = int(np.sum(np.abs((np.arange(geo["Ny"]) - geo["Ny"] // 2)
                                   * geo["dx"]) < geo["fov_hy"]))
        out = torch.empty((len(s), geo["Ny"], geo["Nx"]),
                          dtype=prec.torch_complex, device="cuda")
        try:
            kw = dict(h_mode=h_mode, angles_per_cta=A, cols_per_lane=cpl,
                      out=out, tuned=False, compensated=compensated,
                      h_sum=h_sum, pairs=pairs)
            _solve(seg_list, s, small, xtal, H_gpu, 0, prec, False, **kw)
            torch.cuda.synchronize()
            best = np.inf
            for _ in range(repeats):
                ev0.record()
                _solve(seg_list, s, small, xtal, H_gpu, 0, prec, False,
                       **kw)
                ev1.record()
                torch.cuda.synchronize()
                best = min(best, ev0.elapsed_time(ev1))
        except (ValueError, NotImplementedError, MemoryError):
            continue
        results.append((cpl, A, pairs, best / n_rows * full_rows))
        if verbose:
            print(f"cpl {cpl:2d} angles/CTA {A} pairs {pairs}: "
                  f"{best:.3f} ms on {n_rows} rows, "
                  f"{results[-1][3]:.3f} ms scaled")
    if not results:
        raise RuntimeError("no launch shape could run this problem")
    cpl, A, pairs, ms = min(results, key=lambda r: r[3])
    from .laue import describe
    d = describe(seg_list, s, grid, xtal, H_gpu=H_gpu, precision=prec,
                 h_mode=h_mode, compensated=compensated, h_sum=h_sum)
    with _lock:
        _load()[signature(d)] = {"cols_per_lane": cpl, "angles_per_cta": A,
                                 "pairs": pairs, "ms_full_estimate": ms}
        _save()
    return {"cols_per_lane": cpl, "angles_per_cta": A, "pairs": pairs,
            "ms": ms, "candidates": results}

