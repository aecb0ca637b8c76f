#!/usr/bin/env python
"""Benchmark of the Laue hot path (DYFOX solve_dislocation) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step"): the rocking scan -- diamond (400) at 17 keV,
t = 273 um, dx = 0.25 um, beam width 120 um (grid 544 x 1056, Nz = 490,
481 illuminated rows), 64 seeded random <110> segments, 256 deviation
parameters uniform on [-300, +300] urad: the Volterra phase of every
voxel and the depth march of every angle, all angles in one call.
Unit: voxel-steps (angle x active row x column x depth step).

--impl ours (default): the chosen form -- FP32 march with compensated
(Fast2Sum) amplitude updates and FP32 sincos; the segment sum of H and its
2 pi reduction in FP64; e^{iH} evaluated once per voxel into the workspace
and read by every angle group -- timed on the device with inputs resident.
Its exit waves are checked against the plain FP64 form of the same scan
(all 256 angles, timed once) in the same run: intensity within 1e-5
relative L2, with the phase error reported.  The same march with the
segment sum in float-float and the README-size drop-in (2 angles, one
segment) are timed beside it.  e2e times the public call with host inputs
and a device-to-host read of the exit waves.  reference_gpu times the
reference's own kernel (its CUDA text, launched as DYFOX launches it) on
the same GPU, through the reference arm below.
--impl reference: the reference's Laue kernel (its CUDA text compiled for
the CPU, oracle/_ref; the oracle restatement when absent) on the host cores,
on a bounded sample of rows x angles of the same scan per step.
--impl reference --reference-gpu: the reference's kernel on the GPU (one
JSON object of timings; run by the ours arm as a child process).

Multi-GPU: every rank runs its own replica (the path has no exchange step);
value = all ranks' voxel-steps / max-over-ranks time.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("voxel-steps/s (Laue scan) + Bragg solves/s at ≤1e-5 rel err, "
          "chosen vs plain FP64")
WORKLOAD = ("laue-rocking-scan: diamond(400) 17 keV, t=273um dx=0.25um "
            "beam_width=120um (Ny x Nx = 544 x 1056, Nz=490, 481 active "
            "rows), 64 seeded random <110> segments (lengths log-uniform "
            "20-800 um), 256 s_dev uniform on [-300, +300] urad")
README_WORKLOAD = ("laue-readme: diamond(400) 17 keV, t=200um dx=0.25um "
                   "beam_width=120um (Ny x Nx = 544 x 800, Nz=359), 1 edge "
                   "dislocation line [101] b=(a/2)[10-1] at depth t/2, "
                   "s_dev at 0 and 117.5 urad")
# DRAM bytes (read + write) per launch of the scan's march kernel,
# laue_march_kernel<float, 11, staged e^{iH}, compensated>: an ncu capture
# of the full 256-angle launch (`python bench.py --once scan256`: the staged
# e^{iH} table, 2.0 GB, read once, and the 1.0 GB of exit waves written).
MARCH_SCAN_DRAM_BYTES = 2007279872 + 1023596544
MARCH_SCAN_DRAM_SHAPE = ("ncu dram__bytes_read.sum + dram__bytes_write.sum "
                         "of the 256-angle march launch (11 columns per "
                         "lane, 4 angles per CTA: the block's register "
                         "limit caps the tuner's 8)")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--reference-gpu", action="store_true",
                    help="with --impl reference: time the reference kernel "
                         "on the GPU and print one JSON object")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="skip the reference-kernel-on-GPU leg")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--once", choices=["fp32", "fp64", "bragg", "bragg32",
                                       "bragg32-scan",
                                       "scan", "scan256", "image", "batch",
                                       "unet", "hgrid"],
                    help="run one solve of that form after one warm-up and "
                         "exit (a small, fixed case for ncu)")
    ap.add_argument("--no-bragg", action="store_true")
    ap.add_argument("--no-readme", action="store_true")
    ap.add_argument("--no-com-maps", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--learned-train", type=int, default=16,
                    help="training instances of the learned-guess leg "
                         "(64 solves each)")
    ap.add_argument("--learned-test", type=int, default=2)
    ap.add_argument("--learned-epochs", type=int, default=8)
    ap.add_argument("--learned-tmax", type=float, default=25e-6,
                    help="thickest instance of the learned-guess leg (m); "
                         "the configuration's range ends at 100e-6")
    ap.add_argument("--batched-h-sum", choices=["ff", "fp64"],
                    default="fp64",
                    help="H segment sum of the batched leg's Laue instances: "
                         "IEEE double (the chosen form: its worst instance "
                         "stays within the 1e-5 budget) or float-float "
                         "(FP64-class, faster); the other is timed beside it")
    ap.add_argument("--batched-sample", type=int, default=0,
                    help="batched leg on the first N instances (0: all 512)")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the launch-shape autotuner (use its cache or "
                         "the built-in choice)")
    return ap.parse_args()


def workload():
    from dyfox_gb300.workloads import laue_rocking_scan
    return laue_rocking_scan()


def readme_workload():
    from dyfox_gb300.workloads import laue_readme
    return laue_readme()


def bragg_workload():
    from dyfox_gb300.workloads import bragg_config1
    return bragg_config1()


def active_rows(geo):
    iy = np.arange(geo["Ny"])
    return iy[np.abs((iy - geo["Ny"] // 2) * geo["dx"]) < geo["fov_hy"]]


def max_over_ranks(t_local, world):
    """The largest of every rank's ``t_local`` (a time in seconds); the
    value itself for one rank.  Works on the NCCL (CUDA tensor) and gloo
    (CPU tensor) backends."""
    if world <= 1:
        return float(t_local)
    import torch
    dev = "cuda" if torch.distributed.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(t_local)], dtype=torch.float64, device=dev)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t)


def dist():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return rank, world


class Clocks:
    """nvidia-smi samples (200 ms) over the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in self.lines:
            f = [v.strip() for v in line.split(",")]
            if len(f) < 8:
                continue
            try:
                sm.append(float(f[0]))
                smax.append(float(f[1]))
            except ValueError:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ ours
def _intensity_err(a, b):
    """Relative L2 of |a|^2 against |b|^2 (CUDA tensors, in double)."""
    import torch
    Ia = a.abs().double() ** 2
    Ib = b.abs().double() ** 2
    return float(torch.linalg.vector_norm(Ia - Ib)
                 / torch.linalg.vector_norm(Ib))


def _phase_err(a, b):
    """Intensity-weighted rms phase difference (rad) of a against b."""
    import torch
    a = a.to(torch.complex128)
    w = b.abs() ** 2
    dphi = torch.angle(a * b.conj())
    return float(torch.sqrt((w * dphi ** 2).sum() / w.sum()))


class LaueCall:
    """One dyfox_laue_solve through the C ABI with resident inputs and a
    preallocated workspace and output (the autotuned shape when cached)."""

    def __init__(self, x, geo, segs, s, prec, flags):
        import torch
        from dyfox_gb300 import _lib
        from dyfox_gb300.autotune import lookup
        from dyfox_gb300.laue import _desc
        self.L = _lib.lib()
        table = _lib.segment_table(segs, x.g_vec, x.nu, x.a_core, geo["dx"])
        self.table = table
        self.tdev = _lib.device_table(table)
        self.s_dev = torch.from_numpy(np.asarray(s, float)).cuda()
        d = _desc(x, geo, len(s), prec, _lib.H_SEGMENTS, len(table),
                  flags=flags)
        shape = lookup(d)
        if shape is not None:
            d.cols_per_lane, d.angles_per_cta, pairs = shape
            if pairs:
                d.flags |= _lib.FLAG_PAIRS
        self.d = d
        nb = self.L.dyfox_laue_workspace_bytes(d)
        self.ws = torch.empty(max(nb, 256), dtype=torch.uint8, device="cuda")
        self.out = torch.empty((len(s), geo["Ny"], geo["Nx"]),
                               dtype=prec.torch_complex, device="cuda")
        self.stream = torch.cuda.current_stream()

    def __call__(self):
        from dyfox_gb300 import _lib
        _lib.check(self.L.dyfox_laue_solve(
            self.d, _lib.ptr(self.s_dev), None, _lib.ptr(self.tdev),
            _lib.ptr(self.out), _lib.ptr(self.ws), self.ws.numel(),
            _lib.c_void_p(self.stream.cuda_stream)), "dyfox_laue_solve")

    def check(self):
        """Raises if the last call's bounded device waits ran out."""
        from dyfox_gb300 import _lib
        _lib.check(self.L.dyfox_laue_solve_status(
            self.d, _lib.ptr(self.ws), self.ws.numel(),
            _lib.c_void_p(self.stream.cuda_stream)),
            "dyfox_laue_solve_status")


def timed_steps(fn, steps, warmup, flush, kernel_ms=False):
    """Device time (ms) of each of ``steps`` calls after ``warmup``, CUDA
    events on the current stream, L2 flushed before each call outside the
    events; with ``kernel_ms`` also each call's (prologue, staging, march)
    kernel times from the library's events.  Returns (ms list, kernel ms
    list, launches of this library)."""
    import torch
    from dyfox_gb300 import _lib
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    if kernel_ms:
        _lib.check(L.dyfox_kernel_timing(1), "dyfox_kernel_timing")
    ev = [(torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    km = []
    n0 = L.dyfox_launch_count()
    for a, b in ev:
        flush.zero_()
        a.record(stream)
        fn()
        b.record(stream)
        if kernel_ms:
            km.append(_lib.laue_kernel_ms())
    torch.cuda.synchronize()
    launches = L.dyfox_launch_count() - n0
    if kernel_ms:
        _lib.check(L.dyfox_kernel_timing(0), "dyfox_kernel_timing")
    return [a.elapsed_time(b) for a, b in ev], km, launches


def pipe_peaks():
    """Measured FMA throughput (TFLOP/s) of the FP32 and FP64 pipes."""
    import ctypes
    import torch
    from dyfox_gb300 import _lib
    L = _lib.lib()
    sp = _lib.c_void_p(torch.cuda.current_stream().cuda_stream)
    peaks = {}
    for name, code in (("fp32", _lib.DYFOX_FP32), ("fp64", _lib.DYFOX_FP64)):
        v = _lib.c_double(0)
        _lib.check(L.dyfox_pipe_peak(code, 4096 if name == "fp32" else 256,
                                     ctypes.byref(v), sp), "dyfox_pipe_peak")
        peaks[name] = v.value
    return peaks


def run_ours(args):
    import torch
    from dyfox_gb300 import _lib
    from dyfox_gb300.backend import FP32, FP64
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import solve_dislocation

    rank, world = dist()
    if world > 1:
        torch.distributed.init_process_group(
            "nccl", init_method="env://", rank=rank, world_size=world)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if args.once:
        return run_once(args)
    x, grid, segs, s = workload()
    geo = grid_arrays(grid)
    rows = active_rows(geo)
    n_e = len(s)
    nsteps = geo["Nz"] - 1
    units = n_e * len(rows) * geo["Nx"] * nsteps        # voxel-steps
    voxels = len(rows) * geo["Nx"] * nsteps             # H evaluations

    tuned = {}
    if not args.no_tune:
        from dyfox_gb300.autotune import tune
        for h_sum in ("fp64", "ff"):
            r = tune(segs, s, grid, x, precision="fp32", h_mode="staged",
                     h_sum=h_sum)
            tuned[h_sum] = {"pairs": r.get("pairs", False),
                            "cols_per_lane": r["cols_per_lane"],
                            "angles_per_cta": r["angles_per_cta"]}
    staged = _lib.FLAG_STAGED
    chosen = LaueCall(x, geo, segs, s, FP32, staged | _lib.FLAG_H_FP64)
    n_seg = len(chosen.table)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    peaks = pipe_peaks()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        ms, km, launches = timed_steps(chosen, args.steps, args.warmup,
                                       flush, kernel_ms=True)
        wall = time.perf_counter() - t0
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    chosen.check()
    tot = max_over_ranks(sum(ms) / 1e3, world)
    value = world * units * args.steps / tot
    mean_ms = 1e3 * tot / args.steps
    km = np.array(km)
    march_ms = float(km[:, 2].mean())
    stage_ms = float(km[:, 1].mean())
    prologue_ms = float(km[:, 0].mean())

    # The plain FP64 form of the whole scan, timed once, and the errors of
    # the chosen form against it over all 256 angles.
    plain = LaueCall(x, geo, segs, s, FP64, staged)
    plain_ms, _, _ = timed_steps(plain, 1, 0, flush)
    err_I = _intensity_err(chosen.out, plain.out)
    err_phase = _phase_err(chosen.out, plain.out)
    err_field = float(torch.linalg.vector_norm(
        chosen.out.to(torch.complex128) - plain.out)
        / torch.linalg.vector_norm(plain.out))
    if err_I > 1e-5:
        raise SystemExit(f"chosen form misses the 1e-5 budget: {err_I:.2e}")
    del plain
    torch.cuda.empty_cache()

    # The same march with the segment sum and reduction in float-float.
    ff = LaueCall(x, geo, segs, s, FP32, staged)
    ms_ff, km_ff, _ = timed_steps(ff, max(3, args.steps // 4), 2, flush,
                                  kernel_ms=True)
    ff_err = _intensity_err(ff.out, chosen.out.to(torch.complex128))
    del ff

    # e2e: the public call with host inputs (segment list, deviation
    # parameters) and a device-to-host read of the exit waves.
    host = torch.empty((n_e, geo["Ny"], geo["Nx"]), dtype=torch.complex64,
                       pin_memory=True)
    s_host = np.asarray(s, float)

    def e2e():
        # the exit waves land in pinned host memory, copied row chunk by
        # row chunk while the march proceeds
        solve_dislocation(segs, s_host, grid, x, precision=FP32,
                          h_mode="staged", h_sum="fp64", batch=n_e,
                          host_out=host)
        torch.cuda.synchronize()
    for _ in range(2):
        e2e()
    ke = max(3, args.steps // 4)
    t0 = time.perf_counter()
    for _ in range(ke):
        e2e()
    e2e_s = max_over_ranks((time.perf_counter() - t0) / ke, world)

    # Roofline of the dominant kernel (the march): 40 flops per voxel-step
    # (the 2 x 2 complex propagator and two complex coupling products),
    # over the march kernel's own duration; the staging kernel beside it:
    # 40 flops per segment-voxel of Volterra phase (atan2 and log not
    # counted).
    march_flops = 40.0 * units
    stage_flops = 40.0 * n_seg * voxels
    achieved = march_flops / (march_ms * 1e-3) / 1e12
    stage_tf = stage_flops / (stage_ms * 1e-3) / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": "voxel-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (compensated) + f64 H sum",
        "data": "synthetic (seeded geometry of the benchmark configuration)",
        "config": {"workload": WORKLOAD, "angles": n_e, "segments": n_seg,
                   "active_rows": int(len(rows)), "Nx": geo["Nx"],
                   "Nz": geo["Nz"], "voxel_steps_per_step": units,
                   "form": "FP32 compensated march (Fast2Sum), FP32 sincos; "
                           "segment sum of H and its 2 pi reduction in "
                           "FP64; e^{iH} evaluated once per voxel into the "
                           "workspace, all 256 angles in one call",
                   "l2": "flushed between steps (256 MB write); the staged "
                         "e^{iH} table (2.0 GB) and the exit waves (1.2 GB) "
                         "exceed L2 anyway",
                   "parallelism": f"replicas x{world}"},
        "error_vs_fp64": {
            "intensity_rel_l2": err_I, "field_rel_l2": err_field,
            "phase_rms_rad_intensity_weighted": err_phase,
            "budget_intensity": 1e-5, "angles_compared": n_e},
        "plain_fp64": {"value": world * units / (plain_ms[0] * 1e-3),
                       "ms_per_step": plain_ms[0], "unit": "voxel-steps/s",
                       "form": "plain FP64 march, FP64 Volterra phase "
                               "staged once, all 256 angles, timed once"},
        "h_sum_float_float": {
            "value": world * units / (statistics.mean(ms_ff) * 1e-3),
            "ms_per_step": statistics.mean(ms_ff),
            "stage_ms": float(np.mean([k[1] for k in km_ff])),
            "march_ms": float(np.mean([k[2] for k in km_ff])),
            "unit": "voxel-steps/s",
            "intensity_rel_l2_vs_chosen": ff_err,
            "form": "as the chosen form, segment sum and 2 pi reduction in "
                    "float-float (two-sum) instead of FP64"},
        "kernels_ms": {"prologue": prologue_ms, "stage": stage_ms,
                       "march": march_ms,
                       "source": "CUDA events of dyfox_kernel_timing around "
                                 "each kernel of the timed calls"},
        "e2e": {"value": world * units / e2e_s, "unit": "voxel-steps/s",
                "ms_per_step": e2e_s * 1e3,
                "h2d_bytes_per_step": int(8 * n_e + chosen.table.nbytes),
                "d2h_bytes_per_step": int(host.numel() * 8),
                "call": "solve_dislocation(segs, s_dev, grid, xtal, "
                        "precision=FP32, h_mode='staged', h_sum='fp64', "
                        "batch=256, host_out=<pinned host tensor>): the "
                        "waves copied to the host row chunk by row chunk "
                        "while the march proceeds"},
        "roofline": {"bound": "fp32", "kernel": "laue_march_kernel",
                     "achieved": achieved, "peak": peaks["fp32"],
                     "unit": "TFLOP/s", "frac": achieved / peaks["fp32"],
                     "traffic": MARCH_SCAN_DRAM_BYTES,
                     "traffic_source": MARCH_SCAN_DRAM_SHAPE,
                     "peak_source": "measured FFMA throughput "
                                    "(dyfox_pipe_peak, this run); the "
                                    "measured-peaks file has HBM and bf16 "
                                    "figures only",
                     "algorithmic_flops_per_launch": march_flops,
                     "launch_ms": march_ms},
        "stage_roofline": {"bound": "fp64 (segment sum) and fp32",
                           "kernel": "cs_stage_kernel",
                           "achieved": stage_tf, "peak": peaks["fp32"],
                           "unit": "TFLOP/s",
                           "frac": stage_tf / peaks["fp32"],
                           "algorithmic_flops_per_launch": stage_flops,
                           "launch_ms": stage_ms},
        "pipe_peaks_tflops": peaks,
        "launch_shape": {"tuned": tuned or None,
                         "autotuner": "dyfox_gb300.autotune (cols per lane x "
                                      "angles per CTA, each timed at about "
                                      "2048 CTAs)"},
        "gpu_launches": int(launches),
        "wall_s": wall,
    }
    line["clocks"] = clk.summary()
    del chosen
    torch.cuda.empty_cache()
    if not args.no_readme:
        line["laue_readme"] = readme_leg(args, world, peaks)
    if rank == 0 and world == 1 and not args.no_reference_gpu:
        line["reference_gpu"] = reference_gpu_of_child(value, line)
    if not args.no_bragg:
        line["bragg"] = bragg_leg(args, rank, world, peaks)
    if not args.no_com_maps:
        line["com_maps"] = com_maps_leg(args, world)
    if not args.no_batched:
        line["batched"] = batched_leg(args, world)
    if not args.no_learned:
        line["learned_guess"] = learned_leg(args, world)
        line["unet_conv"] = conv_leg()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(x, grid, segs, s,
                                            args.cpu_seconds)
        rx, rgrid, rseg, rs = readme_workload()
        hv = (line.get("laue_readme") or {}).get("h_variants")
        line["volterra"] = volterra_leg(rx, rgrid, rseg, hv,
                                        min(3.0, args.cpu_seconds))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def reference_gpu_of_child(value, line):
    """The reference kernel on this GPU, timed by the reference arm in a
    child process (``--impl reference --reference-gpu``), and this arm's
    rates over it at both Laue workloads."""
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl",
           "reference", "--reference-gpu"]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=900)
        ref = json.loads(r.stdout.strip().splitlines()[-1])
    except Exception as e:                      # report, do not fail
        return {"unavailable": f"reference-kernel child failed: {e}"}
    if "unavailable" in ref:
        return ref
    scan, readme = ref.get("scan", {}), ref.get("readme", {})
    rm = line.get("laue_readme") or {}
    out = dict(ref)
    ratios = {}
    for prec in ("fp64", "fp32"):
        if prec in scan:
            ratios[f"scan_chosen_over_ref_{prec}_march"] = \
                value / scan[prec]["march_value"]
            ratios[f"scan_chosen_over_ref_{prec}_with_h_grid"] = \
                value / scan[prec]["with_h_grid_value"]
        if prec in readme and rm.get("value"):
            ratios[f"readme_chosen_over_ref_{prec}_march"] = \
                rm["value"] / readme[prec]["march_value"]
    if "fp64" in scan:
        ratios["scan_plain_fp64_over_ref_fp64_march"] = \
            line["plain_fp64"]["value"] / scan["fp64"]["march_value"]
    if "fp64" in readme and rm.get("plain_fp64"):
        ratios["readme_plain_fp64_over_ref_fp64_march"] = \
            rm["plain_fp64"]["value"] / readme["fp64"]["march_value"]
    out["ratio"] = ratios
    return out


def readme_leg(args, world, peaks):
    """The README-size Laue drop-in (544 x 800, Nz 359, one edge
    dislocation, 2 angles): the FP32 compensated march with the Volterra
    phase fused into it (float-float segment sum, and the FP64 sum beside
    it), plain FP64, e2e through solve_dislocation, and the fused phase
    against a stored H grid (h_variants)."""
    import torch
    from dyfox_gb300 import _lib
    from dyfox_gb300.backend import FP32, FP64
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import solve_dislocation
    x, grid, seg, s = readme_workload()
    geo = grid_arrays(grid)
    rows = active_rows(geo)
    n_e = len(s)
    units = n_e * len(rows) * geo["Nx"] * (geo["Nz"] - 1)
    voxels = len(rows) * geo["Nx"] * (geo["Nz"] - 1)
    if not args.no_tune:
        from dyfox_gb300.autotune import tune
        for prec in (FP32, FP64):
            tune(seg, s, grid, x, precision=prec, h_mode="fused")
    fused = _lib.FLAG_FUSED
    ff = LaueCall(x, geo, seg, s, FP32, fused)
    plain = LaueCall(x, geo, seg, s, FP64, fused)
    sum64 = LaueCall(x, geo, seg, s, FP32, fused | _lib.FLAG_H_FP64)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ms, km, _ = timed_steps(ff, args.steps, args.warmup, flush,
                            kernel_ms=True)
    ms_plain, _, _ = timed_steps(plain, max(3, args.steps // 4), 2, flush)
    ms_64, _, _ = timed_steps(sum64, max(3, args.steps // 4), 2, flush)
    err = _intensity_err(ff.out, plain.out)
    err64 = _intensity_err(sum64.out, plain.out)
    t = 1e3 * max_over_ranks(statistics.mean(ms) * 1e-3, world)
    host = torch.empty((n_e, geo["Ny"], geo["Nx"]), dtype=torch.complex64,
                       pin_memory=True)

    def e2e():
        o = solve_dislocation(seg, np.asarray(s, float), grid, x,
                              precision=FP32, h_mode="fused")
        host.copy_(o)
        torch.cuda.synchronize()
    for _ in range(2):
        e2e()
    t0 = time.perf_counter()
    ke = max(3, args.steps // 2)
    for _ in range(ke):
        e2e()
    e2e_s = (time.perf_counter() - t0) / ke
    march_ms = float(np.mean([k[2] for k in km]))
    flops = 40.0 * units + 40.0 * len(ff.table) * voxels
    return {
        "value": world * units / (t * 1e-3), "unit": "voxel-steps/s",
        "ms_per_step": t, "workload": README_WORKLOAD,
        "voxel_steps_per_step": units,
        "form": "FP32 compensated march, Volterra phase fused into the "
                "march (float-float segment sum and 2 pi reduction)",
        "intensity_rel_l2_vs_fp64": err,
        "plain_fp64": {"value": world * units /
                       (statistics.mean(ms_plain) * 1e-3),
                       "ms_per_step": statistics.mean(ms_plain)},
        "fp32_with_fp64_h_sum": {
            "value": world * units / (statistics.mean(ms_64) * 1e-3),
            "ms_per_step": statistics.mean(ms_64),
            "intensity_rel_l2_vs_fp64": err64},
        "e2e": {"value": world * units / e2e_s, "ms_per_step": e2e_s * 1e3,
                "h2d_bytes_per_step": int(8 * n_e + ff.table.nbytes),
                "d2h_bytes_per_step": int(host.numel() * 8)},
        "roofline": {"bound": "fp32", "kernel": "laue_march_kernel",
                     "achieved": flops / (march_ms * 1e-3) / 1e12,
                     "peak": peaks["fp32"], "unit": "TFLOP/s",
                     "frac": flops / (march_ms * 1e-3) / 1e12
                     / peaks["fp32"],
                     "launch_ms": march_ms,
                     "algorithmic_flops_per_launch": flops,
                     "note": "march and fused phase in one kernel: 40 flops "
                             "per voxel-step + 40 per segment-voxel"},
        "h_variants": readme_h_variants(seg, s, grid, x),
    }


def run_once(args):
    """One small, fixed case of one form after one warm-up (for ncu)."""
    import torch
    from dyfox_gb300.backend import FP32, FP64
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import solve_dislocation
    if args.once in ("fp32", "fp64"):
        x, grid, seg, s = readme_workload()
        geo = grid_arrays(grid)
        from dyfox_gb300 import _lib
        fn = LaueCall(x, geo, seg, s, FP32 if args.once == "fp32" else FP64,
                      _lib.FLAG_FUSED)
        for _ in range(2):
            fn()
            torch.cuda.synchronize()
        return
    if args.once in ("scan", "scan256"):
        # scan256: the headline's launch at the shape the autotuner picks
        # for it (11 columns per lane; 8 angles per CTA requested, 4 fit)
        from dyfox_gb300.laue import _solve
        from dyfox_gb300.workloads import laue_rocking_scan
        sx, sgrid, ssegs, ss = laue_rocking_scan(
            n_angles=32 if args.once == "scan" else 256)
        shape = {} if args.once == "scan" else dict(cols_per_lane=11,
                                                    angles_per_cta=8)
        for _ in range(2):
            _solve(ssegs, ss, sgrid, sx, None, len(ss), "fp32", False,
                   h_mode="staged", h_sum="fp64", tuned=False, **shape)
            torch.cuda.synchronize()
        return
    if args.once == "hgrid":
        from dyfox_gb300.dislocations import compute_H_grid
        from dyfox_gb300.grid import LaueGrid
        rx, rgrid, rseg, rs = readme_workload()
        small = LaueGrid(rx, 100e-6, 0.25e-6, 60e-6)
        for _ in range(2):
            compute_H_grid(rseg, small, rx)
            torch.cuda.synchronize()
        return
    if args.once == "image":
        from dyfox_gb300.optics import Optics, image_intensity
        from dyfox_gb300.workloads import laue_rocking_scan
        sx, sgrid, ssegs, ss = laue_rocking_scan(n_angles=16)
        stack = solve_dislocation(ssegs, ss, sgrid, sx, precision="fp32",
                                  h_mode="staged", batch=len(ss))
        lens = Optics(NA=1e-4, f_lens=0.274, xtal=sx, precision="fp32")
        pup = lens.spiral(stack.shape[-1], stack.shape[-2], sgrid.dx, 2)
        for _ in range(2):
            image_intensity(stack, pup)
            torch.cuda.synchronize()
        return
    if args.once in ("bragg", "bragg32", "bragg32-scan"):
        # 4 deviation parameters x 8 planes, or (bragg32-scan) the whole
        # 20 um scan, 21 x 64, in mixed precision
        from dyfox_gb300.bragg import solve_scan
        bx, bcfg, bseg, bs, bys, bg = bragg_workload()
        prec = "fp64" if args.once == "bragg" else "fp32"
        full = args.once == "bragg32-scan"
        for _ in range(2):
            solve_scan(bseg, bs if full else bs[:4], bcfg,
                       bys if full else bys[:8], bx, bg, precision=prec)
            torch.cuda.synchronize()
        return
    if args.once == "batch":
        # the first 12 Laue instances of the batched-uneven set, one graph
        from dyfox_gb300.batch import Batch, from_workload
        from dyfox_gb300.workloads import batched_uneven
        W = [w for w in batched_uneven() if w["kind"] == "laue"][:12]
        b = Batch(from_workload(W), h_sum="fp64")
        for _ in range(2):
            b.run()
        torch.cuda.synchronize()
        return
    if args.once == "unet":
        # two training steps of the U-Net at batch 8 x 256 x 256
        from dyfox_gb300.learned import UNet
        torch.manual_seed(0)
        net = UNet(batch=8, H=256, W=256, seed=3)
        xin = (torch.randn(8, 256, 256, 32, device="cuda") * 0.5).to(
            torch.bfloat16)
        tgt = torch.randn(8, 256, 256, 2, device="cuda")
        for _ in range(2):
            net.forward(xin)
            net.backward(tgt)
            net.step(1e-3)
        torch.cuda.synchronize()
        return


def _fp64_row_checks(W, outs, n_streams=16):
    """Per Laue instance: plain FP64 solve of the central row at the first
    and last deviation parameter (one fused launch each, spread over
    streams, own workspaces), and the exit-intensity relative L2 of the
    batch's row against it."""
    import torch
    from dyfox_gb300 import _lib
    from dyfox_gb300.backend import FP64
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import _desc
    L = _lib.lib()
    streams = [torch.cuda.Stream() for _ in range(n_streams)]
    pend = []
    for k, (w, out) in enumerate(zip(W, outs)):
        x = w["xtal"]
        geo = grid_arrays(w["grid"])
        geo["fov_hy"] = 0.5 * geo["dx"]          # the row Ny / 2 only
        sel = sorted({0, len(w["s"]) - 1})
        tab = _lib.segment_table(w["segs"], x.g_vec, x.nu, x.a_core,
                                 geo["dx"])
        src = _lib.H_SEGMENTS if len(tab) else _lib.H_NONE
        d = _desc(x, geo, len(sel), FP64, src, len(tab), None,
                  _lib.FLAG_FUSED)
        st = streams[k % n_streams]
        with torch.cuda.stream(st):
            table = _lib.device_table(tab) if len(tab) else None
            sd = torch.tensor(np.asarray(w["s"])[sel], dtype=torch.float64,
                              device="cuda")
            ws = torch.empty(max(L.dyfox_laue_workspace_bytes(d), 256),
                             dtype=torch.uint8, device="cuda")
            ref = torch.empty((len(sel), geo["Ny"], geo["Nx"]),
                              dtype=torch.complex128, device="cuda")
            _lib.check(L.dyfox_laue_solve(
                d, _lib.ptr(sd), None, _lib.ptr(table), _lib.ptr(ref),
                _lib.ptr(ws), ws.numel(), _lib.c_void_p(st.cuda_stream)),
                "dyfox_laue_solve")
        pend.append((ref, out, sel, geo["Ny"] // 2, table, sd, ws))
    torch.cuda.synchronize()
    errs = []
    for ref, out, sel, r, *_ in pend:
        a = (out[sel, r].to(torch.complex128).abs() ** 2)
        b = ref[:, r].abs() ** 2
        errs.append(float(torch.linalg.vector_norm(a - b) /
                          max(float(torch.linalg.vector_norm(b)), 1e-300)))
    return errs


def _instance_shape(w):
    """Sizes of one Laue instance of the batched set, for the report."""
    from dyfox_gb300.grid import grid_arrays
    geo = grid_arrays(w["grid"])
    return {"Nx": geo["Nx"], "Ny": geo["Ny"], "Nz": geo["Nz"],
            "t_um": w["grid"].t_crystal * 1e6, "dx_um": w["grid"].dx * 1e6,
            "segments": len(w["segs"]), "angles": len(w["s"])}


def batched_leg(args, world):
    """Batched uneven instances: 512 seeded instances (70% Laue, 30% Bragg),
    one CUDA graph per replay (per-instance set-up, one persistent Laue
    march launch, one Bragg launch).  Laue: compensated FP32 march
    (complex64 state) with an FP64-class H: the segment sum and 2 pi
    reduction in IEEE double (``--batched-h-sum fp64``, the chosen form) or
    in float-float (``ff``); the Laue part is timed alone in both.  Bragg:
    mixed-precision solve to true residual 1e-10.  Launch shape
    from the batch autotuner.  Per-instance error against plain FP64 (Laue:
    central row at the first and last angle; Bragg: every system); a
    sample of the instances is also timed as plain FP64 single calls and as
    FP32 single calls."""
    import torch
    from dyfox_gb300 import _lib
    from dyfox_gb300.batch import Batch, autotune, from_workload
    from dyfox_gb300.bragg import solve_scan
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import solve_dislocation
    from dyfox_gb300.workloads import batched_uneven
    L = _lib.lib()
    hs = args.batched_h_sum
    W = batched_uneven()
    if args.batched_sample:
        W = W[:args.batched_sample]
    inst = from_workload(W)
    t0 = time.perf_counter()
    if args.no_tune:
        tuned = {"cols_per_lane": 5, "warps": 8, "ms": None}
    else:
        tuned = autotune(inst, h_sum=hs)
    tune_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = Batch(inst, cols_per_lane=tuned["cols_per_lane"],
              warps=tuned["warps"], h_sum=hs)
    plan_s = time.perf_counter() - t0
    for _ in range(2):
        b.run()
    torch.cuda.synchronize()
    steps = 3
    times = []
    n0 = L.dyfox_launch_count()
    for _ in range(steps):
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record()
        b.run()
        a1.record()
        torch.cuda.synchronize()
        times.append(a0.elapsed_time(a1))
    launches = (L.dyfox_launch_count() - n0) // steps
    ms = 1e3 * max_over_ranks(statistics.mean(times) * 1e-3, world)
    laue_vs, bragg_solves, bragg_sys = 0, 0, 0
    for w in W:
        if w["kind"] == "laue":
            geo = grid_arrays(w["grid"])
            rows = int(np.sum(np.abs((np.arange(geo["Ny"]) - geo["Ny"] // 2)
                                     * geo["dx"]) < geo["fov_hy"]))
            laue_vs += len(w["s"]) * rows * geo["Nx"] * (geo["Nz"] - 1)
        else:
            bragg_solves += len(w["s"])
            bragg_sys += len(w["s"]) * len(w["ys"])
    li = [i for i, w in enumerate(W) if w["kind"] == "laue"]
    bi = [i for i, w in enumerate(W) if w["kind"] == "bragg"]
    # the two parts alone (each its own graph)
    part_ms = {}
    other = "fp64" if hs == "ff" else "ff"
    for key, idx, h in (("laue", li, hs), ("bragg", bi, hs),
                        ("laue_" + other, li, other)):
        if not idx:
            continue
        pb = Batch([inst[i] for i in idx],
                   cols_per_lane=tuned["cols_per_lane"],
                   warps=tuned["warps"], h_sum=h)
        pb.run()
        torch.cuda.synchronize()
        a0 = torch.cuda.Event(enable_timing=True)
        a1 = torch.cuda.Event(enable_timing=True)
        a0.record()
        for _ in range(2):
            pb.run()
        a1.record()
        torch.cuda.synchronize()
        part_ms[key] = 1e3 * max_over_ranks(a0.elapsed_time(a1) * 5e-4,
                                            world)
        pb.close()
        del pb
    # per-instance error against FP64
    t0 = time.perf_counter()
    laue_err = _fp64_row_checks([W[i] for i in li], [b.outputs[i] for i in li])
    bragg_err, bragg_res = [], []
    for i in bi:
        w = W[i]
        ref, _ = solve_scan(w["segs"], w["s"], w["cfg"], w["ys"], w["xtal"],
                            w["g"])
        bragg_err.append(float(torch.linalg.vector_norm(b.outputs[i] - ref) /
                               torch.linalg.vector_norm(ref)))
        bragg_res.append(float(b.infos[i][:, 0].max()))
    check_s = time.perf_counter() - t0
    # a sample as single calls: plain FP64 and FP32
    samp = li[:12] + bi[:6]
    sub = Batch([inst[i] for i in samp], cols_per_lane=tuned["cols_per_lane"],
                warps=tuned["warps"], h_sum=hs)
    sub.run()
    torch.cuda.synchronize()

    def wall(fn):
        torch.cuda.synchronize()
        t = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) * 1e3

    def singles(prec):
        for i in samp:
            w = W[i]
            if w["kind"] == "laue":
                solve_dislocation(w["segs"], w["s"], w["grid"], w["xtal"],
                                  precision=prec,
                                  h_sum=hs if prec == "fp32" else "ff")
            else:
                solve_scan(w["segs"], w["s"], w["cfg"], w["ys"], w["xtal"],
                           w["g"], precision=prec)
    sub_ms = wall(sub.run)
    single32_ms = wall(lambda: singles("fp32"))
    single64_ms = wall(lambda: singles("fp64"))
    sec = ms * 1e-3
    return {
        "instances": len(W), "laue": len(li), "bragg": len(bi),
        "ms_per_batch": ms, "instances_per_s": world * len(W) / sec,
        "laue_voxel_steps": laue_vs,
        "bragg_solves": bragg_solves, "bragg_systems": bragg_sys,
        "laue_part_alone": {
            "ms": part_ms.get("laue"),
            "voxel_steps_per_s": world * laue_vs / (part_ms["laue"] * 1e-3)
            if "laue" in part_ms else None},
        "laue_part_alone_h_sum_" + other: {
            "ms": part_ms.get("laue_" + other),
            "voxel_steps_per_s":
                world * laue_vs / (part_ms["laue_" + other] * 1e-3)
                if "laue_" + other in part_ms else None},
        "bragg_part_alone": {
            "ms": part_ms.get("bragg"),
            "solves_per_s": world * bragg_solves / (part_ms["bragg"] * 1e-3)
            if "bragg" in part_ms else None},
        "form": "one CUDA graph per replay: per-instance set-up, one "
                "persistent Laue march launch (compensated FP32, segment sum "
                "and 2 pi reduction " + ("in float-float, FP64-class"
                                         if hs == "ff" else "in double") +
                ", e^{iH} of each row evaluated once by the CTA that "
                "marches it), one mixed-precision Bragg launch",
        "h_sum": hs,
        "launch_shape": {"cols_per_lane": tuned["cols_per_lane"],
                         "warps": tuned["warps"], "tuner_ms": tuned["ms"],
                         "tuner_s": tune_s},
        "plan_s": plan_s, "gpu_launches": int(launches),
        "laue_intensity_rel_l2_vs_fp64": {
            "max": max(laue_err) if laue_err else None,
            "median": float(np.median(laue_err)) if laue_err else None,
            "worst": _instance_shape(W[li[int(np.argmax(laue_err))]])
            if laue_err else None,
            "checked": "central row, first and last angle, every instance"},
        "bragg_rel_l2_vs_fp64": {
            "max": max(bragg_err) if bragg_err else None,
            "median": float(np.median(bragg_err)) if bragg_err else None,
            "max_true_residual": max(bragg_res) if bragg_res else None},
        "fp64_checks_s": check_s,
        "sample": {"instances": len(samp), "batched_ms": sub_ms,
                   "fp32_single_calls_ms": single32_ms,
                   "fp64_single_calls_ms": single64_ms,
                   "timing": "host wall clock, synchronised"},
    }


def conv_leg(reps=20):
    """The U-Net's widest 3x3 convolution (e0b: batch 8 x 256 x 256, 32 ->
    32 channels) forward and weight gradient, and the data gradient of d2a
    (batch 8 x 64 x 64, 128 -> 384 channels), on the tcgen05 tensor cores
    and with the mma.sync implicit GEMM, CUDA events, L2 flushed between
    launches (the weight gradient's time includes its split reduction).
    Flops = 2 M N K; bytes = the activations read and written once and the
    weights."""
    import torch
    from dyfox_gb300.learned import conv, tc_error
    peak, src = bf16_peak()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    g = torch.Generator(device="cuda").manual_seed(3)
    res = {}
    for name, (N, H, W, Cin, Cout, mode) in (
            ("e0b_fwd", (8, 256, 256, 32, 32, "fwd")),
            ("e0b_wgrad", (8, 256, 256, 32, 32, "wgrad")),
            ("d2a_dgrad", (8, 64, 64, 384, 128, "dgrad"))):
        if mode == "wgrad":
            X = torch.randn(N, H, W, Cin, device="cuda", generator=g).to(
                torch.bfloat16)
            G = torch.randn(N, H, W, Cout, device="cuda", generator=g).to(
                torch.bfloat16)
            kw = dict(X=X, G=G, Cin=Cin, Cout=Cout)
            Ncols, K = Cout, N * H * W          # M = 9 Cin
            nbytes = 2 * N * H * W * (Cin + Cout) + 4 * 9 * Cin * Cout
        elif mode == "fwd":
            X = torch.randn(N, H, W, Cin, device="cuda", generator=g).to(
                torch.bfloat16)
            Wk = (0.1 * torch.randn(Cout, 9, Cin, device="cuda",
                                    generator=g)).to(torch.bfloat16)
            b = torch.zeros(Cout, device="cuda")
            kw = dict(X=X, Wk=Wk, bias=b, Cout=Cout)
            Ncols, K = Cout, 9 * Cin
            nbytes = 2 * N * H * W * (Cin + Cout) + 2 * Wk.numel()
        else:
            G = torch.randn(N, H, W, Cout, device="cuda", generator=g).to(
                torch.bfloat16)
            Wk = (0.1 * torch.randn(Cin, 9, Cout, device="cuda",
                                    generator=g)).to(torch.bfloat16)
            kw = dict(G=G, Wk=Wk, Cin=Cin, Cout=Cout)
            Ncols, K = Cin, 9 * Cout
            nbytes = 2 * N * H * W * Cout + 4 * N * H * W * Cin + \
                2 * Wk.numel()
        flops = 2.0 * (9 * Cin if mode == "wgrad" else N * H * W) * Ncols * K
        entry = {"shape_N_H_W_Cin_Cout": [N, H, W, Cin, Cout],
                 "gflop": flops * 1e-9, "bytes": nbytes}
        for form, mma in (("tcgen05", False), ("mma_sync", True)):
            for _ in range(3):
                conv(mode, mma_sync=mma, **kw)
            ts = []
            for _ in range(reps):
                flush.zero_()
                a = torch.cuda.Event(enable_timing=True)
                c = torch.cuda.Event(enable_timing=True)
                a.record()
                conv(mode, mma_sync=mma, **kw)
                c.record()
                torch.cuda.synchronize()
                ts.append(a.elapsed_time(c))
            ms = statistics.median(ts)
            tf = flops / (ms * 1e-3) / 1e12
            entry[form] = {"ms": ms, "tflops": tf, "frac_bf16_peak": tf / peak,
                           "hbm_gbs": nbytes / (ms * 1e-3) / 1e9}
        res[name] = entry
    res["peak_tflops"] = peak
    res["peak_source"] = src
    res["tc_error"] = tc_error(clear=True)
    return res


def bf16_peak():
    """(TFLOP/s, source) of the bf16 GEMM rate measured on this machine."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                        "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["bf16_tflops"]), \
                "MEASURED_PEAKS.json bf16_tflops"
    except (OSError, ValueError, KeyError):
        return 1900.0, "fallback 1.9 PFLOP/s"


def learned_leg(args, world):
    """Learned shooting guess (Bragg, dx 0.25 um, 256 planes x 256 px
    field, 1-32 segments within 5 um of the surface, 64 s over +-5 Darwin
    widths; thickness 10 um .. ``--learned-tmax``).  Training data: the
    plain solves (zero start, mixed precision, true residual 1e-6, ample
    for a starting guess) of ``--learned-train`` instances, each giving 64
    samples at the field of interest and at 2 more lateral windows; the
    U-Net is trained on the GPU by the library's kernels.  On
    ``--learned-test`` held-out instances every system is solved to true
    residual 1e-8 from the zero start (plain), the perfect-crystal start
    and the learned start (the network applied to the whole periodic
    lateral grid; inference included in its time), in the mixed-precision
    form, and from the zero start in plain FP64.  r0 = |A x0 + d| / |d| is
    the initial shooting residual of each start (the zero start's is 1)."""
    import torch
    from dyfox_gb300 import learned as Lm
    from dyfox_gb300.bragg import apply_operator
    from dyfox_gb300.workloads import learned_guess_instances
    inst = learned_guess_instances(args.learned_train + args.learned_test,
                                   t_range=(10e-6, args.learned_tmax))
    train, test = inst[:args.learned_train], inst[args.learned_train:]
    rng = np.random.default_rng(0)
    t0 = time.perf_counter()
    Xs, Ts, it_train = [], [], []
    for w in train:
        h = Lm.instance_h(w)
        v, info, _ = Lm.solve_instance(w, tol=1e-6)
        Nx = w["cfg"].Nx
        for c0 in [w["col0"]] + [int(rng.integers(0, Nx)) for _ in range(2)]:
            X, h0, v0 = Lm.instance_inputs(w, col0=c0, h=h)
            Xs.append(X)
            Ts.append(Lm.targets(v, h0, v0, c0, w["field"]))
        it_train.append(float(info[:, 1].float().mean()))
        del v, info, h
    X = torch.cat(Xs)
    T = torch.cat(Ts)
    del Xs, Ts
    data_s = time.perf_counter() - t0
    net = Lm.UNet(batch=8, H=256, W=256, seed=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    hist = net.train(X, T, epochs=args.learned_epochs, lr=1e-3,
                     decay_every=max(1, args.learned_epochs // 3))
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    n_samples = X.shape[0]
    target_var = float(T.pow(2).mean())
    del X, T

    def r0(w, x0):
        if x0 is None:
            return 1.0
        inc = torch.ones((len(w["s"]), len(w["ys"]), w["cfg"].Nx),
                         dtype=torch.complex128, device="cuda")
        d = apply_operator(w["segs"], w["s"], w["cfg"], w["ys"], w["xtal"],
                           w["g"], "march", in0=inc)
        Ax = apply_operator(w["segs"], w["s"], w["cfg"], w["ys"], w["xtal"],
                            w["g"], "march", in1=x0)
        return float(torch.linalg.vector_norm(Ax + d)
                     / torch.linalg.vector_norm(d))

    rows = []
    for w in test:
        h = Lm.instance_h(w)
        _, h0, v0 = Lm.instance_inputs(w, h=h)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        Lm.predict_full(net, w, h=h, batch=4)          # builds the wide net
        a.record()
        y = Lm.predict_full(net, w, h=h, batch=4)
        x0 = Lm.initial_guess(w, v0, y, col0=0)
        b.record()
        torch.cuda.synchronize()
        infer_ms = a.elapsed_time(b)
        row = {"Nz": w["cfg"].Nz, "Nx": w["cfg"].Nx,
               "segments": len(w["segs"]), "inference_ms": infer_ms}
        for name, start, prec in (("zero", None, "fp32"),
                                  ("pristine", Lm.initial_guess(w, v0), "fp32"),
                                  ("learned", x0, "fp32"),
                                  ("zero_fp64", None, "fp64")):
            v, info, ms = Lm.solve_instance(w, x0=start, tol=1e-8,
                                            precision=prec)
            inf = info.cpu().numpy()
            row[name] = {"ms": ms + (infer_ms if name == "learned" else 0.0),
                         "iterations_mean": float(inf[:, 1].mean()),
                         "iterations_max": int(inf[:, 1].max()),
                         "max_true_residual": float(inf[:, 0].max()),
                         "converged": bool((inf[:, 2] == 0).all()),
                         "r0": r0(w, start)}
            del v, info
        rows.append(row)
        del h, y, x0

    def tot(key, f):
        return sum(r[key][f] for r in rows)
    n_solves = sum(len(w["s"]) for w in test)
    keys = ("zero", "pristine", "learned", "zero_fp64")
    return {
        "train_instances": len(train), "train_samples": n_samples,
        "test_instances": len(test), "test_solves": n_solves,
        "planes": len(inst[0]["ys"]), "field_px": inst[0]["field"],
        "t_range_um": [10.0, args.learned_tmax * 1e6],
        "data_generation_s": data_s, "training_s": train_s,
        "epochs": args.learned_epochs, "loss_first_epoch": hist[0],
        "loss_last_epoch": hist[-1],
        "loss_of_predicting_zero": 0.5 * target_var,
        "train_iterations_mean": float(np.mean(it_train)),
        "per_instance": rows,
        "iterations_mean": {k: tot(k, "iterations_mean") / len(rows)
                            for k in keys},
        "r0_mean": {k: tot(k, "r0") / len(rows) for k in keys},
        "bragg_solves_per_s": {k: world * n_solves / (tot(k, "ms") * 1e-3)
                               for k in keys},
        "form": "learned start: mixed-precision solve from v0 + U-Net "
                "prediction on the whole lateral grid, inference included; "
                "zero_fp64: plain FP64 from the zero start (the repo's "
                "start); tolerance 1e-8",
        "reading": "the configuration trains on 20k solves of thickness "
                   "10-100 um; this leg trains on --learned-train x 64 "
                   "solves up to --learned-tmax so that the default bench "
                   "stays within minutes",
    }


def readme_h_variants(seg, s, grid, x, reps=5):
    """The README step (FP32 compensated march) with the Volterra phase
    fused into the march, against e^{iH} staged once in the workspace and
    against the reference's layout: the whole H grid (Ny, Nz, Nx) built in
    HBM first (compute_H_grid, float32 or float64) and read by the march.
    All through solve_dislocation, L2 flushed before each call; ms medians
    and the intensity error of each against the plain FP64 solve."""
    import torch
    from dyfox_gb300.dislocations import compute_H_grid
    from dyfox_gb300.laue import solve_dislocation
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ref = solve_dislocation(seg, s, grid, x, precision="fp64")
    I64 = ref.abs() ** 2

    def timed(fn, check=True):
        fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            out = fn()
            b.record()
            torch.cuda.synchronize()
            ts.append(a.elapsed_time(b))
        if not check:
            return statistics.median(ts), None
        I = out.abs().double() ** 2
        err = float(torch.linalg.vector_norm(I - I64) /
                    torch.linalg.vector_norm(I64))
        return statistics.median(ts), err

    res = {}
    for name, mode in (("fused", "fused"), ("staged_cs", "staged")):
        ms, err = timed(lambda: solve_dislocation(seg, s, grid, x,
                                                  precision="fp32",
                                                  h_mode=mode))
        res[name] = {"ms": ms, "intensity_rel_l2": err}
    for name, hp in (("h_grid_f32", "fp32"), ("h_grid_f64", "fp64")):
        H = compute_H_grid(seg, grid, x, precision=hp)
        h_ms, _ = timed(lambda: compute_H_grid(seg, grid, x, precision=hp),
                        check=False)
        m_ms, err = timed(lambda: solve_dislocation(seg, s, grid, x,
                                                    H_gpu=H,
                                                    precision="fp32"))
        res[name] = {"ms": h_ms + m_ms, "h_grid_ms": h_ms, "march_ms": m_ms,
                     "h_grid_bytes": int(H.numel() * H.element_size()),
                     "intensity_rel_l2": err}
        del H
    return res


def hbm_peak():
    """(GB/s, source) of the HBM copy rate measured on this machine, else the
    fallback figure."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                        "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s"


def com_maps_leg(args, world):
    """Centre-of-mass maps (analysis.rocking.com_maps) of the 256-angle
    rocking scan of the scan leg through spiral-plate charges 0 and 2 (NA
    1e-4, f 0.274 m): the FP32 march of all angles in one call, the images
    and the fused double-precision reduction, ending with the maps on the
    host.  The imaging pass is also timed alone on resident exit waves (16
    per launch, L2 flushed between launches) for its roofline: 8 bytes read
    and 4 written per pixel.  Accuracy: maps from 16 of the angles against
    the same maps in FP64, over the pixels holding 99% of the weight."""
    import torch
    from dyfox_gb300 import _lib
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import solve_dislocation
    from dyfox_gb300.optics import Optics, image_intensity
    from dyfox_gb300.rocking import com_maps
    from dyfox_gb300.workloads import laue_rocking_scan
    x, grid, segs, s = laue_rocking_scan()
    geo = grid_arrays(grid)
    Ny, Nx = geo["Ny"], geo["Nx"]
    ells = (0, 2)
    lens = Optics(NA=1e-4, f_lens=0.274, xtal=x, precision="fp32")
    L = _lib.lib()
    stream = torch.cuda.current_stream()

    def run(ss, prec="fp32"):
        return com_maps(segs, ss, grid, x, lens if prec == "fp32" else
                        Optics(NA=1e-4, f_lens=0.274, xtal=x), ells,
                        precision=prec, h_mode="staged")

    run(s)
    torch.cuda.synchronize()
    times = []
    n0 = L.dyfox_launch_count()
    steps = max(3, args.steps // 8)
    for _ in range(steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        run(s)
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    launches = (L.dyfox_launch_count() - n0) // steps
    ms = 1e3 * max_over_ranks(statistics.mean(times) * 1e-3, world)

    # Imaging alone: 16 resident exit waves per launch through one pupil.
    chunk = 16
    stack = solve_dislocation(segs, s[:chunk], grid, x, precision="fp32",
                              h_mode="staged", batch=chunk)
    pup = lens.spiral(Nx, Ny, grid.dx, 2)
    image_intensity(stack, pup)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    itimes = []
    for _ in range(max(5, args.steps)):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        image_intensity(stack, pup)
        b.record(stream)
        torch.cuda.synchronize()
        itimes.append(a.elapsed_time(b))
    ims = statistics.median(itimes)
    alg_bytes = chunk * Ny * Nx * (8 + 4)
    peak, src = hbm_peak()
    achieved = alg_bytes / (ims * 1e-3) / 1e9

    # Accuracy on 16 angles: FP32 maps against FP64 maps.
    pick = np.linspace(0, len(s) - 1, 16).round().astype(int)
    c32, r32, w32 = run(s[pick])
    c64, r64, w64 = run(s[pick], "fp64")
    dev = {}
    for e in ells:
        w = w64[e].ravel()
        order = np.argsort(w)[::-1]
        keep = order[:np.searchsorted(np.cumsum(w[order]), 0.99 * w.sum()) + 1]
        dev[str(e)] = float(np.abs(c32[e].ravel()[keep]
                                   - c64[e].ravel()[keep]).max())
    return {"value": world * len(s) / (ms * 1e-3), "unit": "scan angles/s",
            "ms_per_scan": ms, "angles": len(s), "charges": list(ells),
            "Ny": Ny, "Nx": Nx, "gpu_launches": int(launches),
            "form": "FP32 march of all angles in one call (e^{iH} staged "
                    "once), batched 2-D FFT imaging per charge, fused "
                    "double-precision sums of phi I and I, maps to host",
            "imaging": {"images_per_s": chunk / (ims * 1e-3),
                        "ms_per_launch": ims, "images_per_launch": chunk,
                        "roofline": {"bound": "hbm", "achieved": achieved,
                                     "peak": peak, "unit": "GB/s",
                                     "frac": achieved / peak,
                                     "traffic": None,
                                     "algorithmic_bytes_per_launch":
                                         alg_bytes, "peak_source": src}},
            "max_com_deviation_urad_vs_fp64_16_angles": dev}


def bragg_flops(inf, Nx, Nz, restart):
    """Algorithmic flops of a scan's solves from the per-system inner
    iteration counts (info column 1): per inner iteration the march
    (28 (Nz - 1) Nx), the preconditioner (two Nx-point FFTs, 5 N log2 N
    each, and the 1/T22s product, 6 Nx) and modified Gram-Schmidt against
    the j + 1 basis vectors of the cycle (16 (j + 1) Nx); per system two
    more marches (right-hand side and at least one true residual).  Returns
    (Krylov-product flops, Gram-Schmidt flops)."""
    march = 28.0 * (Nz - 1) * Nx
    prec = 2 * 5.0 * Nx * np.log2(Nx) + 6.0 * Nx
    prod = mgs = 0.0
    for it in inf[:, 1].astype(int):
        prod += it * (march + prec) + 2 * march
        j = np.arange(it) % restart
        mgs += float(np.sum(16.0 * (j + 1) * Nx))
    return prod, mgs


def bragg_leg(args, rank, world, peaks=None):
    """Bragg solves/s of the 20 um scan (diamond (400), Nx 456, Nz 90): all
    21 deviation parameters x 64 planes in one batched launch (one solve =
    one deviation parameter over all planes, to true relative residual
    <= 1e-10).  The chosen form is the
    mixed-precision solve (single-precision Krylov products, float-float
    right-hand side and true residuals, double Gram-Schmidt and solution);
    plain FP64 is timed beside it, and the two answers are compared."""
    import torch
    from dyfox_gb300 import _lib
    from dyfox_gb300.bragg import solve_scan
    x, cfg, seg, s, ys, g = bragg_workload()
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    steps = max(3, args.steps // 4)

    def timed(prec):
        for _ in range(2):
            out, info = solve_scan(seg, s, cfg, ys, x, g, precision=prec)
        torch.cuda.synchronize()
        times = []
        n0 = L.dyfox_launch_count()
        for _ in range(steps):
            flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            out, info = solve_scan(seg, s, cfg, ys, x, g, precision=prec)
            b.record(stream)
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
        launches = (L.dyfox_launch_count() - n0) // steps
        return out, info.cpu().numpy(), statistics.mean(times), launches

    o32, inf, ms, launches = timed("fp32")
    o64, inf64, ms64, _ = timed("fp64")
    ms = 1e3 * max_over_ranks(ms * 1e-3, world)
    ms64 = 1e3 * max_over_ranks(ms64 * 1e-3, world)
    diff = float(torch.linalg.vector_norm(o32 - o64) /
                 torch.linalg.vector_norm(o64))
    res = {"value": world * len(s) / (ms * 1e-3), "unit": "Bragg solves/s",
           "ms_per_scan": ms, "solves_per_scan": len(s),
           "planes": len(ys), "Nx": cfg.Nx, "Nz": cfg.Nz,
           "form": "mixed precision: FP32 march + FFT preconditioner in the "
                   "Arnoldi products, float-float (FP64-class) right-hand "
                   "side and true residuals, FP64 Gram-Schmidt, rotations "
                   "and solution; per-plane GMRES(40), one launch per scan",
           "max_true_residual": float(inf[:, 0].max()),
           "max_inner_iterations": int(inf[:, 1].max()),
           "converged": bool((inf[:, 0] <= 1e-10).all()),
           "rel_l2_vs_fp64": diff,
           "gpu_launches": int(launches),
           "plain_fp64": {"value": world * len(s) / (ms64 * 1e-3),
                          "ms_per_scan": ms64,
                          "max_true_residual": float(inf64[:, 0].max()),
                          "max_inner_iterations": int(inf64[:, 1].max())}}
    if peaks:
        # Pipe roofline of both forms (TFLOP/s of the algorithmic count).
        p32, g32 = bragg_flops(inf, cfg.Nx, cfg.Nz, 40)
        p64, g64 = bragg_flops(inf64, cfg.Nx, cfg.Nz, 40)
        t32, t64 = ms * 1e-3 * 1e12, ms64 * 1e-3 * 1e12
        res["roofline"] = {
            "bound": "latency (FP32 Krylov products, FP64 Gram-Schmidt)",
            "algorithmic_gflop_per_scan": (p32 + g32) * 1e-9,
            "fp32_part_tflops": world * p32 / t32,
            "fp32_part_frac": world * p32 / t32 / peaks["fp32"],
            "fp64_part_tflops": world * g32 / t32,
            "fp64_part_frac": world * g32 / t32 / peaks["fp64"],
            "unit": "TFLOP/s", "peak_source": "measured FMA throughput "
            "(dyfox_pipe_peak, this run)"}
        res["plain_fp64"]["roofline"] = {
            "bound": "fp64", "achieved": world * (p64 + g64) / t64,
            "peak": peaks["fp64"], "unit": "TFLOP/s",
            "frac": world * (p64 + g64) / t64 / peaks["fp64"],
            "algorithmic_gflop_per_scan": (p64 + g64) * 1e-9}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        from oracle import bragg_oracle as BO
        t0 = time.perf_counter()
        _, cinfo = BO.solve_surface(seg, float(s[len(s) // 2]), cfg, ys, x,
                                    g)
        dt = time.perf_counter() - t0
        res["cpu_baseline"] = {
            "value": 1.0 / dt, "unit": "Bragg solves/s", "cores": 1,
            "kind": "port", "sample": "1 of 21 deviation parameters, 64 "
            "planes (the reference's chunked SciPy GMRES restated in "
            f"NumPy; NumPy elementwise and FFT are single-threaded), "
            f"{dt:.1f} s, {cinfo['iterations']} iterations"}
    return res


# ------------------------------------------------------------- CPU legs
def cpu_sampler(x, grid, seg, s):
    """A callable running the reference march (H + march) on `nr` rows."""
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    from dyfox_gb300.grid import grid_arrays
    from oracle import oracle as O
    O.build()
    geo = grid_arrays(grid)
    rows_all = active_rows(geo)
    kind = "reference" if O.ref_cpu() is not None else "port"

    def sample(nr):
        rows = rows_all[len(rows_all) // 2 - nr // 2:][:nr]
        H = O.h_rows(seg, x.g_vec, x.nu, x.a_core, geo["Nx"], geo["Nz"],
                     geo["dx"], geo["dz"], O.grid_y(geo["Ny"], geo["dx"],
                                                    rows))
        if kind == "reference":
            Hf = np.zeros((rows.max() + 1, geo["Nz"], geo["Nx"]))
            Hf[rows] = H
            O.ref_laue_march("fullfield", x, s, geo, H_grid=Hf, rows=rows)
        else:
            O.laue_march("fullfield", x, s, geo, H_rows=H, rows=rows)
        return len(s) * len(rows) * geo["Nx"] * (geo["Nz"] - 1)
    return sample, kind, O.num_threads()


def cpu_baseline(x, grid, seg, s, seconds):
    """The reference march on the host cores over a bounded sample of rows
    (all angles; the (row, angle) blocks spread over the cores), sized to
    about ``seconds``."""
    sample, kind, cores = cpu_sampler(x, grid, seg, s)
    t0 = time.perf_counter()
    sample(2)
    per = (time.perf_counter() - t0) / 2
    nr = int(max(2, min(481, seconds / max(per, 1e-6))))
    t0 = time.perf_counter()
    units = sample(nr)
    dt = time.perf_counter() - t0
    return {"value": units / dt, "unit": "voxel-steps/s", "cores": cores,
            "kind": kind, "sample": f"{nr} of 481 active rows x {len(s)} "
            f"angles (H of the {len(seg)} segments on those rows + FP64 "
            f"march), {dt:.1f} s"}


def volterra_leg(x, grid, seg, h_variants, seconds, max_rows=64):
    """The Volterra phase of the README workload as the H grid (Ny, Nz, Nx)
    that compute_H_grid builds: the GPU build in FP64 (its time from
    ``h_variants``) beside the oracle's C restatement of the same formula
    on all host cores, timed on blocks of ``max_rows`` central rows
    repeated for about ``seconds``.  Unit: H evaluations (segment x voxel)
    per second."""
    os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
    from dyfox_gb300.grid import grid_arrays
    from oracle import oracle as O
    O.build()
    geo = grid_arrays(grid)
    Ny, Nz, Nx = geo["Ny"], geo["Nz"], geo["Nx"]
    n_seg = len(O.segment_frames(seg, x.g_vec))
    nr = min(Ny, max_rows)
    rows = np.arange(Ny // 2 - nr // 2, Ny // 2 - nr // 2 + nr)
    y = O.grid_y(Ny, geo["dx"], rows)

    def block():
        O.h_rows(seg, x.g_vec, x.nu, x.a_core, Nx, Nz, geo["dx"], geo["dz"],
                 y)
    block()                                   # warm-up (and page-in)
    reps, t0 = 0, time.perf_counter()
    while True:
        block()
        reps += 1
        dt = time.perf_counter() - t0
        if dt >= seconds:
            break
    units = reps * nr * Nz * Nx * n_seg
    res = {"unit": "H evaluations/s", "grid": [Ny, Nz, Nx],
           "segments": n_seg,
           "cpu_baseline": {
               "value": units / dt, "unit": "H evaluations/s",
               "cores": O.num_threads(), "kind": "port",
               "sample": f"{reps} x {nr} of {Ny} rows of the FP64 H grid "
                         f"(C restatement of the Volterra formula), "
                         f"{dt:.1f} s"}}
    hv = (h_variants or {}).get("h_grid_f64")
    if hv:
        res["gpu_fp64"] = {
            "value": Ny * Nz * Nx * n_seg / (hv["h_grid_ms"] * 1e-3),
            "ms": hv["h_grid_ms"],
            "form": "compute_H_grid, FP64, whole grid written to HBM"}
    return res


def run_reference(args):
    rank, world = dist()
    if rank != 0:
        return
    if args.reference_gpu:
        print(json.dumps(reference_gpu()), flush=True)
        return
    x, grid, segs, s = workload()
    sample, kind, cores = cpu_sampler(x, grid, segs, s)
    t0 = time.perf_counter()
    sample(2)
    per = (time.perf_counter() - t0) / 2
    nr = int(max(2, min(481, 4.0 / max(per, 1e-6))))
    for _ in range(args.warmup):
        sample(2)
    times, units = [], 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        units = sample(nr)
        times.append(time.perf_counter() - t0)
    v = units * len(times) / sum(times)
    smp = (f"{nr} of 481 active rows x all {len(s)} angles per step (H of "
           f"the 64 segments on those rows + the FP64 march)")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v,
        "unit": "voxel-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD + "; sample: " + smp,
                   "sample_rows": nr},
        "cpu_baseline": {"value": v, "unit": "voxel-steps/s", "cores": cores,
                         "kind": kind, "sample": smp},
        "e2e": {"value": v, "unit": "voxel-steps/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
        flush=True)


def reference_gpu(reps_small=5):
    """The reference's own Laue kernel on this GPU: its CUDA text
    (tt3d_fullfield_batch, built by oracle/make_ref.py into oracle/_ref)
    launched as DYFOX's solve_dislocation launches it (laue/solver.py:62-90:
    64 angles a launch, grid Ny x angles, 256 threads, planar output packed
    into complex), fed the H grid of this build's compute_H_grid (the
    reference's formula; DYFOX builds it with CuPy, absent here) in the
    launch's precision.  FP64 and FP32 at the README workload and the
    rocking scan; CUDA events on the current stream."""
    import torch
    from dyfox_gb300.dislocations import compute_H_grid
    from dyfox_gb300.grid import grid_arrays
    from oracle import oracle as O
    O.build_ref_gpu()
    if O.ref_gpu() is None:
        return {"unavailable": "the reference kernel text (oracle/_ref) was "
                               "not generated in this checkout"}
    stream = torch.cuda.current_stream()

    def ev():
        return torch.cuda.Event(enable_timing=True)
    res = {"form": "reference tt3d_fullfield_batch, 64 angles per launch as "
                   "laue/solver.py:62-90, H grid from compute_H_grid",
           "unit": "voxel-steps/s"}
    for name, wl in (("readme", readme_workload), ("scan", workload)):
        x, grid, segs, s = wl()
        geo = grid_arrays(grid)
        rows = active_rows(geo)
        n_e = len(s)
        units = n_e * len(rows) * geo["Nx"] * (geo["Nz"] - 1)
        entry = {"voxel_steps": units}
        for prec in ("fp64", "fp32"):
            fp32 = prec == "fp32"
            reps = reps_small if name == "readme" else (1 if not fp32 else 2)
            out = torch.empty((n_e, geo["Ny"], geo["Nx"]),
                              dtype=torch.complex64 if fp32
                              else torch.complex128, device="cuda")

            def march(H):
                for bs in range(0, n_e, 64):
                    be = min(bs + 64, n_e)
                    out[bs:be] = O.ref_gpu_laue_march(
                        "fullfield", x, s[bs:be], geo, H_grid=H, fp32=fp32)
            h0, h1 = ev(), ev()
            h0.record(stream)
            H = compute_H_grid(segs, grid, x, precision=prec)
            h1.record(stream)
            march(H)                                    # warm-up
            torch.cuda.synchronize()
            h_ms = h0.elapsed_time(h1)
            times = []
            for _ in range(reps):
                a, b = ev(), ev()
                a.record(stream)
                march(H)
                b.record(stream)
                torch.cuda.synchronize()
                times.append(a.elapsed_time(b))
            m_ms = statistics.median(times)
            entry[prec] = {"march_ms": m_ms, "h_grid_ms": h_ms,
                           "march_value": units / (m_ms * 1e-3),
                           "with_h_grid_value": units / ((m_ms + h_ms)
                                                         * 1e-3),
                           "reps": reps}
            del H, out
            torch.cuda.empty_cache()
        res[name] = entry
    return res


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
