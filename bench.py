#!/usr/bin/env python
"""Benchmark of the Laue hot path (DYFOX solve_dislocation) on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one "step"): the README-size Laue drop-in -- diamond (400) at
17 keV, t = 200 um, dx = 0.25 um, beam width 120 um (grid 544 x 800,
Nz = 359), one edge dislocation on [101] with b = (a/2)[10-1] crossing the
beam column at t/2 (half a pixel off the sampled rows), deviation
parameters at 0 and 117.5 urad: Volterra phase + depth march for both
angles.  Unit: voxel-steps (angle x active row x column x depth step).

--impl ours (default): the chosen form -- FP32 compensated march with the
Volterra phase evaluated inside it (float-float segment sum, single-precision
2 pi reduction) -- timed on the device with inputs resident; its exit intensity is checked
against the plain FP64 form (<= 1e-5 relative L2) in the same run, and the
plain FP64 form is timed beside it.  e2e times the public call with host
inputs and a device-to-host read of the exit waves.
--impl reference: the reference's Laue kernel (its CUDA text compiled for the
CPU, oracle/_ref; the oracle restatement when absent) on the host cores, on
a bounded sample of rows per step.

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
WORKLOAD = ("laue-readme: diamond(400) 17 keV, t=200um dx=0.25um "
            "beam_width=120um (Ny x Nx = 544 x 800, Nz=359), 1 edge "
            "dislocation line [101] b=(a/2)[10-1] at depth t/2, "
            "s_dev at 0 and 117.5 urad")
# DRAM bytes (read + write) of one launch of the chosen-form march on the
# readme workload, from the ncu capture summarised in
# profiles/laue_march_fp32_readme.md.
MARCH_FP32_README_DRAM_BYTES = 2843392


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--once", choices=["fp32", "fp64", "bragg", "bragg32",
                                       "scan", "image", "batch", "unet"],
                    help="run one solve of that form after one warm-up and "
                         "exit (a small, fixed case for ncu)")
    ap.add_argument("--no-bragg", action="store_true")
    ap.add_argument("--no-scan", action="store_true")
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
def run_ours(args):
    import torch
    from dyfox_gb300 import _lib
    from dyfox_gb300.backend import FP32, FP64
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import _desc, solve_dislocation

    rank, world = dist()
    if world > 1:
        torch.distributed.init_process_group(
            "nccl", init_method="env://", rank=rank, world_size=world)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    L = _lib.lib()
    x, grid, seg, s = workload()
    geo = grid_arrays(grid)
    rows = active_rows(geo)
    n_e = len(s)
    nsteps = geo["Nz"] - 1
    units = n_e * len(rows) * geo["Nx"] * nsteps        # voxel-steps
    voxels = len(rows) * geo["Nx"] * nsteps             # H evaluations

    table = _lib.segment_table(seg, x.g_vec, x.nu, x.a_core, geo["dx"])
    tdev = _lib.device_table(table)
    s_dev = torch.from_numpy(np.asarray(s, float)).cuda()
    stream = torch.cuda.current_stream()
    sp = _lib.c_void_p(stream.cuda_stream)

    from dyfox_gb300.autotune import lookup, tune
    tuned = {}
    if not args.no_tune and not args.once:
        for name, prec in (("fp32", FP32), ("fp64", FP64)):
            r = tune(seg, s, grid, x, precision=prec, h_mode="fused")
            tuned[name] = {"pairs": r.get("pairs", False),
                           "cols_per_lane": r["cols_per_lane"],
                           "angles_per_cta": r["angles_per_cta"]}

    def make(prec, extra=0):
        d = _desc(x, geo, n_e, prec, _lib.H_SEGMENTS, len(table),
                  flags=_lib.FLAG_FUSED | extra)
        shape = lookup(d)
        if shape is not None:
            d.cols_per_lane, d.angles_per_cta, pairs = shape
            if pairs:
                d.flags |= _lib.FLAG_PAIRS
        nb = L.dyfox_laue_workspace_bytes(d)
        ws = torch.empty(max(nb, 256), dtype=torch.uint8, device="cuda")
        out = torch.empty((n_e, geo["Ny"], geo["Nx"]),
                          dtype=prec.torch_complex, device="cuda")

        def call():
            _lib.check(L.dyfox_laue_solve(
                d, _lib.ptr(s_dev), None, _lib.ptr(tdev), _lib.ptr(out),
                _lib.ptr(ws), ws.numel(), sp), "dyfox_laue_solve")
        return call, out

    chosen, out32 = make(FP32)
    plain, out64 = make(FP64)
    sum64, out32b = make(FP32, _lib.FLAG_H_FP64)
    if args.once in ("fp32", "fp64"):
        fn = chosen if args.once == "fp32" else plain
        fn()
        torch.cuda.synchronize()
        fn()
        torch.cuda.synchronize()
        return
    if args.once == "scan":
        from dyfox_gb300.workloads import laue_rocking_scan
        sx, sgrid, ssegs, ss = laue_rocking_scan(n_angles=32)
        for _ in range(2):
            solve_dislocation(ssegs, ss, sgrid, sx, precision="fp32",
                              h_mode="staged", batch=len(ss))
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
    if args.once in ("bragg", "bragg32"):
        from dyfox_gb300.bragg import solve_scan
        bx, bcfg, bseg, bs, bys, bg = bragg_workload()
        prec = "fp32" if args.once == "bragg32" else "fp64"
        for _ in range(2):
            solve_scan(bseg, bs[:4], bcfg, bys[:8], bx, bg, precision=prec)
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
    flush =torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def timed(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True),
               torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        n0 = L.dyfox_launch_count()
        for a, b in ev:
            flush.zero_()                 # L2 flush outside the events
            a.record(stream)
            fn()
            b.record(stream)
        torch.cuda.synchronize()
        launches = L.dyfox_launch_count() - n0
        return [a.elapsed_time(b) for a, b in ev], launches

    # accuracy of the chosen form against plain FP64, in this run
    chosen()
    plain()
    torch.cuda.synchronize()
    I32 = out32.abs().double() ** 2
    I64 = out64.abs() ** 2
    err = float(torch.linalg.vector_norm(I32 - I64)
                / torch.linalg.vector_norm(I64))
    if err > 1e-5:
        raise SystemExit(f"chosen form misses the 1e-5 budget: {err:.2e}")

    peaks = {}
    for name, code in (("fp32", _lib.DYFOX_FP32), ("fp64", _lib.DYFOX_FP64)):
        v = _lib.c_double(0)
        _lib.check(L.dyfox_pipe_peak(code, 4096 if name == "fp32" else 256,
                                     __import__("ctypes").byref(v), sp),
                   "dyfox_pipe_peak")
        peaks[name] = v.value

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with Clocks(local) as clk:
        t0 = time.perf_counter()
        ms, launches = timed(chosen, args.steps, args.warmup)
        wall = time.perf_counter() - t0
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms_plain, _ = timed(plain, max(3, args.steps // 4), 2)
    ms_sum64, _ = timed(sum64, max(3, args.steps // 4), 2)
    torch.cuda.synchronize()
    I32b = out32b.abs().double() ** 2
    err_sum64 = float(torch.linalg.vector_norm(I32b - I64)
                      / torch.linalg.vector_norm(I64))

    tot = max_over_ranks(sum(ms) / 1e3, world)
    value = world * units * args.steps / tot
    mean_ms = 1e3 * tot / args.steps
    plain_ms = statistics.mean(ms_plain)

    h_variants = None if args.once else readme_h_variants(seg, s, grid, x)

    # e2e: public API, host inputs, device-to-host read of the exit waves
    host = torch.empty((n_e, geo["Ny"], geo["Nx"]), dtype=torch.complex64,
                       pin_memory=True)
    s_host = np.asarray(s, float)

    def e2e():
        o = solve_dislocation(seg, s_host, grid, x, precision=FP32,
                              h_mode="fused")
        host.copy_(o)
        torch.cuda.synchronize()
    for _ in range(2):
        e2e()
    t0 = time.perf_counter()
    ke = max(3, args.steps // 2)
    for _ in range(ke):
        e2e()
    e2e_s = (time.perf_counter() - t0) / ke

    # roofline of the march kernel: 40 flops per voxel-step (2x2 complex
    # propagator + two complex coupling products) + 40 flops per segment-
    # voxel of Volterra phase (atan2, log not counted)
    flops = 40.0 * units + 40.0 * len(table) * voxels
    achieved = flops / (mean_ms * 1e-3) / 1e12
    line = {
        "metric": METRIC, "value": value, "unit": "voxel-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (compensated)",
        "data": "synthetic (seeded geometry of the benchmark configuration)",
        "config": {"workload": WORKLOAD, "angles": n_e,
                   "active_rows": int(len(rows)), "Nx": geo["Nx"],
                   "Nz": geo["Nz"], "voxel_steps_per_step": units,
                   "form": "FP32 compensated march, Volterra phase fused "
                           "(float-float segment sum and 2 pi reduction)",
                   "l2": "flushed between steps (256 MB write)",
                   "parallelism": f"replicas x{world}"},
        "error_vs_fp64": {"intensity_rel_l2": err, "budget": 1e-5},
        "plain_fp64": {"value": units / (plain_ms * 1e-3),
                       "ms_per_step": plain_ms,
                       "unit": "voxel-steps/s"},
        "fp32_with_fp64_h_sum": {
            "value": units / (statistics.mean(ms_sum64) * 1e-3),
            "ms_per_step": statistics.mean(ms_sum64),
            "unit": "voxel-steps/s", "intensity_rel_l2": err_sum64,
            "form": "as the chosen form, segment sum and 2 pi reduction "
                    "in double"},
        "e2e": {"value": world * units / e2e_s, "unit": "voxel-steps/s",
                "ms_per_step": e2e_s * 1e3,
                "h2d_bytes_per_step": int(8 * n_e + table.nbytes),
                "d2h_bytes_per_step": int(host.numel() * 8)},
        "roofline": {"bound": "fp32", "achieved": achieved,
                     "peak": peaks["fp32"], "unit": "TFLOP/s",
                     "frac": achieved / peaks["fp32"],
                     "traffic": MARCH_FP32_README_DRAM_BYTES,
                     "traffic_source": "ncu dram__bytes_read.sum + "
                                       "dram__bytes_write.sum of one launch "
                                       "(profiles/laue_march_fp32_readme.md)",
                     "peak_source": "measured FFMA throughput "
                                    "(dyfox_pipe_peak, this run)",
                     "algorithmic_flops_per_launch": flops},
        "pipe_peaks_tflops": peaks,
        "launch_shape": {"tuned": tuned or None,
                         "autotuner": "dyfox_gb300.autotune (cols per lane x "
                                      "angles per CTA, each timed at about "
                                      "2048 CTAs)"},
        "gpu_launches": int(launches),
        "wall_s": wall,
        "h_variants": h_variants,
    }
    clk_sum = clk.summary()
    line["clocks"] = clk_sum
    if not args.no_bragg:
        line["bragg"] = bragg_leg(args, rank, world, peaks)
    if not args.no_scan:
        line["laue_scan"] = scan_leg(args, world, peaks)
    if not args.no_com_maps:
        line["com_maps"] = com_maps_leg(args, world)
    if not args.no_batched:
        line["batched"] = batched_leg(args, world)
    if not args.no_learned:
        line["learned_guess"] = learned_leg(args, world)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(x, grid, seg, s, args.cpu_seconds)
        line["volterra"] = volterra_leg(x, grid, seg, h_variants,
                                        min(3.0, args.cpu_seconds))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


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


def scan_leg(args, world, peaks=None):
    """The 256-angle rocking scan (t = 273 um, 544 x 1056, Nz 490, 64 random
    <110> segments): chosen FP32 form, e^{iH} staged once (float-float
    segment sum) and read by every angle group.  Accuracy is checked
    against plain FP64 on 8 of the 256 angles."""
    import torch
    from dyfox_gb300 import _lib
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import solve_dislocation
    from dyfox_gb300.workloads import laue_rocking_scan
    x, grid, segs, s = laue_rocking_scan()
    geo = grid_arrays(grid)
    rows = active_rows(geo)
    units = len(s) * len(rows) * geo["Nx"] * (geo["Nz"] - 1)
    stream = torch.cuda.current_stream()
    L = _lib.lib()
    shape = None
    if not args.no_tune:
        from dyfox_gb300.autotune import tune
        r = tune(segs, s, grid, x, precision="fp32", h_mode="staged")
        shape = {"cols_per_lane": r["cols_per_lane"],
                 "angles_per_cta": r["angles_per_cta"]}
    for _ in range(2):
        solve_dislocation(segs, s, grid, x, precision="fp32",
                          h_mode="staged", batch=len(s))
    torch.cuda.synchronize()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    times = []
    n0 = L.dyfox_launch_count()
    steps = max(3, args.steps // 4)
    for _ in range(steps):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        out = solve_dislocation(segs, s, grid, x, precision="fp32",
                                h_mode="staged", batch=len(s))
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    launches = L.dyfox_launch_count() - n0
    pick = np.linspace(0, len(s) - 1, 8).round().astype(int)
    t0 = time.perf_counter()
    ref = solve_dislocation(segs, s[pick], grid, x, precision="fp64")
    torch.cuda.synchronize()
    fp64_s = time.perf_counter() - t0
    I32 = out[torch.as_tensor(pick, device="cuda")].abs().double() ** 2
    I64 = ref.abs() ** 2
    err = float(torch.linalg.vector_norm(I32 - I64)
                / torch.linalg.vector_norm(I64))
    ms = 1e3 * max_over_ranks(statistics.mean(times) * 1e-3, world)
    return {"value": world * units / (ms * 1e-3), "unit": "voxel-steps/s",
            "ms_per_scan": ms, "voxel_steps_per_scan": units,
            "angles": len(s), "segments": len(segs), "active_rows":
            int(len(rows)), "Nx": geo["Nx"], "Nz": geo["Nz"],
            "form": "FP32 compensated march, e^{iH} staged once "
                    "(float-float segment sum), all angles in one call",
            "intensity_rel_l2_vs_fp64_8_angles": err,
            "fp64_8_angles_s": fp64_s, "gpu_launches": int(launches),
            "launch_shape": shape,
            "roofline": None if not peaks else {
                "bound": "fp32",
                # 40 flops a voxel-step (march) and 40 a segment-voxel (the
                # staged phase, atan2 and log not counted)
                "achieved": world * 40.0 * (units + len(rows) * geo["Nx"] *
                                            (geo["Nz"] - 1) * len(segs))
                / (ms * 1e-3) / 1e12,
                "peak": peaks["fp32"], "unit": "TFLOP/s",
                "frac": world * 40.0 * (units + len(rows) * geo["Nx"] *
                                        (geo["Nz"] - 1) * len(segs))
                / (ms * 1e-3) / 1e12 / peaks["fp32"]}}


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
    """Bragg solves/s of config 1: all 21 deviation parameters x 64 planes
    in one batched launch (one solve = one deviation parameter over all
    planes, to true relative residual <= 1e-10).  The chosen form is the
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
    sample, kind, cores = cpu_sampler(x, grid, seg, s)
    t0 = time.perf_counter()
    sample(cores)
    per = (time.perf_counter() - t0) / cores
    nr = int(max(cores, min(481, seconds / max(per, 1e-6))))
    t0 = time.perf_counter()
    units = sample(nr)
    dt = time.perf_counter() - t0
    return {"value": units / dt, "unit": "voxel-steps/s", "cores": cores,
            "kind": kind, "sample": f"{nr} of 481 active rows x {len(s)} "
            f"angles (H on those rows + FP64 march), {dt:.1f} s"}


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
    x, grid, seg, s = workload()
    sample, kind, cores = cpu_sampler(x, grid, seg, s)
    t0 = time.perf_counter()
    sample(cores)
    per = (time.perf_counter() - t0) / cores
    nr = int(max(cores, min(481, 2.0 / max(per, 1e-6))))
    for _ in range(args.warmup):
        sample(cores)
    times, units = [], 0
    for _ in range(args.steps):
        t0 = time.perf_counter()
        units = sample(nr)
        times.append(time.perf_counter() - t0)
    v = units * len(times) / sum(times)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v,
        "unit": "voxel-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_rows": nr},
        "cpu_baseline": {"value": v, "unit": "voxel-steps/s", "cores": cores,
                         "kind": kind,
                         "sample": f"{nr} of 481 active rows x {len(s)} "
                                   "angles per step"},
        "e2e": {"value": v, "unit": "voxel-steps/s",
                "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
        flush=True)


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
