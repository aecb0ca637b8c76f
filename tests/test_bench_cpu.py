"""bench.py's host arithmetic on the CPU: the multi-rank timing on two
gloo ranks (the timed region is the maximum over ranks, and the whole-job
value counts every rank's units), the clock record, the Bragg flop count
and the headline workload's unit count."""

import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    t = bench.max_over_ranks(1.0 + rank, world)
    q.put((rank, t))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = dict(q.get(timeout=10) for _ in range(2))
    assert got == {0: 2.0, 1: 2.0}


def test_single_rank_is_identity():
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_clock_summary_of_fake_samples():
    """The clocks record is the median SM clock under load, the largest
    maximum clock and every throttle reason seen active; lines that are
    not samples are skipped."""
    import bench
    c = bench.Clocks(0)
    c.lines = [
        "2070, 2070, 900.1, 0x0000000000000000, Not Active, Not Active, "
        "Not Active, Not Active",
        "1980, 2070, 1390.0, 0x0000000000000004, Not Active, Not Active, "
        "Not Active, Active",
        "2055, 2070, 1200.0, 0x0000000000000000, Not Active, Not Active, "
        "Not Active, Not Active",
        "[N/A], 2070, 10.0, 0x0, Not Active, Not Active, Not Active, "
        "Not Active",
        "garbage",
    ]
    s = c.summary()
    assert s == {"sm_mhz": 2055.0, "sm_max_mhz": 2070.0,
                 "reasons": ["sw_power_cap"], "samples": 3}
    c.lines.append("1500, 2070, 1400.0, 0x48, Active, Not Active, Active, "
                   "Not Active")
    assert c.summary()["reasons"] == ["hw_slowdown", "sw_power_cap",
                                      "sw_thermal_slowdown"]
    assert bench.Clocks(0).summary()["samples"] == 0


def test_bragg_flop_count():
    """Per inner iteration: march 28 (Nz-1) Nx, preconditioner
    10 Nx log2 Nx + 6 Nx, Gram-Schmidt 16 (j+1) Nx with j the position in
    the restart cycle; two more marches per system."""
    import numpy as np
    import bench
    Nx, Nz, m = 456, 90, 40
    inf = np.array([[0.0, 18, 0, 0], [0.0, 45, 0, 0]])
    prod, mgs = bench.bragg_flops(inf, Nx, Nz, m)
    march = 28 * (Nz - 1) * Nx
    prec = 10 * Nx * np.log2(Nx) + 6 * Nx
    assert np.isclose(prod, 63 * (march + prec) + 4 * march, rtol=1e-14)
    j = np.concatenate([np.arange(18), np.arange(45) % m])
    assert np.isclose(mgs, 16 * Nx * np.sum(j + 1), rtol=1e-14)


def test_scan_and_readme_workload_counts():
    """The headline workload is the rocking scan, 544 x 1056 x 490 with
    481 active rows, 64 segments and 256 deviation parameters: 6.36e10
    active voxel-steps; the README drop-in beside it is 544 x 800 x 359
    with two deviation parameters: 2.76e8."""
    import bench
    from dyfox_gb300.grid import grid_arrays
    x, grid, segs, s = bench.workload()
    geo = grid_arrays(grid)
    assert (geo["Ny"], geo["Nx"], geo["Nz"]) == (544, 1056, 490)
    rows = len(bench.active_rows(geo))
    assert rows == 481 and len(s) == 256 and len(segs) == 64
    assert 256 * rows * 1056 * 489 == 63_585_460_224
    x, grid, seg, s = bench.readme_workload()
    geo = grid_arrays(grid)
    assert (geo["Ny"], geo["Nx"], geo["Nz"]) == (544, 800, 359)
    rows = len(bench.active_rows(geo))
    assert rows == 481
    assert len(s) == 2
    assert 2 * rows * 800 * 358 == 275_516_800


def test_volterra_leg_on_the_host():
    """The Volterra leg's CPU baseline runs the oracle's H rows on the
    host; the GPU rate is the whole grid's evaluations over the measured
    FP64 grid time."""
    import bench
    x, grid, seg, s = bench.readme_workload()
    r = bench.volterra_leg(x, grid, seg, {"h_grid_f64": {"h_grid_ms": 40.0}},
                           0.05, max_rows=2)
    assert r["grid"] == [544, 359, 800] and r["segments"] == 1
    cb = r["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] > 0 and cb["cores"] >= 1
    assert abs(r["gpu_fp64"]["value"] - 544 * 359 * 800 / 0.040) < 1.0
    assert "gpu_fp64" not in bench.volterra_leg(x, grid, seg, None, 0.01,
                                                max_rows=1)
