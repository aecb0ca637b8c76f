"""The CUDA Laue path against the oracle, the reference's golden vectors and
(when oracle/_ref was generated) the reference's own kernel run on the GPU.

Tolerances: plain FP64 matches the reference to <= 1e-12 relative L2 on the
complex exit wave; the compensated FP32 mode matches FP64 to <= 1e-5
relative L2 on the exit intensity |D_g|^2.
"""

import numpy as np
import pytest

from conftest import golden, rel_l2
from oracle import closed_forms as CF
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_INTENSITY_TOL = 1e-5


def np_(t):
    return t.detach().cpu().numpy()


def geometry_n(xtal, grid, sign=+1, y0=0.0, half=400e-6):
    from dyfox_gb300.dislocations import burgers_vector, straight_segment
    xi = np.array([1.0, 0.0, 1.0]) / np.sqrt(2.0)
    b = burgers_vector(np.eye(3), [1, 0, -1], xtal.b_mag, sign)
    z0 = grid.t_crystal / 2
    return straight_segment(xi, b, [-z0 * xtal.tan_tB, y0, z0], half)


def mixed_on_x(xtal, grid, sign=+1):
    from dyfox_gb300.dislocations import burgers_vector, straight_segment
    b = burgers_vector(np.eye(3), [1, 1, 0], xtal.b_mag, sign)
    return straight_segment([1.0, 0.0, 0.0], b,
                            [0.0, grid.dx / 2, grid.t_crystal / 2], 400e-6)


def random_segments(xtal, grid, n, rng):
    """<110> lines and (a/2)<110> Burgers vectors with random sign, cores in
    the illuminated volume, half-lengths log-uniform in [10, 400] um."""
    from dyfox_gb300.dislocations import straight_segment
    dirs = np.array([[1, 1, 0], [1, -1, 0], [1, 0, 1], [1, 0, -1],
                     [0, 1, 1], [0, 1, -1]], float)
    segs = []
    t = grid.t_crystal
    for _ in range(n):
        xi = dirs[rng.integers(6)] * rng.choice([-1, 1])
        b = dirs[rng.integers(6)] * rng.choice([-1, 1])
        c = [rng.uniform(-t * xtal.tan_tB, t * xtal.tan_tB),
             rng.uniform(-grid.beam_width / 2, grid.beam_width / 2)
             + grid.dx / 2, rng.uniform(0, t)]
        segs += straight_segment(xi / np.linalg.norm(xi),
                                 xtal.b_mag * b / np.linalg.norm(b), c,
                                 np.exp(rng.uniform(np.log(10e-6),
                                                    np.log(400e-6))))
    return segs


def geo_of(grid):
    from dyfox_gb300.grid import grid_arrays
    return grid_arrays(grid)


# ----------------------------------------------------------------- Volterra
@pytest.mark.parametrize("name", ["n", "x", "r", "screw", "zero"])
def test_h_rows_match_h_plane_golden(gpu, diamond400, name):
    from dyfox_gb300.dislocations import H_rows
    v = golden("volterra")
    segs = [(s[:3], s[3:6], s[6:]) for s in v[f"segs_{name}"]]
    H = np_(H_rows(segs, int(v["Nx"]), int(v["Nz"]), float(v["dx"]),
                   float(v["dz"]), diamond400.g_vec, diamond400.nu,
                   diamond400.a_core, v["y_planes"]))
    want = v[f"H_{name}"]
    assert np.abs(H - want).max() <= 1e-13 * max(np.abs(want).max(), 1.0)


def test_h_rows_over_several_segment_tiles(gpu, diamond400, small_grid,
                                           rng):
    """400 segments on two planes: more than one shared-memory tile of
    segments, the partial sums carried in the output between tiles."""
    from dyfox_gb300.dislocations import H_rows
    geo = geo_of(small_grid)
    segs = random_segments(diamond400, small_grid, 400, rng)
    y = O.grid_y(geo["Ny"], geo["dx"])[[10, 50]]
    want = O.h_rows(segs, diamond400.g_vec, diamond400.nu, diamond400.a_core,
                    geo["Nx"], geo["Nz"], geo["dx"], geo["dz"], y)
    got = np_(H_rows(segs, geo["Nx"], geo["Nz"], geo["dx"], geo["dz"],
                     diamond400.g_vec, diamond400.nu, diamond400.a_core, y))
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()


@pytest.mark.parametrize("n_seg", [7, 60])
def test_h_grid_matches_the_oracle(gpu, diamond400, small_grid, rng, n_seg):
    """7 segments: the kernel keeps every segment's column terms in shared
    memory; 60: too many for that, the column terms per voxel."""
    from dyfox_gb300.backend import FP32, FP64
    from dyfox_gb300.dislocations import compute_H_grid
    geo = geo_of(small_grid)
    segs = random_segments(diamond400, small_grid, n_seg, rng)
    want = O.h_rows(segs, diamond400.g_vec, diamond400.nu, diamond400.a_core,
                    geo["Nx"], geo["Nz"], geo["dx"], geo["dz"],
                    O.grid_y(geo["Ny"], geo["dx"]))
    got = np_(compute_H_grid(segs, small_grid, diamond400, precision=FP64))
    assert got.shape == (geo["Ny"], geo["Nz"], geo["Nx"])
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    want32 = O.h_rows(segs, diamond400.g_vec, diamond400.nu,
                      diamond400.a_core, geo["Nx"], geo["Nz"], geo["dx"],
                      geo["dz"], O.grid_y(geo["Ny"], geo["dx"]),
                      cast_fp32=True)
    got32 = np_(compute_H_grid(segs, small_grid, diamond400, precision=FP32))
    assert got32.dtype == np.float32
    assert np.abs(got32 - want32).max() <= 1e-5 * np.abs(want32).max()


def test_zero_burgers_vector_leaves_no_phase(gpu, diamond400, small_grid):
    from dyfox_gb300.dislocations import compute_H_grid
    seg = geometry_n(diamond400, small_grid)
    dead = [(seg[0][0], seg[0][1], np.zeros(3))]
    assert float(compute_H_grid(dead, small_grid, diamond400).abs().max()) \
        == 0.0


def test_h_grid_is_deterministic(gpu, diamond400, small_grid, rng):
    from dyfox_gb300.dislocations import compute_H_grid
    segs = random_segments(diamond400, small_grid, 3, rng)
    a = np_(compute_H_grid(segs, small_grid, diamond400))
    b = np_(compute_H_grid(segs, small_grid, diamond400, chunk_y=1))
    assert a.tobytes() == b.tobytes()


def test_phase_winds_by_g_dot_b(gpu, diamond400, small_grid):
    """H winds by 2 pi g.b around the core (reference test_laue_gpu.py:93)."""
    from dyfox_gb300.dislocations import compute_H_grid, g_dot_b
    for sign in (+1, -1):
        seg = geometry_n(diamond400, small_grid, sign)
        H = np_(compute_H_grid(seg, small_grid, diamond400))
        Ny_, Nz_, Nx_ = H.shape
        plane = H[:, :, Nx_ // 2]
        (ra, rb, bv), = seg
        xi = (rb - ra) / np.linalg.norm(rb - ra)
        core = (ra + rb) / 2.0
        tpar = (0.0 - core[0]) / xi[0]
        cy = Ny_ / 2 + (core[1] + tpar * xi[1]) / small_grid.dx
        cz = (core[2] + tpar * xi[2]) / small_grid.geometry()[2]
        ang = np.linspace(0, 2 * np.pi, 1440, endpoint=False)
        ys = np.clip((cy + 20 * np.cos(ang)).astype(int), 0, Ny_ - 1)
        zs = np.clip((cz + 20 * np.sin(ang)).astype(int), 0, Nz_ - 1)
        p = plane[ys, zs]
        wind = (np.sum(np.angle(np.exp(1j * np.diff(p))))
                + np.angle(np.exp(1j * (p[0] - p[-1])))) / (2 * np.pi)
        assert wind == pytest.approx(g_dot_b(diamond400.g_vec, bv), abs=0.05)


# --------------------------------------------------------------- the march
def test_fp64_matches_reference_golden(gpu, diamond400, small_grid):
    """Full field (H grid, fused segments), pristine and closed form
    against the reference kernel's own output (golden)."""
    from dyfox_gb300.dislocations import compute_H_grid
    from dyfox_gb300.laue import solve_dislocation, solve_pristine
    g = golden("laue_small")
    v = golden("volterra")
    rows, s = g["rows"], g["s_dev"]
    seg = [(q[:3], q[3:6], q[6:]) for q in v["segs_n"]]
    H = compute_H_grid(seg, small_grid, diamond400)
    a = np_(solve_dislocation(seg, s, small_grid, diamond400, H_gpu=H))
    assert a.dtype == np.complex128
    assert rel_l2(a[:, rows], g["fullfield"]) < FP64_TOL
    b = np_(solve_dislocation(seg, s, small_grid, diamond400))
    assert rel_l2(b[:, rows], g["fullfield"]) < FP64_TOL
    c = np_(solve_pristine(s, small_grid, diamond400))
    assert rel_l2(c[:, rows], g["pristine"]) < FP64_TOL
    seg_x = [(q[:3], q[3:6], q[6:]) for q in v["segs_x"]]
    d = np_(solve_dislocation(seg_x, s, small_grid, diamond400))
    assert rel_l2(d[:, rows], g["analytic"]) < FP64_TOL


def test_interpolating_grid_matches_reference_golden(gpu, diamond400):
    from dyfox_gb300.grid import LaueGrid
    from dyfox_gb300.laue import solve_pristine
    g = golden("laue_small")
    grid = LaueGrid(diamond400, 40e-6, 0.25e-6, 8e-6, beam_thickness=1e-6,
                    Nz=301)
    assert not grid.exact
    a = np_(solve_pristine(g["s_dev"], grid, diamond400))
    assert rel_l2(a[:, g["rows"]], g["interp_pristine"]) < FP64_TOL


@pytest.mark.parametrize("t", [200e-6, 273e-6])
def test_fp64_matches_oracle_at_benchmark_size(gpu, diamond400, t):
    """README-size grid (544 x 800, Nz 359) and the 273 um grid: GPU vs the
    C oracle on rows through and beside the dislocation."""
    from dyfox_gb300.grid import LaueGrid
    from dyfox_gb300.laue import solve_dislocation
    from dyfox_gb300.units import deviation_from_urad
    grid = LaueGrid(diamond400, t, 0.25e-6, 120e-6)
    geo = geo_of(grid)
    seg = geometry_n(diamond400, grid, y0=grid.dx / 2, half=800e-6)
    s = deviation_from_urad([0.0, 117.5], diamond400)
    got = np_(solve_dislocation(seg, s, grid, diamond400))
    Ny = geo["Ny"]
    rows = np.array([Ny // 2 - 200, Ny // 2 - 1, Ny // 2, Ny // 2 + 1,
                     Ny // 2 + 37])
    H = O.h_rows(seg, diamond400.g_vec, diamond400.nu, diamond400.a_core,
                 geo["Nx"], geo["Nz"], geo["dx"], geo["dz"],
                 O.grid_y(Ny, geo["dx"], rows))
    want = O.laue_march("fullfield", diamond400, s, geo, H_rows=H, rows=rows)
    assert rel_l2(got[:, rows], want) < FP64_TOL


def rows_clear_of_cores(segs, geo, candidates, min_px=0.05):
    """The candidate rows on which every segment line (infinite, through the
    segment's midpoint, as the Volterra field treats it) passes at least
    ``min_px`` pixels from every sample node (x_i, y_row, z_k).  A core that
    sits on a node puts atan2 at its own singularity, where two correct
    evaluations can differ completely (reference tests/test_laue_gpu.py:
    116-138); off the nodes the field is smooth at rounding level.

    Within a row plane, a node at in-plane distance q from the line's
    crossing point is at least q |xi_y| from the line, so the 5 x 5 nodes
    around the crossing hold the minimum for the <110> lines (|xi_y| =
    1/sqrt 2); a line lying in a plane y = c is |y_row - c| away."""
    Nx, dx, dz = geo["Nx"], geo["dx"], geo["dz"]
    keep = []
    for r in candidates:
        y = (r - geo["Ny"] / 2) * dx
        dmin = np.inf
        for ra, rb, _ in segs:
            ra, rb = np.asarray(ra, float), np.asarray(rb, float)
            xi = (rb - ra) / np.linalg.norm(rb - ra)
            c = (ra + rb) / 2
            if abs(xi[1]) < 1e-12:
                dmin = min(dmin, abs(y - c[1]))
                continue
            p = c + (y - c[1]) / xi[1] * xi
            i0 = int(np.floor(p[0] / dx + Nx / 2))
            k0 = int(np.floor(p[2] / dz))
            ii, kk = np.meshgrid(np.arange(i0 - 2, i0 + 3),
                                 np.arange(k0 - 2, k0 + 3))
            q = np.stack([(ii - Nx / 2) * dx, np.full(ii.shape, y),
                          kk * dz], axis=-1) - c
            dist = np.linalg.norm(np.cross(q, xi), axis=-1)
            dmin = min(dmin, float(dist.min()))
        if dmin >= min_px * dx:
            keep.append(int(r))
    return np.array(keep)


def test_fp64_scan_of_64_segments_matches_the_oracle(gpu, diamond400):
    """The rocking-scan configuration in plain FP64 (t = 273 um, 544 x
    1056, Nz 490, the 64 seeded random segments): the fused Volterra phase,
    summed over the segments in list order inside the march, against the
    C oracle (the reference's formula and march) on six rows across the
    beam chosen clear of every core, at the two ends and the middle of the
    scan: <= 1e-12 relative L2."""
    from dyfox_gb300.laue import solve_dislocation
    from dyfox_gb300.workloads import laue_rocking_scan
    x, grid, segs, s_all = laue_rocking_scan()
    assert len(segs) == 64
    s = s_all[[0, 128, 255]]
    geo = geo_of(grid)
    Ny = geo["Ny"]
    half = int(grid.beam_width / 2 / geo["dx"])
    cand = np.linspace(Ny // 2 - half + 3, Ny // 2 + half - 3, 24).astype(int)
    rows = rows_clear_of_cores(segs, geo, cand)
    assert len(rows) >= 6
    rows = rows[np.linspace(0, len(rows) - 1, 6).astype(int)]
    got = np_(solve_dislocation(segs, s, grid, x, precision="fp64"))
    H = O.h_rows(segs, x.g_vec, x.nu, x.a_core, geo["Nx"], geo["Nz"],
                 geo["dx"], geo["dz"], O.grid_y(Ny, geo["dx"], rows))
    want = O.laue_march("fullfield", x, s, geo, H_rows=H, rows=rows)
    assert np.abs(want).max() > 0
    assert rel_l2(got[:, rows], want) < FP64_TOL


def test_fp64_matches_the_reference_kernel_on_the_gpu(gpu, diamond400):
    """The reference's own CUDA kernel (oracle/_ref, built from its source)
    launched as laue/solver.py launches it, fed the same H grid."""
    if O.ref_gpu() is None:
        pytest.skip("oracle/_ref was not generated")
    from dyfox_gb300.dislocations import compute_H_grid
    from dyfox_gb300.grid import LaueGrid
    from dyfox_gb300.laue import solve_dislocation, solve_pristine
    from dyfox_gb300.units import deviation_from_urad
    grid = LaueGrid(diamond400, 200e-6, 0.25e-6, 120e-6)
    geo = geo_of(grid)
    seg = geometry_n(diamond400, grid, y0=grid.dx / 2, half=800e-6)
    s = deviation_from_urad([0.0, 117.5], diamond400)
    H = compute_H_grid(seg, grid, diamond400)
    ref = np_(O.ref_gpu_laue_march("fullfield", diamond400, s, geo, H_grid=H))
    assert rel_l2(np_(solve_dislocation(seg, s, grid, diamond400, H_gpu=H)),
                  ref) < FP64_TOL
    assert rel_l2(np_(solve_dislocation(seg, s, grid, diamond400)),
                  ref) < FP64_TOL
    ref_p = np_(O.ref_gpu_laue_march("pristine", diamond400, s, geo))
    assert rel_l2(np_(solve_pristine(s, grid, diamond400)), ref_p) < FP64_TOL


@pytest.mark.parametrize("mode", ["fused", "staged"])
@pytest.mark.parametrize("h_sum", ["ff", "fp64"])
def test_fp32_compensated_meets_the_intensity_budget(gpu, diamond400, mode,
                                                     h_sum, rng):
    from dyfox_gb300.backend import FP32
    from dyfox_gb300.grid import LaueGrid
    from dyfox_gb300.laue import solve_dislocation
    from dyfox_gb300.units import deviation_from_urad
    grid = LaueGrid(diamond400, 200e-6, 0.25e-6, 120e-6)
    seg = geometry_n(diamond400, grid, y0=grid.dx / 2, half=800e-6)
    seg += random_segments(diamond400, grid, 6, rng)
    s = deviation_from_urad([0.0, 117.5, -300.0, 30.0], diamond400)
    a = np_(solve_dislocation(seg, s, grid, diamond400, h_mode=mode))
    b = np_(solve_dislocation(seg, s, grid, diamond400, precision=FP32,
                              h_mode=mode, h_sum=h_sum))
    assert b.dtype == np.complex64
    err = rel_l2(np.abs(b) ** 2, np.abs(a) ** 2)
    assert 0 < err < FP32_INTENSITY_TOL
    c = np_(solve_dislocation(seg, s, grid, diamond400, precision=FP32,
                              h_mode=mode, compensated=False, h_sum=h_sum))
    assert rel_l2(np.abs(c) ** 2, np.abs(a) ** 2) < FP32_INTENSITY_TOL


def test_batching_does_not_change_the_scan(gpu, diamond400, small_grid):
    from dyfox_gb300.dislocations import compute_H_grid
    from dyfox_gb300.laue import solve_dislocation
    seg = geometry_n(diamond400, small_grid)
    s = np.linspace(-3e5, 3e5, 9)
    H = compute_H_grid(seg, small_grid, diamond400)
    a = np_(solve_dislocation(seg, s, small_grid, diamond400, H_gpu=H,
                              batch=64))
    b = np_(solve_dislocation(seg, s, small_grid, diamond400, H_gpu=H,
                              batch=2))
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("prec,h_sum", [("fp64", "ff"), ("fp32", "ff"),
                                         ("fp32", "fp64")])
def test_fused_and_staged_phase_agree_bitwise(gpu, diamond400, small_grid,
                                             prec, h_sum, rng):
    from dyfox_gb300.laue import solve_dislocation
    segs = random_segments(diamond400, small_grid, 4, rng)
    s = np.linspace(-3e5, 3e5, 5)
    a = np_(solve_dislocation(segs, s, small_grid, diamond400, precision=prec,
                              h_mode="fused", h_sum=h_sum))
    b = np_(solve_dislocation(segs, s, small_grid, diamond400, precision=prec,
                              h_mode="staged", h_sum=h_sum))
    assert a.tobytes() == b.tobytes()


@pytest.mark.parametrize("prec,h_mode,pairs", [("fp32", "staged", False),
                                              ("fp32", "fused", False),
                                              ("fp32", "staged", True),
                                              ("fp64", "auto", False)])
def test_host_out_copies_every_row_chunk(gpu, diamond400, small_grid, rng,
                                         prec, h_mode, pairs):
    """host_out: the march in row chunks with each chunk's rows of every
    wave copied to pinned host memory while the next marches (and the rows
    outside the beam copied at once) gives the device call's bytes, for
    several angle counts, through the scalar and the pair march and in
    FP64; a host_out of the wrong shape is refused."""
    from dyfox_gb300.laue import _solve, solve_dislocation
    torch = gpu
    segs = random_segments(diamond400, small_grid, 3, rng)
    for n_e in (2, 19, 40):
        s = np.linspace(-3e5, 3e5, n_e)
        kw = dict(precision=prec, h_mode=h_mode, batch=n_e)
        want = np_(_solve(segs, s, small_grid, diamond400, None, n_e, prec,
                          False, h_mode=h_mode, pairs=pairs, tuned=False))
        host = torch.empty(want.shape, dtype=torch.complex64 if prec ==
                           "fp32" else torch.complex128, pin_memory=True)
        host.fill_(float("nan"))
        got = _solve(segs, s, small_grid, diamond400, None, n_e, prec, False,
                     h_mode=h_mode, pairs=pairs, tuned=False, host_out=host)
        assert got is host
        assert host.numpy().tobytes() == want.tobytes(), n_e
    with pytest.raises(ValueError):
        solve_dislocation(segs, s[:3], small_grid, diamond400,
                          host_out=torch.empty(1, dtype=torch.complex128),
                          **kw)


@pytest.mark.parametrize("t_um", [0.5, 1.0, 1.8, 2.5, 3.0, 3.6])
def test_staged_march_of_a_few_depth_steps(gpu, diamond400, rng, t_um):
    """The staged march's ring of three row stages (one bulk copy a step,
    an mbarrier phase a stage) at 1 to 6 depth steps, where the unrolled
    rounds of three leave 0, 1 or 2 steps over: the bytes of the fused
    march, in FP32 with both segment sums and in FP64, every bounded wait
    completed."""
    from dyfox_gb300 import _lib
    from dyfox_gb300.grid import LaueGrid, grid_arrays
    from dyfox_gb300.laue import _desc
    from dyfox_gb300.backend import precision as as_precision
    torch = gpu
    grid = LaueGrid(diamond400, t_um * 1e-6, 0.25e-6, 4e-6,
                    beam_thickness=1e-6)
    geo = grid_arrays(grid)
    segs = random_segments(diamond400, grid, 3, rng)
    s = np.linspace(-3e5, 3e5, 5)
    for prec, hflag in (("fp32", _lib.FLAG_H_FP64), ("fp32", 0),
                        ("fp64", 0)):
        p = as_precision(prec)
        table = _lib.segment_table(segs, diamond400.g_vec, diamond400.nu,
                                   diamond400.a_core, geo["dx"])
        tdev = _lib.device_table(table)
        s_dev = torch.from_numpy(s).cuda()
        outs = []
        for mode in (_lib.FLAG_FUSED, _lib.FLAG_STAGED):
            d = _desc(diamond400, geo, len(s), p, _lib.H_SEGMENTS,
                      len(table), flags=mode | hflag)
            ws = torch.empty(_lib.lib().dyfox_laue_workspace_bytes(d),
                             dtype=torch.uint8, device="cuda")
            out = torch.full((len(s), geo["Ny"], geo["Nx"]), float("nan"),
                             dtype=p.torch_complex, device="cuda")
            stream = torch.cuda.current_stream()
            _lib.check(_lib.lib().dyfox_laue_solve(
                d, _lib.ptr(s_dev), None, _lib.ptr(tdev), _lib.ptr(out),
                _lib.ptr(ws), ws.numel(),
                _lib.c_void_p(stream.cuda_stream)), "dyfox_laue_solve")
            _lib.check(_lib.lib().dyfox_laue_solve_status(
                d, _lib.ptr(ws), ws.numel(),
                _lib.c_void_p(stream.cuda_stream)),
                "dyfox_laue_solve_status")
            outs.append(np_(out))
        assert geo["Nz"] >= 2
        assert np.isfinite(outs[1]).all(), (prec, geo["Nz"])
        assert outs[0].tobytes() == outs[1].tobytes(), (prec, geo["Nz"])


@pytest.mark.parametrize("n_chunks", [1, 3, 1000])
def test_host_copy_row_chunks_through_the_c_abi(gpu, diamond400, small_grid,
                                                rng, n_chunks):
    """dyfox_laue_solve_to_host with an explicit row-chunk count (one, a
    count that leaves a short last chunk, and more than the rows allow,
    which the library caps): host_out and out hold the bytes of
    dyfox_laue_solve."""
    from dyfox_gb300 import _lib
    from dyfox_gb300.grid import grid_arrays
    from dyfox_gb300.laue import _desc
    from dyfox_gb300.backend import precision as as_precision
    torch = gpu
    segs = random_segments(diamond400, small_grid, 3, rng)
    geo = grid_arrays(small_grid)
    s = np.linspace(-3e5, 3e5, 7)
    p = as_precision("fp32")
    table = _lib.segment_table(segs, diamond400.g_vec, diamond400.nu,
                               diamond400.a_core, geo["dx"])
    tdev = _lib.device_table(table)
    s_dev = torch.from_numpy(s).cuda()
    d = _desc(diamond400, geo, len(s), p, _lib.H_SEGMENTS, len(table),
              flags=_lib.FLAG_STAGED | _lib.FLAG_H_FP64)
    ws = torch.empty(_lib.lib().dyfox_laue_workspace_bytes(d),
                     dtype=torch.uint8, device="cuda")
    shape = (len(s), geo["Ny"], geo["Nx"])
    stream = torch.cuda.current_stream()
    want = torch.empty(shape, dtype=p.torch_complex, device="cuda")
    _lib.check(_lib.lib().dyfox_laue_solve(
        d, _lib.ptr(s_dev), None, _lib.ptr(tdev), _lib.ptr(want),
        _lib.ptr(ws), ws.numel(), _lib.c_void_p(stream.cuda_stream)),
        "dyfox_laue_solve")
    out = torch.full(shape, float("nan"), dtype=p.torch_complex,
                     device="cuda")
    host = torch.full(shape, float("nan"), dtype=p.torch_complex,
                      pin_memory=True)
    _lib.check(_lib.lib().dyfox_laue_solve_to_host(
        d, _lib.ptr(s_dev), None, _lib.ptr(tdev), _lib.ptr(out),
        _lib.c_void_p(host.data_ptr()), _lib.ptr(ws), ws.numel(), n_chunks,
        _lib.c_void_p(stream.cuda_stream), None), "dyfox_laue_solve_to_host")
    _lib.check(_lib.lib().dyfox_laue_solve_status(
        d, _lib.ptr(ws), ws.numel(), _lib.c_void_p(stream.cuda_stream)),
        "dyfox_laue_solve_status")
    torch.cuda.synchronize()
    w = np_(want)
    assert np_(out).tobytes() == w.tobytes()
    assert host.numpy().tobytes() == w.tobytes()


@pytest.mark.parametrize("h_mode,h_sum", [("fused", "ff"),
                                           ("fused", "fp64"),
                                           ("staged", "ff")])
@pytest.mark.parametrize("n_seg", [1, 4])
def test_pair_march_agrees_with_scalar_march_bitwise(gpu, diamond400,
                                                    small_grid, h_mode, h_sum,
                                                    n_seg, rng):
    """Two deviation parameters per thread in packed f32x2 arithmetic give
    the scalar march's bits, at every pair shape, for even and odd angle
    counts (the last pair of an odd count repeats its angle)."""
    from dyfox_gb300.laue import _solve
    segs = geometry_n(diamond400, small_grid) if n_seg == 1 else \
        random_segments(diamond400, small_grid, n_seg, rng)
    for n_e in (2, 5):
        s = np.linspace(-3e5, 3e5, n_e)
        ref = np_(_solve(segs, s, small_grid, diamond400, None, 0, "fp32",
                         False, h_mode=h_mode, h_sum=h_sum, pairs=False,
                         tuned=False))
        for cpl, A in ((3, 2), (5, 4), (7, 6)):
            got = np_(_solve(segs, s, small_grid, diamond400, None, 0,
                             "fp32", False, h_mode=h_mode, h_sum=h_sum,
                             pairs=True, cols_per_lane=cpl, angles_per_cta=A,
                             tuned=False))
            assert got.tobytes() == ref.tobytes(), (n_e, cpl, A)


def test_general_march_agrees_with_register_march(gpu, diamond400,
                                                 small_grid):
    from dyfox_gb300.dislocations import compute_H_grid
    from dyfox_gb300.laue import _solve
    seg = geometry_n(diamond400, small_grid)
    s = [0.0, 1.2e6]
    H = compute_H_grid(seg, small_grid, diamond400)
    a = np_(_solve(seg, s, small_grid, diamond400, H, 0, "fp64", False))
    b = np_(_solve(seg, s, small_grid, diamond400, H, 0, "fp64", False,
                   general=True))
    assert rel_l2(a, b) < 1e-13


def test_rows_outside_the_beam_are_zero(gpu, diamond400, small_grid):
    from dyfox_gb300.laue import solve_pristine
    out = np_(solve_pristine([0.0, 1e5], small_grid, diamond400))
    Ny = out.shape[1]
    y = (np.arange(Ny) - Ny // 2) * small_grid.dx
    dead = np.abs(y) >= small_grid.beam_width / 2
    assert dead.any() and np.all(out[:, dead] == 0)
    assert np.all(np.abs(out[:, ~dead]).max(axis=-1) > 0)


def test_pristine_matches_the_plane_wave_rocking_curve(gpu, diamond400):
    """Reference test_laue_gpu.py:59-70 (interpolating grid, Nz=801)."""
    from dyfox_gb300.grid import LaueGrid
    from dyfox_gb300.laue import solve_pristine
    grid = LaueGrid(diamond400, t_crystal=45e-6 / diamond400.tan_tB,
                    dx=0.25e-6, beam_width=20e-6, beam_thickness=120e-6,
                    Nz=801)
    Ny, Nx = grid.shape
    s = np.linspace(-6, 6, 25) / diamond400.xi_g
    got = np.abs(np_(solve_pristine(s, grid, diamond400))[:, Ny // 2,
                                                            Nx // 2]) ** 2
    want = CF.planewave_rocking(s, diamond400, grid.t_crystal)
    resid = got / got.max() - want / want.max()
    assert float(np.sqrt(np.mean(resid ** 2))) < 0.02


def test_the_coupling_sign_on_a_uniform_shear(gpu, diamond400):
    """H = q y imposed through H_gpu: the exit phase slope is -q."""
    from dyfox_gb300.grid import LaueGrid
    from dyfox_gb300.laue import solve_dislocation
    torch = gpu
    grid = LaueGrid(diamond400, t_crystal=20e-6, dx=0.25e-6,
                    beam_width=40e-6, beam_thickness=1e-6, Nz=101)
    Ny, Nx = grid.shape
    q = 2 * np.pi / 10e-6
    y = (torch.arange(Ny, dtype=torch.float64, device="cuda") - Ny / 2) \
        * grid.dx
    H = (q * y)[:, None, None].expand(Ny, grid.Nz, Nx).contiguous()
    out = np_(solve_dislocation([], [0.0], grid, diamond400, H_gpu=H))[0]
    rows = slice(Ny // 2 - 60, Ny // 2 + 60)
    phi = np.unwrap(np.angle(out[rows, Nx // 2]))
    slope = np.polyfit(np.arange(len(phi)) * grid.dx, phi, 1)[0]
    assert slope == pytest.approx(-q, rel=0.05)


def test_closed_form_and_grid_agree_on_a_line_along_x(gpu, diamond400,
                                                      small_grid):
    from dyfox_gb300.dislocations import (analytic_line_params,
                                          compute_H_grid)
    from dyfox_gb300.laue import solve_dislocation
    from dyfox_gb300.units import deviation_from_urad
    seg = mixed_on_x(diamond400, small_grid)
    assert analytic_line_params(seg, diamond400) is not None
    s = [float(deviation_from_urad(117.5, diamond400))]
    a = np_(solve_dislocation(seg, s, small_grid, diamond400))
    H = compute_H_grid(seg, small_grid, diamond400)
    b = np_(solve_dislocation(seg, s, small_grid, diamond400, H_gpu=H))
    assert rel_l2(a, b) < 1e-6


def test_zero_burgers_vector_march_is_pristine(gpu, diamond400, small_grid):
    from dyfox_gb300.laue import solve_dislocation, solve_pristine
    seg = geometry_n(diamond400, small_grid)
    dead = [(seg[0][0], seg[0][1], np.zeros(3))]
    s = [0.0, 5e5]
    a = np_(solve_dislocation(dead, s, small_grid, diamond400))
    b = np_(solve_pristine(s, small_grid, diamond400))
    assert rel_l2(a, b) < 1e-13


def test_bad_inputs_raise(gpu, diamond400, small_grid):
    from dyfox_gb300.laue import solve_dislocation, solve_pristine
    torch = gpu
    with pytest.raises(ValueError):
        solve_pristine([np.nan], small_grid, diamond400)
    with pytest.raises(ValueError):
        solve_dislocation([], [0.0], small_grid, diamond400,
                          H_gpu=torch.zeros(3, 3, 3, device="cuda",
                                            dtype=torch.float64))


def test_rocking_scan_configuration_meets_the_budget(gpu, diamond400):
    """The 273 um, 64-segment scan configuration on 8 of its angles: FP32
    compensated (staged and fused phase) against plain FP64."""
    from dyfox_gb300.laue import solve_dislocation
    from dyfox_gb300.workloads import laue_rocking_scan
    x, grid, segs, s = laue_rocking_scan(n_angles=8)
    assert len(segs) == 64
    a = np_(solve_dislocation(segs, s, grid, x, precision="fp64"))
    for mode in ("staged", "fused"):
        b = np_(solve_dislocation(segs, s, grid, x, precision="fp32",
                                  h_mode=mode))
        assert rel_l2(np.abs(b) ** 2, np.abs(a) ** 2) < FP32_INTENSITY_TOL


def test_autotuner_caches_a_shape_that_changes_nothing(gpu, diamond400,
                                                      small_grid, tmp_path,
                                                      monkeypatch):
    """The tuner times (columns per lane, angles per CTA) candidates, caches
    the fastest, and solves read the cache; the shape never changes a bit
    of the result."""
    from dyfox_gb300 import autotune
    from dyfox_gb300.laue import describe, solve_dislocation
    monkeypatch.setenv("DYFOX_TUNE_CACHE", str(tmp_path / "tune.json"))
    monkeypatch.setattr(autotune, "_cache", None)
    seg = geometry_n(diamond400, small_grid)
    s = np.linspace(-3e5, 3e5, 3)
    before = np_(solve_dislocation(seg, s, small_grid, diamond400,
                                   precision="fp32"))
    r = autotune.tune(seg, s, small_grid, diamond400, precision="fp32",
                      ctas=64)
    assert len(r["candidates"]) >= 2
    assert (tmp_path / "tune.json").exists()
    d = describe(seg, s, small_grid, diamond400, precision="fp32")
    assert autotune.lookup(d) == (r["cols_per_lane"], r["angles_per_cta"],
                                  r["pairs"])
    after = np_(solve_dislocation(seg, s, small_grid, diamond400,
                                  precision="fp32"))
    assert before.tobytes() == after.tobytes()


def test_wave_cache_solves_once_and_reloads(gpu, diamond400, small_grid,
                                            tmp_path):
    """A miss solves and stores complex64 under the key's file name; a hit
    reads it back; other inputs get another file."""
    import os
    from dyfox_gb300.cache import WaveCache
    from dyfox_gb300.laue import solve_dislocation
    torch = gpu
    seg = geometry_n(diamond400, small_grid)
    s = [0.0, 1e5]
    cache = WaveCache(str(tmp_path))
    a = cache.solve(seg, s, small_grid, diamond400)
    path = cache.path(seg, s, small_grid, diamond400)
    assert os.path.exists(path)
    ref = np_(solve_dislocation(seg, s, small_grid, diamond400))
    assert np.array_equal(np_(a), ref)
    b = cache.solve(seg, s, small_grid, diamond400)
    assert b.dtype == torch.complex64 and b.is_cuda
    assert np.array_equal(np_(b), ref.astype(np.complex64))
    cache.solve(seg, [0.0], small_grid, diamond400)
    assert len(os.listdir(tmp_path)) == 2
