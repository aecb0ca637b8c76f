"""Batched uneven instances (one CUDA graph: one persistent Laue march
launch, one Bragg launch) against the same instances solved one call at a
time, and against FP64.

The batch runs the very arithmetic of the single-instance paths (the
e^{iH} staging of dyfox_laue_solve's staged mode, the same compensated
update, the same GMRES), so its Laue answers equal ``solve_dislocation(...,
precision="fp32", h_mode="staged")`` bit for bit and its Bragg answers
equal ``solve_scan`` (same CTA size) bit for bit.
"""

import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu


def np_(t):
    return t.detach().cpu().numpy()


def _small_set(x):
    from dyfox_gb300.bragg_geometry import BraggConfig, bragg_g_vector
    from dyfox_gb300.units import deviation_from_urad
    from dyfox_gb300.workloads import ExplicitLaueGrid, _segments_in_box
    rng = np.random.default_rng(11)
    out = []
    for (t, dx, Ny, Nx, nseg, n_e) in ((30e-6, 0.25e-6, 40, 128, 3, 5),
                                       (45e-6, 0.5e-6, 24, 256, 1, 1),
                                       (20e-6, 0.125e-6, 16, 96, 7, 9),
                                       (25e-6, 0.25e-6, 20, 200, 0, 3)):
        g = ExplicitLaueGrid(x, t, dx, Ny, Nx, beam_width=0.8 * Ny * dx,
                             sheet_hw=Nx * dx / 8)
        segs = _segments_in_box(x, rng, nseg, Nx * dx / 2, 0.4 * Ny * dx,
                                0.0, g.t_crystal) if nseg else []
        s = deviation_from_urad(np.linspace(-200, 150, n_e), x)
        out.append(dict(kind="laue", xtal=x, grid=g, segs=segs, s=s))
    for (t, dx, field, n_y, nseg, n_s) in ((6e-6, 0.5e-6, 32, 3, 2, 4),
                                           (9e-6, 0.25e-6, 32, 2, 5, 3)):
        cfg = BraggConfig(x, t_crystal=t, dx=dx, half_x=field * dx / 2)
        ys = (np.arange(n_y) - n_y / 2 + 0.5) * dx
        segs = _segments_in_box(x, rng, nseg, field * dx / 2, n_y * dx / 2,
                                0.0, cfg.t_crystal)
        s = deviation_from_urad(np.linspace(-8, 8, n_s), x)
        out.append(dict(kind="bragg", xtal=x, cfg=cfg, segs=segs, s=s, ys=ys,
                        g=bragg_g_vector(x)))
    return out


@pytest.fixture(scope="module")
def small_set(gpu, diamond400):
    return _small_set(diamond400)


@pytest.mark.parametrize("h_sum", ["ff", "fp64"])
def test_batch_equals_single_calls(gpu, small_set, h_sum):
    from dyfox_gb300.batch import Batch, from_workload
    from dyfox_gb300.bragg import solve_scan
    from dyfox_gb300.laue import solve_dislocation
    torch = gpu
    b = Batch(from_workload(small_set), h_sum=h_sum)
    b.run()
    b.check()          # every bounded wait of the replay completed
    torch.cuda.synchronize()
    for w, out, info in zip(small_set, b.outputs, b.infos):
        if w["kind"] == "laue":
            want = solve_dislocation(w["segs"], w["s"], w["grid"], w["xtal"],
                                     precision="fp32", h_mode="staged",
                                     h_sum=h_sum)
            assert out.dtype == torch.complex64
            assert torch.equal(out, want)
        else:
            want, winfo = solve_scan(w["segs"], w["s"], w["cfg"], w["ys"],
                                     w["xtal"], w["g"], precision="fp32")
            assert torch.equal(out, want)
            assert torch.equal(info, winfo)
            assert float(info[:, 0].max()) < 1e-10


def test_replays_are_identical_and_counted(gpu, small_set):
    from dyfox_gb300 import _lib
    from dyfox_gb300.batch import Batch, from_workload
    torch = gpu
    b = Batch(from_workload(small_set))
    n_kernels = b.kernel_count
    assert n_kernels >= 3
    n0 = _lib.lib().dyfox_launch_count()
    first = [o.clone() for o in b.run()]
    b.run()
    torch.cuda.synchronize()
    assert _lib.lib().dyfox_launch_count() - n0 == 2 * n_kernels
    for a, c in zip(first, b.outputs):
        assert torch.equal(a, c)


@pytest.mark.parametrize("cpl,warps", [(7, 4), (9, 16), (11, 8)])
def test_launch_shapes_change_nothing(gpu, small_set, cpl, warps):
    from dyfox_gb300.batch import Batch, from_workload
    torch = gpu
    ref = Batch(from_workload(small_set))
    ref.run()
    b = Batch(from_workload(small_set), cols_per_lane=cpl, warps=warps,
              ctas_per_sm=1)
    b.run()
    torch.cuda.synchronize()
    for w, a, c in zip(small_set, ref.outputs, b.outputs):
        if w["kind"] == "laue":
            assert torch.equal(a, c)


def test_laue_batch_matches_fp64(gpu, small_set):
    """Every Laue instance of the batch against the plain FP64 solve:
    exit-intensity relative L2 <= 1e-5."""
    from dyfox_gb300.batch import Batch, from_workload
    from dyfox_gb300.laue import solve_dislocation
    b = Batch(from_workload(small_set))
    b.run()
    for w, out in zip(small_set, b.outputs):
        if w["kind"] != "laue":
            continue
        ref = np_(solve_dislocation(w["segs"], w["s"], w["grid"], w["xtal"]))
        got = np_(out).astype(np.complex128)
        assert rel_l2(np.abs(got) ** 2, np.abs(ref) ** 2) < 1e-5


def test_mixed_precisions_of_bragg(gpu, small_set):
    """FP64 and mixed Bragg instances in one batch (two launches)."""
    from dyfox_gb300.backend import FP64
    from dyfox_gb300.batch import Batch, from_workload
    torch = gpu
    inst = from_workload(small_set)
    inst[-1].prec = FP64
    b = Batch(inst)
    b.run()
    torch.cuda.synchronize()
    bi = [i for i, w in enumerate(small_set) if w["kind"] == "bragg"]
    o32, o64 = b.outputs[bi[0]], b.outputs[bi[1]]
    for i in bi:
        assert float(b.infos[i][:, 0].max()) < 1e-10
    assert o32.abs().max() > 0 and o64.abs().max() > 0


def test_bad_items_are_rejected(gpu, small_set, diamond400):
    from dyfox_gb300.batch import Batch, LaueInstance
    from dyfox_gb300.workloads import ExplicitLaueGrid
    w = small_set[0]
    odd = ExplicitLaueGrid(diamond400, 30e-6, 0.25e-6, 16, 127,
                           beam_width=2e-6, sheet_hw=4e-6)
    with pytest.raises(NotImplementedError):
        Batch([LaueInstance(w["segs"], w["s"], odd, diamond400)])
    wide = ExplicitLaueGrid(diamond400, 30e-6, 0.25e-6, 16, 4096,
                            beam_width=2e-6, sheet_hw=4e-6)
    with pytest.raises(NotImplementedError):
        Batch([LaueInstance(w["segs"], w["s"], wide, diamond400)], warps=4)
    with pytest.raises(ValueError):
        Batch([LaueInstance(w["segs"], w["s"], w["grid"], diamond400)],
              cols_per_lane=6)


def test_empty_batch(gpu):
    from dyfox_gb300.batch import Batch
    b = Batch([])
    b.run()
    assert b.outputs == []


def _sample_of_the_configuration(n_laue=6, n_bragg=3, seed=4):
    """A seeded sample of ``workloads.batched_uneven()`` (the 512-instance
    configuration itself, not a hand-made set), limited to instances whose
    plain-FP64 check costs seconds: Laue instances of at most 1.5e9
    segment-voxel evaluations and 2e9 voxel-steps (316 of the 358 Laue
    instances are under 4e9), Bragg instances of at most 5e6 voxel-steps
    per march over all their systems."""
    from dyfox_gb300.workloads import batched_uneven
    inst = batched_uneven()
    laue, bragg = [], []
    for w in inst:
        if w["kind"] == "laue":
            g = w["grid"]
            vox = g.Ny * g.Nx * g.Nz
            if vox * len(w["segs"]) <= 1.5e9 and vox * len(w["s"]) <= 2e9:
                laue.append(w)
        else:
            c = w["cfg"]
            if c.Nx * c.Nz * len(w["ys"]) * len(w["s"]) <= 5e6:
                bragg.append(w)
    rng = np.random.default_rng(seed)
    pick_l = rng.choice(len(laue), n_laue, replace=False)
    pick_b = rng.choice(len(bragg), n_bragg, replace=False)
    return [laue[i] for i in pick_l] + [bragg[i] for i in pick_b]


def test_sampled_configuration_instances_match_fp64(gpu):
    """Nine instances drawn (seeded) from the batched configuration, solved
    in one batch in its measured form (complex64 Laue march with the H sum
    in double, mixed-precision Bragg), each against its own plain-FP64
    solve: Laue exit intensity <= 1e-5 relative L2; Bragg true residual
    <= 1e-10 and exit waves <= 1e-8 relative L2."""
    from dyfox_gb300.batch import Batch, from_workload
    from dyfox_gb300.bragg import solve_scan
    from dyfox_gb300.laue import solve_dislocation
    torch = gpu
    sample = _sample_of_the_configuration()
    assert sum(w["kind"] == "laue" for w in sample) == 6
    assert max(len(w["segs"]) for w in sample) > 1
    b = Batch(from_workload(sample), h_sum="fp64")
    b.run()
    torch.cuda.synchronize()
    for w, out, info in zip(sample, b.outputs, b.infos):
        if w["kind"] == "laue":
            ref = np_(solve_dislocation(w["segs"], w["s"], w["grid"],
                                        w["xtal"]))
            got = np_(out).astype(np.complex128)
            assert rel_l2(np.abs(got) ** 2, np.abs(ref) ** 2) < 1e-5
        else:
            ref, rinfo = solve_scan(w["segs"], w["s"], w["cfg"], w["ys"],
                                    w["xtal"], w["g"])
            assert float(info[:, 0].max()) < 1e-10
            assert rel_l2(np_(out), np_(ref)) < 1e-8
