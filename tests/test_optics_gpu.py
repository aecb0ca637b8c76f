"""Imaging and rocking-scan maps against the reference's own optics
(golden vectors of tests/golden/optics_small.npz, made from DYFOX
optics.py) and the com_maps reduction restated with NumPy in the test.

Tolerances: FP64 pupils and images <= 1e-12 relative (FFT rounding);
FP32 images <= 1e-5; the double-precision sums <= 1e-12."""

import numpy as np
import pytest

from conftest import golden, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def og(gpu):
    return golden("optics_small")


def _lens(og, diamond400, precision="fp64"):
    from dyfox_gb300.optics import Optics
    assert diamond400.lam == pytest.approx(float(og["lam"]), rel=1e-15)
    return Optics(NA=float(og["NA"]), f_lens=float(og["f_lens"]),
                  xtal=diamond400, precision=precision)


def test_pupils_match_the_reference(gpu, og, diamond400):
    lens = _lens(og, diamond400)
    Ny, Nx, dx = int(og["Ny"]), int(og["Nx"]), float(og["dx"])
    for k, ell in enumerate(og["case_ell"]):
        p = lens.pupil(Nx, Ny, dx, int(ell),
                       aperture_f=tuple(og["case_aperture"][k]),
                       singularity_f=tuple(og["case_singularity"][k]),
                       dc_zero=str(og["case_dc"][k]),
                       levels=int(og["case_levels"][k]), cache=False)
        got = p.cpu().numpy()
        want = og["pupils"][k]
        assert np.array_equal(np.abs(got) > 0, np.abs(want) > 0), k
        assert np.abs(got - want).max() < 1e-12, k


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("fp32", 1e-5)])
def test_images_match_the_reference(gpu, og, precision, tol):
    from dyfox_gb300.optics import image_intensity
    torch = gpu
    cdt = torch.complex128 if precision == "fp64" else torch.complex64
    stack = torch.tensor(og["stack"]).to(cdt).cuda()
    for j, k in enumerate(og["image_pupils"]):
        pup = torch.tensor(og["pupils"][k]).to(cdt).cuda()
        img = image_intensity(stack, pup).cpu().numpy()
        assert rel_l2(img, og["images"][j]) < tol, k
        one = image_intensity(stack[1], pup).cpu().numpy()
        assert rel_l2(one, og["images"][j][1]) < tol


def test_com_reduction(gpu, og):
    """sum_I, sum_wI and the rocking curve of one batch, accumulated onto
    existing sums, against NumPy on the reference's images."""
    from dyfox_gb300.optics import accumulate_com
    torch = gpu
    stack = torch.tensor(og["stack"]).cuda()
    pup = torch.tensor(og["pupils"][og["image_pupils"][1]]).cuda()
    want_I = og["images"][1]
    phi = og["phi"]
    base = np.random.default_rng(1).random((int(og["Ny"]), int(og["Nx"])))
    sI = torch.tensor(base).cuda()
    sW = torch.tensor(2 * base).cuda()
    rock = accumulate_com(stack, pup, phi, sW, sI)
    assert rel_l2(sI.cpu().numpy(), base + want_I.sum(0)) < 1e-12
    assert rel_l2(sW.cpu().numpy(),
                  2 * base + (phi[:, None, None] * want_I).sum(0)) < 1e-12
    assert rel_l2(rock, want_I.sum(axis=(1, 2))) < 1e-12


@pytest.mark.parametrize("batch,chunk", [(3, 16), (None, 2)])
def test_com_maps_end_to_end(gpu, diamond400, small_grid, batch, chunk):
    """com_maps over a small scan (in march batches of 3 angles, or all at
    once imaged 2 at a time) equals the same reduction written out over the
    whole stack with the library's own solve and imaging calls."""
    from dyfox_gb300.laue import solve_dislocation
    from dyfox_gb300.optics import Optics, image_intensity
    from dyfox_gb300.rocking import com_maps
    from dyfox_gb300.units import deviation_from_urad, urad_from_deviation
    torch = gpu
    grid = small_grid
    lens = Optics(NA=2e-4, f_lens=0.274, xtal=diamond400)
    s = deviation_from_urad(np.linspace(-60, 60, 7), diamond400)
    b = diamond400.b_mag * np.array([1.0, 0.0, -1.0]) / np.sqrt(2.0)
    seg = [(np.array([-200e-6, 0.3e-6, 10e-6]),
            np.array([200e-6, 0.3e-6, 10e-6]), b)]
    com, rock, weight = com_maps(seg, s, grid, diamond400, lens,
                                 ells=(0, 2), batch=batch, image_chunk=chunk)
    phi = urad_from_deviation(s, diamond400)
    stack = solve_dislocation(seg, s, grid, diamond400)
    for ell in (0, 2):
        pup = lens.spiral(stack.shape[-1], stack.shape[-2], grid.dx, ell)
        I = image_intensity(stack, pup).cpu().numpy()
        sI = I.sum(0)
        assert rel_l2(weight[ell], sI) < 1e-12
        assert rel_l2(rock[ell], I.sum(axis=(1, 2))) < 1e-12
        want = (phi[:, None, None] * I).sum(0) / np.maximum(sI, 1e-300)
        assert np.abs(com[ell] - want).max() < 1e-9 * np.abs(phi).max()
