"""Rocking-scan maps: drop-in for DYFOX ``analysis/rocking.py``.

    com, rock, weight = com_maps(segs, s_dev, grid, xtal, optics, ells=(0, 2))

``com_maps`` (analysis/rocking.py:37-83) runs a scan in batches of angles
and reduces it to one number per pixel, the angle that pixel's intensity is
centred on:

    COM(x, y) = sum_s phi(s) I(x, y, s) / sum_s I(x, y, s)

with I the image through each pupil charge.  By default the whole scan is
marched in one call (the e^{iH} field of the segments is then evaluated or
staged once for all angles; a 256-angle complex64 scan of 544 x 1056 is
1.2 GB), and the exit waves go in chunks of ``image_chunk`` straight into
``dyfox_image``, which images them and adds phi I and I into
double-precision sums on the GPU.  ``batch`` marches fewer angles at a time
where memory is short, as the reference does.  ``planewave_rocking`` is the
closed-form perfect-crystal curve (analysis/rocking.py:16-34).
"""

import numpy as np

from . import _lib
from .backend import FP64
from .laue import solve_dislocation
from .optics import accumulate_com
from .units import urad_from_deviation


def planewave_rocking(s_dev, xtal, t_crystal, absorption=True):
    """|D_g|^2 against deviation parameter for a perfect crystal."""
    s_dev = np.asarray(s_dev)
    sig_h = complex(xtal.sig_h)
    sig_hbar = complex(xtal.sig_hbar)
    alpha = -2 * np.pi * s_dev
    gam = np.sqrt(np.abs(sig_h * sig_hbar) + alpha ** 2 / 4)
    spath = t_crystal / xtal.cos_tB
    rc = np.abs(sig_h) ** 2 / gam ** 2 * np.sin(gam * spath) ** 2
    if absorption:
        rc = rc * np.exp(2 * complex(xtal.sig0).real * spath)
    return rc


def com_maps(seg_list, s_dev_arr, grid, xtal, optics, ells=(0, 2), *,
             batch=None, precision=FP64, image_chunk=16, h_mode="auto"):
    """Centre-of-mass maps of a rocking scan, per pupil charge.

    Returns (com, rock, weight): dicts keyed by charge of the maps in
    microradians (Ny, Nx), the integrated rocking curve (n_s), and the
    summed intensity that weighted the maps (Ny, Nx), all NumPy.
    ``batch``: angles per march call (None: all); ``image_chunk``: exit
    waves per imaging launch (their intermediate spectra stay in L2).
    """
    torch = _lib.torch_cuda()
    s = np.asarray(s_dev_arr, dtype=float)
    Nx, Ny = grid.geometry()[:2]
    phi = urad_from_deviation(s, xtal)
    sums_wI = {e: torch.zeros((Ny, Nx), dtype=torch.float64, device="cuda")
               for e in ells}
    sums_I = {e: torch.zeros((Ny, Nx), dtype=torch.float64, device="cuda")
              for e in ells}
    rock = {e: np.zeros(len(s)) for e in ells}
    batch = len(s) if not batch else int(batch)
    chunk = max(1, int(image_chunk))
    for bs in range(0, len(s), batch):
        be = min(bs + batch, len(s))
        stack = solve_dislocation(seg_list, s[bs:be], grid, xtal,
                                  precision=precision, h_mode=h_mode,
                                  batch=be - bs)
        for e in ells:
            pup = optics.spiral(Nx, Ny, grid.dx, e)
            if pup.dtype != stack.dtype:
                pup = pup.to(stack.dtype)
            for cs in range(0, be - bs, chunk):
                ce = min(cs + chunk, be - bs)
                rock[e][bs + cs:bs + ce] = accumulate_com(
                    stack[cs:ce], pup, phi[bs + cs:bs + ce], sums_wI[e],
                    sums_I[e])
        del stack
    com = {e: (sums_wI[e] / torch.clamp(sums_I[e], min=1e-300)).cpu().numpy()
           for e in ells}
    weight = {e: sums_I[e].cpu().numpy() for e in ells}
    return com, rock, weight
