"""The imaging stage: an objective, a pupil, and a spiral phase plate.

Drop-in for DYFOX ``optics.py``:

    lens = Optics(NA=1e-4, f_lens=0.274, xtal=xtal)
    open_img = lens.image(stack, dx, ell=0)
    spiral = lens.image(stack, dx, ell=+2)

Pupils, arguments, caching and the DC-zero policies follow
optics.py:37-167; images are ``|ifft2(fft2(u) ifftshift(P))|^2`` computed
by ``dyfox_image`` (for even grid sizes this equals the reference's
shifted composition, optics.py:170-207).  Arrays are torch CUDA tensors;
complex128 stacks give float64 images, complex64 stacks float32 images.
``object_spectrum`` / ``image_from_spectrum`` (the shifted spectra as
separate steps) are not provided: the images are computed in one pass.
"""

import ctypes

import numpy as np

from . import _lib
from .backend import FP64, precision as as_precision

_SIG = {
    "dyfox_pupil": (_lib.c_int, [
        _lib.c_int, _lib.c_int, _lib.c_double, _lib.c_double, _lib.c_int,
        _lib.c_double, _lib.c_double, _lib.c_double, _lib.c_double,
        _lib.c_int, _lib.c_int, _lib.c_int, _lib.c_void_p, _lib.c_void_p]),
    "dyfox_image_workspace_bytes": (_lib.c_int, [
        _lib.c_int, _lib.c_int, _lib.c_int, _lib.c_int,
        ctypes.POINTER(_lib.c_size_t)]),
    "dyfox_image": (_lib.c_int, [
        _lib.c_void_p, _lib.c_int, _lib.c_int, _lib.c_int, _lib.c_int,
        _lib.c_void_p, _lib.c_void_p, _lib.c_void_p, _lib.c_void_p,
        _lib.c_void_p, _lib.c_void_p, _lib.c_void_p, _lib.c_size_t,
        _lib.c_void_p]),
}
_bound = False
_ws = {}


def _L():
    global _bound
    L = _lib.lib()
    if not _bound:
        for name, (res, args) in _SIG.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _bound = True
    return L


def _prec_of(t):
    torch = _lib.torch_cuda()
    if t.dtype == torch.complex128:
        return _lib.DYFOX_FP64
    if t.dtype == torch.complex64:
        return _lib.DYFOX_FP32
    raise ValueError(f"expected a complex64 or complex128 tensor, not "
                     f"{t.dtype}")


def _workspace(nbytes):
    torch = _lib.torch_cuda()
    dev = torch.cuda.current_device()
    buf = _ws.get(dev)
    if buf is None or buf.numel() < nbytes:
        buf = torch.empty(max(int(nbytes), 256), dtype=torch.uint8,
                          device="cuda")
        _ws[dev] = buf
    return buf


class Optics:
    """An objective of given numerical aperture, viewing a given crystal.
    Pupils are cached on every argument that shapes them."""

    def __init__(self, NA, f_lens, xtal, *, precision=FP64, xp=None):
        self.NA = float(NA)
        self.f_lens = float(f_lens)
        self.xtal = xtal
        self.precision = as_precision(precision)
        self.xp = xp
        self._cache = {}

    @property
    def aperture_f(self):
        """Radius of the NA disc in spatial frequency."""
        return self.NA / self.xtal.lam

    def resolution(self):
        """Rayleigh resolution in metres."""
        return 0.61 * self.xtal.lam / self.NA

    def pupil(self, Nx, Ny, dx, ell=0, *, aperture_f=(0.0, 0.0),
              singularity_f=(0.0, 0.0), dc_zero="exact", levels=0,
              cache=True):
        """The pupil on the fftshifted frequency grid, (Ny, Nx) complex
        CUDA tensor of the optics' precision."""
        torch = _lib.torch_cuda()
        ax, ay = float(aperture_f[0]), float(aperture_f[1])
        sx, sy = float(singularity_f[0]), float(singularity_f[1])
        key = (Nx, Ny, float(dx), int(ell), ax, ay, sx, sy, dc_zero,
               int(levels), self.precision.name, self.NA, self.xtal.lam)
        if cache and key in self._cache:
            return self._cache[key]
        zero = int(ell) != 0 and self._zero_dc(dc_zero, sx, sy,
                                               1.0 / (Nx * dx))
        out = torch.empty((int(Ny), int(Nx)),
                          dtype=self.precision.torch_complex, device="cuda")
        _lib.check(_L().dyfox_pupil(
            int(Nx), int(Ny), float(dx), self.aperture_f, int(ell), ax, ay,
            sx, sy, 1 if zero else 0, int(levels), self.precision.code,
            _lib.ptr(out), _lib.stream_ptr()), "dyfox_pupil")
        if cache:
            self._cache[key] = out
        return out

    @staticmethod
    def _zero_dc(policy, sx, sy, fx_step):
        if policy == "never":
            return False
        if policy == "exact":
            return sx == 0.0 and sy == 0.0
        if policy == "half_bin":
            return abs(sx) < 0.5 * fx_step and abs(sy) < 0.5 * fx_step
        raise ValueError(f"dc_zero is 'exact', 'half_bin' or 'never', "
                         f"not {policy!r}")

    def spiral(self, Nx, Ny, dx, ell=0, offset_bfp=(0.0, 0.0), levels=0,
               cache=True):
        """Pupil with the plate displaced by ``offset_bfp`` metres in the
        back focal plane (the singularity moves, the aperture stays)."""
        dfx = offset_bfp[0] / (self.xtal.lam * self.f_lens)
        dfy = offset_bfp[1] / (self.xtal.lam * self.f_lens)
        return self.pupil(Nx, Ny, dx, ell, singularity_f=(dfx, dfy),
                          dc_zero="exact", levels=levels, cache=cache)

    def chromatic(self, Nx, Ny, dx, ell, delta_E, levels=0,
                  dc_zero="never", cache=True):
        """Pupil seen by photons at a relative energy offset ``delta_E``:
        aperture and singularity slide by sin(2 theta_B) delta_E /
        lambda."""
        dfx = self.xtal.sin_2tB * delta_E / self.xtal.lam
        return self.pupil(Nx, Ny, dx, ell, aperture_f=(dfx, 0.0),
                          singularity_f=(dfx, 0.0), dc_zero=dc_zero,
                          levels=levels, cache=cache)

    def image(self, stack, dx, ell=0, offset_bfp=(0.0, 0.0), levels=0):
        """Image intensity of a stack of exit waves through one pupil."""
        Ny, Nx = stack.shape[-2:]
        pup = self.spiral(Nx, Ny, dx, ell, offset_bfp, levels)
        return image_intensity(stack, pup)

    def images(self, field, dx, ells=(0, 2), offset_bfp=(0.0, 0.0)):
        """One exit wave through several charges: (n_ells, Ny, Nx)."""
        Ny, Nx = field.shape[-2:]
        pups = [self.spiral(Nx, Ny, dx, e, offset_bfp) for e in ells]
        return apply_pupils(field, pups)

    def clear_cache(self):
        self._cache.clear()

    def __repr__(self):
        return (f"Optics(NA={self.NA:g}, f={self.f_lens:g} m, "
                f"{getattr(self.xtal, 'label', '')}, "
                f"{int(self.resolution() * 1e9)} nm)")


def _run_image(stack, pupil, out=None, phi=None, sum_wI=None, sum_I=None,
               rock=None):
    torch = _lib.torch_cuda()
    st = stack.contiguous()
    squeeze = st.ndim == 2
    if squeeze:
        st = st[None]
    n, Ny, Nx = st.shape
    prec = _prec_of(st)
    pup = pupil.contiguous()
    if pup.dtype != st.dtype or tuple(pup.shape) != (Ny, Nx):
        raise ValueError("pupil must match the stack's (Ny, Nx) and dtype")
    nb = _lib.c_size_t()
    _lib.check(_L().dyfox_image_workspace_bytes(n, Ny, Nx, prec,
                                                ctypes.byref(nb)),
               "dyfox_image_workspace_bytes")
    ws = _workspace(nb.value)
    _lib.check(_L().dyfox_image(
        _lib.ptr(st), n, Ny, Nx, prec, _lib.ptr(pup), _lib.ptr(out),
        _lib.ptr(phi), _lib.ptr(sum_wI), _lib.ptr(sum_I), _lib.ptr(rock),
        _lib.ptr(ws), ws.numel(), _lib.stream_ptr()), "dyfox_image")
    return squeeze


def image_intensity(stack, pupil):
    """A stack (n, Ny, Nx) or one wave (Ny, Nx) through one pupil."""
    torch = _lib.torch_cuda()
    real = torch.float64 if stack.dtype == torch.complex128 else torch.float32
    out = torch.empty(stack.shape, dtype=real, device="cuda")
    _run_image(stack, pupil, out=out)
    return out


def apply_pupils(field, pupils):
    """One exit wave through several pupils: (n_pupils, Ny, Nx)."""
    torch = _lib.torch_cuda()
    return torch.stack([image_intensity(field, p) for p in pupils])


def accumulate_com(stack, pupil, phi, sum_wI, sum_I):
    """The reduction of com_maps for one batch of a scan: sum_I += sum_s I,
    sum_wI += sum_s phi(s) I over the stack's images (double sums on the
    GPU, accumulated in place); returns sum_xy I per image (NumPy)."""
    torch = _lib.torch_cuda()
    n = stack.shape[0]
    ph = torch.as_tensor(np.asarray(phi, np.float64), dtype=torch.float64)
    ph = ph.to("cuda")
    rock = torch.empty(n, dtype=torch.float64, device="cuda")
    _run_image(stack, pupil, phi=ph, sum_wI=sum_wI, sum_I=sum_I, rock=rock)
    return rock.cpu().numpy()
