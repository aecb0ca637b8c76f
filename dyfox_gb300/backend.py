"""The two floating-point precisions and array helpers.

Mirrors DYFOX ``backend.py:49-99``: ``FP64`` and ``FP32`` objects carry their
NumPy/torch dtypes and are passed to the solvers as ``precision=``.  FP64 is
the parity mode (double everywhere).  FP32 here is the compensated mode: a
single-precision march with compensated (Fast2Sum) amplitude updates, the
displacement phase summed over segments and reduced mod 2 pi in
float-float (or in double, ``h_sum="fp64"``); in the Bragg solve,
single-precision Krylov products with float-float residuals.
Results come back as torch CUDA tensors; ``to_numpy`` copies any of them to
the host.
"""

import numpy as np

from . import _lib


class Precision:
    """One precision: ``real``/``complex`` NumPy dtypes, ``torch_real``/
    ``torch_complex`` torch dtypes, ``code`` for the C ABI."""

    def __init__(self, name):
        if name not in ("fp64", "fp32"):
            raise ValueError(f"precision is 'fp64' or 'fp32', not {name!r}")
        self.name = name
        self.is_fp32 = name == "fp32"
        self.real = np.float32 if self.is_fp32 else np.float64
        self.complex = np.complex64 if self.is_fp32 else np.complex128
        self.itemsize = 4 if self.is_fp32 else 8
        self.code = _lib.DYFOX_FP32 if self.is_fp32 else _lib.DYFOX_FP64

    @property
    def torch_real(self):
        import torch
        return torch.float32 if self.is_fp32 else torch.float64

    @property
    def torch_complex(self):
        import torch
        return torch.complex64 if self.is_fp32 else torch.complex128

    def scalar(self, x):
        return self.real(x)

    def __repr__(self):
        return f"Precision({self.name!r})"


FP64 = Precision("fp64")
FP32 = Precision("fp32")


def precision(name):
    """FP64 or FP32 from a name or a Precision (duck-typed on ``is_fp32``)."""
    if isinstance(name, Precision):
        return name
    if hasattr(name, "is_fp32"):
        return FP32 if name.is_fp32 else FP64
    return FP32 if str(name).lower() in ("fp32", "32", "single") else FP64


def to_numpy(a):
    """Host copy of a torch tensor, a CuPy array or anything array-like."""
    if hasattr(a, "detach") and hasattr(a, "cpu"):
        return a.detach().cpu().numpy()
    if hasattr(a, "get"):
        return a.get()
    return np.asarray(a)


def free_gpu():
    """Return cached device memory to the driver."""
    import sys
    torch = sys.modules.get("torch")
    if torch is not None and torch.cuda.is_available():
        torch.cuda.empty_cache()
