"""Exit waves stored on disk, keyed by the inputs that produced them.

Drop-in for DYFOX ``laue/cache.py:35-75`` with the same file format, so
caches written by either interoperate: the key is the first 16 hex digits
of the SHA-1 of a sorted-keys JSON of the segments, deviation parameters,
``grid.key()``, ``xtal.key()``, precision name, stored dtype and format
version (9); files are ``<precision>_[<tag>_]<key>.npy`` holding the stack
as complex64 unless ``store_dtype`` says otherwise.

    waves = WaveCache("output/data/waves")
    stack = waves.solve(segs, s_dev, grid, xtal, tag="edge_+1")

``solve`` returns a torch CUDA tensor (from disk on a hit, from
``laue.solve_dislocation`` on a miss).

Restates DYFOX's WaveCache key and file format (MIT licence: see NOTICE).
"""

import hashlib
import json
import os

import numpy as np

from . import _lib
from .backend import FP64, precision as as_precision

VERSION = 9


class WaveCache:
    """A directory of solved exit waves, keyed by what produced them."""

    def __init__(self, directory, version=VERSION,
                 store_dtype=np.complex64):
        self.directory = directory
        self.version = version
        self.store_dtype = store_dtype

    def key(self, seg_list, s_dev_arr, grid, xtal, precision=FP64):
        """The hash under which this solve is filed."""
        prec = as_precision(precision)
        segs = [[[float(v) for v in np.asarray(part, float).ravel()]
                 for part in seg] for seg in seg_list]
        payload = dict(segments=segs,
                       s_dev=[float(s) for s in np.atleast_1d(s_dev_arr)],
                       grid=grid.key(), crystal=xtal.key(),
                       precision=prec.name,
                       store=np.dtype(self.store_dtype).name,
                       version=self.version)
        blob = json.dumps(payload, sort_keys=True).encode()
        return hashlib.sha1(blob).hexdigest()[:16]

    def path(self, seg_list, s_dev_arr, grid, xtal, precision=FP64, tag=""):
        """Where such a solve would live (the tag is for reading by eye)."""
        prec = as_precision(precision)
        key = self.key(seg_list, s_dev_arr, grid, xtal, prec)
        stem = f"{tag}_{key}" if tag else key
        return os.path.join(self.directory, f"{prec.name}_{stem}.npy")

    def solve(self, seg_list, s_dev_arr, grid, xtal, *, precision=FP64,
              H_gpu=None, batch=64, tag="", use_cache=True):
        """The exit-wave stack, from disk if it is there, else solved (and
        stored)."""
        from .laue import solve_dislocation
        torch = _lib.torch_cuda()
        if not use_cache:
            return solve_dislocation(seg_list, s_dev_arr, grid, xtal,
                                     H_gpu=H_gpu, batch=batch,
                                     precision=precision)
        path = self.path(seg_list, s_dev_arr, grid, xtal, precision, tag)
        if os.path.exists(path):
            return torch.from_numpy(np.load(path)).to("cuda")
        stack = solve_dislocation(seg_list, s_dev_arr, grid, xtal,
                                  H_gpu=H_gpu, batch=batch,
                                  precision=precision)
        os.makedirs(self.directory, exist_ok=True)
        np.save(path, stack.cpu().numpy().astype(self.store_dtype))
        return stack

    def __repr__(self):
        return f"WaveCache({self.directory!r}, v{self.version})"
