"""Learned shooting guess for the Bragg solve.

A 4-level U-Net (32 base channels, bfloat16 storage, FP32 accumulation)
maps the near-surface displacement phase of a set of y-planes, plus the
deviation parameter, to the shooting unknown D_g(z=0) of every plane (the
``v`` of the solve, before the phase restoration).  It is trained on
answers of the plain solve and used only as the GMRES starting vector: the
solve keeps its own true-residual test, so a poor guess costs iterations,
never accuracy, and the zero start remains the fallback.  Training and
inference run on this library's kernels (dyfox_unet_*); there is no DYFOX
counterpart.

    net = UNet(batch=8, H=256, W=256, seed=0)
    hist = net.train(X, T, epochs=8, lr=1e-3)     # X bf16 (n,H,W,32), T f32 (n,H,W,2)
    y = net.predict(X)                            # (n, H, W, 2) float32

Input channels: cos and sin of H on the first 8 depth slices (channel 2k,
2k + 1), s / s_scale (channel 16), zeros (17..31); the rows are y-planes,
the columns a window of the lateral grid (``features``).  The network
predicts v minus the perfect-crystal solution v0(s) (``pristine_v``), so an
untrained network starts from the perfect-crystal guess.
"""

import ctypes

import numpy as np

from . import _lib

_SIG = {
    "dyfox_unet_param_count": (_lib.c_size_t, []),
    "dyfox_unet_workspace_bytes": (_lib.c_int, [
        _lib.c_int, _lib.c_int, _lib.c_int, ctypes.POINTER(_lib.c_size_t)]),
    "dyfox_unet_create": (_lib.c_int, [
        _lib.c_int, _lib.c_int, _lib.c_int, _lib.c_void_p, _lib.c_size_t,
        ctypes.POINTER(_lib.c_void_p)]),
    "dyfox_unet_destroy": (_lib.c_int, [_lib.c_void_p]),
    "dyfox_unet_params": (_lib.c_int, [
        _lib.c_void_p, ctypes.POINTER(_lib.c_void_p),
        ctypes.POINTER(_lib.c_void_p)]),
    "dyfox_unet_init": (_lib.c_int, [_lib.c_void_p, ctypes.c_ulonglong,
                                     _lib.c_void_p]),
    "dyfox_unet_refresh": (_lib.c_int, [_lib.c_void_p, _lib.c_void_p]),
    "dyfox_unet_forward": (_lib.c_int, [_lib.c_void_p, _lib.c_void_p,
                                        _lib.c_int, _lib.c_void_p,
                                        _lib.c_void_p]),
    "dyfox_unet_backward": (_lib.c_int, [_lib.c_void_p, _lib.c_void_p,
                                         _lib.c_void_p, _lib.c_void_p]),
    "dyfox_unet_adam": (_lib.c_int, [_lib.c_void_p, ctypes.c_float,
                                     ctypes.c_float, ctypes.c_float,
                                     ctypes.c_float, _lib.c_void_p]),
    "dyfox_unet_features": (_lib.c_int, [
        _lib.c_void_p, _lib.c_int, _lib.c_int, _lib.c_int, _lib.c_int,
        _lib.c_void_p, _lib.c_int, _lib.c_void_p, _lib.c_void_p]),
    "dyfox_unet_buffer": (_lib.c_int, [_lib.c_void_p, _lib.c_int, _lib.c_int,
                                       ctypes.POINTER(_lib.c_void_p),
                                       ctypes.POINTER(_lib.c_size_t)]),
    "dyfox_unet_conv": (_lib.c_int, [_lib.c_int] + [_lib.c_void_p] * 5
                        + [_lib.c_int] * 5 + [_lib.c_void_p, _lib.c_size_t,
                                              _lib.c_void_p]),
}
_bound = False

C_IN = 32
N_SLICES = 8
# Spatial level (size >> level) of each 3x3 convolution's output.
LEVEL_OF = (0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0)


def _L():
    global _bound
    L = _lib.lib()
    if not _bound:
        for name, (res, args) in _SIG.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        _bound = True
    return L


def param_count():
    return int(_L().dyfox_unet_param_count())


class UNet:
    """The network, its Adam state and its activations in one workspace."""

    def __init__(self, batch=8, H=256, W=256, seed=0):
        torch = _lib.torch_cuda()
        self.torch = torch
        self.batch, self.H, self.W = int(batch), int(H), int(W)
        L = _L()
        nb = _lib.c_size_t(0)
        _lib.check(L.dyfox_unet_workspace_bytes(self.batch, self.H, self.W,
                                                ctypes.byref(nb)),
                   "dyfox_unet_workspace_bytes")
        self.workspace = torch.empty(int(nb.value) + 256, dtype=torch.uint8,
                                     device="cuda")
        base = self.workspace.data_ptr()
        pad = (-base) % 256
        h = _lib.c_void_p()
        _lib.check(L.dyfox_unet_create(self.batch, self.H, self.W,
                                       _lib.c_void_p(base + pad), nb.value,
                                       ctypes.byref(h)), "dyfox_unet_create")
        self._h = h
        p, g = _lib.c_void_p(), _lib.c_void_p()
        _lib.check(L.dyfox_unet_params(h, ctypes.byref(p), ctypes.byref(g)),
                   "dyfox_unet_params")
        n = param_count()
        self.n_params = n
        self.params = self._view(p.value, n)
        self.grads = self._view(g.value, n)
        self.init(seed)

    def _view(self, ptr, n):
        off = ptr - self.workspace.data_ptr()
        return self.workspace[off:off + 4 * n].view(self.torch.float32)

    def buffer(self, which, index, n=None):
        """A copy of an internal buffer of the last pass, NHWC, first n
        samples: ("act", i) conv output, ("pool", l), ("cat", c),
        ("dout", i) gradient of conv output i."""
        torch = self.torch
        code = {"act": 0, "pool": 1, "cat": 2, "dout": 3}[which]
        p, nb = _lib.c_void_p(), _lib.c_size_t()
        _lib.check(_L().dyfox_unet_buffer(self._h, code, index,
                                          ctypes.byref(p), ctypes.byref(nb)),
                   "dyfox_unet_buffer")
        off = p.value - self.workspace.data_ptr()
        raw = self.workspace[off:off + nb.value]
        t = raw.view(torch.float32 if code == 3 else torch.bfloat16)
        if code in (0, 3):
            lv = LEVEL_OF[index]
        elif code == 1:
            lv = index + 1
        else:
            lv = 2 - index
        h, w = self.H >> lv, self.W >> lv
        t = t.view(self.batch, h, w, -1)
        return (t if n is None else t[:n]).float().clone()

    def init(self, seed=0):
        _lib.check(_L().dyfox_unet_init(self._h, int(seed), _lib.stream_ptr()),
                   "dyfox_unet_init")

    def load(self, flat):
        """Sets the FP32 parameters (flat, oracle layout) and refreshes the
        bfloat16 copies."""
        t = self.torch.as_tensor(np.asarray(flat, np.float32)
                                 if not hasattr(flat, "data_ptr") else flat)
        self.params.copy_(t.to(self.params.device, self.torch.float32))
        _lib.check(_L().dyfox_unet_refresh(self._h, _lib.stream_ptr()),
                   "dyfox_unet_refresh")

    def _check_x(self, x):
        torch = self.torch
        if x.dtype != torch.bfloat16 or x.device.type != "cuda":
            raise ValueError("x must be a CUDA bfloat16 tensor")
        if tuple(x.shape[1:]) != (self.H, self.W, C_IN) or x.shape[0] < 1 \
                or x.shape[0] > self.batch:
            raise ValueError(f"x has shape {tuple(x.shape)}, the network "
                             f"takes (<= {self.batch}, {self.H}, {self.W}, "
                             f"{C_IN})")
        return x.contiguous()

    def forward(self, x):
        """Head output (n, H, W, 2) float32 for a bf16 input (n, H, W, 32)."""
        x = self._check_x(x)
        y = self.torch.empty((x.shape[0], self.H, self.W, 2),
                             dtype=self.torch.float32, device="cuda")
        _lib.check(_L().dyfox_unet_forward(self._h, _lib.ptr(x), x.shape[0],
                                           _lib.ptr(y), _lib.stream_ptr()),
                   "dyfox_unet_forward")
        self._last = x
        return y

    def backward(self, target):
        """Gradients of L = sum((y - t)^2) / (2 y.size) for the last
        forward; returns L as a 0-d CUDA tensor."""
        t = target.contiguous()
        loss = self.torch.empty((), dtype=self.torch.float32, device="cuda")
        _lib.check(_L().dyfox_unet_backward(self._h, _lib.ptr(t),
                                            _lib.ptr(loss), _lib.stream_ptr()),
                   "dyfox_unet_backward")
        return loss

    def step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        _lib.check(_L().dyfox_unet_adam(self._h, lr, beta1, beta2, eps,
                                        _lib.stream_ptr()), "dyfox_unet_adam")

    def train(self, X, T, epochs=8, lr=1e-3, seed=0, lr_decay=0.5,
              decay_every=None, verbose=False):
        """Adam over shuffled mini-batches of ``batch`` samples; returns the
        mean loss of every epoch."""
        torch = self.torch
        n = X.shape[0]
        rng = np.random.default_rng(seed)
        hist = []
        for ep in range(epochs):
            lr_ep = lr * (lr_decay ** (ep // decay_every)) if decay_every \
                else lr
            order = rng.permutation(n)
            losses = []
            for b0 in range(0, n - self.batch + 1, self.batch):
                idx = torch.as_tensor(order[b0:b0 + self.batch],
                                      device="cuda")
                self.forward(X.index_select(0, idx))
                losses.append(self.backward(T.index_select(0, idx)))
                self.step(lr_ep)
            hist.append(float(torch.stack(losses).mean()))
            if verbose:
                print(f"epoch {ep}: loss {hist[-1]:.4e}")
        return hist

    def predict(self, X):
        """Head output for any number of samples (in batches)."""
        torch = self.torch
        out = torch.empty((X.shape[0], self.H, self.W, 2),
                          dtype=torch.float32, device="cuda")
        for b0 in range(0, X.shape[0], self.batch):
            out[b0:b0 + self.batch] = self.forward(X[b0:b0 + self.batch])
        return out

    def close(self):
        if getattr(self, "_h", None) is not None:
            _L().dyfox_unet_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def features(h_top, col0, W, s_scaled):
    """Network input (n_s, n_y, W, 32) bf16 from the top 8 depth slices of
    H (a (n_y, 8, Nx) float64 CUDA tensor) over columns [col0, col0 + W)
    and the scaled deviation parameters (n_s float64)."""
    torch = _lib.torch_cuda()
    h = h_top.contiguous()
    n_y, ns, Nx = h.shape
    if ns != N_SLICES:
        raise ValueError(f"h_top needs {N_SLICES} depth slices, has {ns}")
    s = torch.as_tensor(np.asarray(s_scaled, np.float64)
                        if not hasattr(s_scaled, "data_ptr") else s_scaled,
                        dtype=torch.float64).to("cuda")
    out = torch.empty((len(s), n_y, W, C_IN), dtype=torch.bfloat16,
                      device="cuda")
    _lib.check(_L().dyfox_unet_features(_lib.ptr(h), n_y, Nx, col0, W,
                                        _lib.ptr(s), len(s), _lib.ptr(out),
                                        _lib.stream_ptr()),
               "dyfox_unet_features")
    return out


def conv(mode, *, X=None, G=None, Wk=None, bias=None, Cin=None, Cout=None,
         mma_sync=False):
    """One 3x3 convolution product of the training kernels (checks):
    mode "fwd" -> bf16 relu(conv(X, Wk) + bias), "dgrad" -> float data
    gradient of G (Wk transposed [Cin][9][Cout]), "wgrad" -> float weight
    gradient [Cout][9][Cin] of X and G.  Tensors NHWC on the GPU.  The
    three products run on the tcgen05 tensor cores when the image rows fit
    their 128-pixel tiles; ``mma_sync=True`` takes the mma.sync implicit
    GEMM instead."""
    torch = _lib.torch_cuda()
    ref = X if X is not None else G
    N, H, W = ref.shape[:3]
    Cin = Cin if Cin is not None else X.shape[3]
    Cout = Cout if Cout is not None else G.shape[3]
    m = {"fwd": 0, "dgrad": 1, "wgrad": 2}[mode]
    flags = CONV_MMA_SYNC if mma_sync else 0
    ws = None
    if m == 0:
        out = torch.empty((N, H, W, Cout), dtype=torch.bfloat16, device="cuda")
    elif m == 1:
        out = torch.empty((N, H, W, Cin), dtype=torch.float32, device="cuda")
    else:
        out = torch.empty((Cout, 9, Cin), dtype=torch.float32, device="cuda")
        ws = torch.empty(64 * 9 * Cin * Cout * 4, dtype=torch.uint8,
                         device="cuda")
    _lib.check(_L().dyfox_unet_conv(
        m | flags, _lib.ptr(X), _lib.ptr(G), _lib.ptr(Wk), _lib.ptr(bias),
        _lib.ptr(out), N, H, W, Cin, Cout, _lib.ptr(ws),
        0 if ws is None else ws.numel(), _lib.stream_ptr()),
        "dyfox_unet_conv")
    return out


CONV_MMA_SYNC = 16


def tc_error(clear=True):
    """Error code of the tcgen05 convolutions' bounded waits (0: none)."""
    import ctypes
    code = ctypes.c_int(0)
    f = _L().dyfox_unet_tc_error
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    _lib.check(f(ctypes.byref(code), int(bool(clear))), "dyfox_unet_tc_error")
    return code.value


# ---------------------------------------------------------------------------
# The shooting guess of the Bragg solve.

def s_scale(xtal):
    """The deviation parameter of 5 Darwin widths (input scaling)."""
    from .bragg_geometry import darwin_width_urad
    from .units import deviation_from_urad
    return float(deviation_from_urad(5 * darwin_width_urad(xtal), xtal))


def pristine_v(s_values, cfg, xtal):
    """Perfect-crystal shooting unknown v0(s) = -T21 / T22 of the lateral
    DC mode (plane-wave incidence), per deviation parameter."""
    from .bragg import perfect_symbol
    s0 = complex(xtal.sig0)
    out = np.empty(len(s_values), complex)
    for i, s in enumerate(np.atleast_1d(s_values)):
        alpha = -2.0 * np.pi * float(s)
        e0 = np.exp(s0 * cfg.ds)
        eg = np.exp((s0 + 1j * alpha) * cfg.ds)
        T21, T22 = perfect_symbol(e0, eg, cfg.ds, cfg.Nz, cfg.Nx, xtal)
        out[i] = -T21[0] / T22[0]
    return out


def full_width(Nx):
    """Network width covering a periodic lateral grid of Nx columns."""
    return -(-int(Nx) // 8) * 8


def instance_h(inst):
    """H on the first 8 depth slices of every plane, (n_y, 8, Nx)."""
    torch = _lib.torch_cuda()
    from .dislocations import H_rows
    cfg, x = inst["cfg"], inst["xtal"]
    ys = np.asarray(inst["ys"], float)
    if inst["segs"]:
        return H_rows(inst["segs"], cfg.Nx, N_SLICES, cfg.dx, cfg.dz,
                      inst["g"], x.nu, x.a_core, ys)
    return torch.zeros((len(ys), N_SLICES, cfg.Nx), dtype=torch.float64,
                       device="cuda")


def instance_inputs(inst, col0=None, width=None, h=None):
    """(features (n_s, n_y, width, 32) bf16 of columns col0 .. col0 +
    width (mod Nx), H at z = 0 (n_y, Nx) float64, v0 (n_s,) complex) of a
    learned-guess instance; the field of interest by default."""
    x = inst["xtal"]
    h = instance_h(inst) if h is None else h
    col0 = inst["col0"] if col0 is None else col0
    width = inst["field"] if width is None else width
    X = features(h, col0, width, np.asarray(inst["s"], float) / s_scale(x))
    return X, h[:, 0, :].contiguous(), pristine_v(inst["s"], inst["cfg"], x)


def solve_instance(inst, x0=None, tol=1e-8, precision="fp32", restart=40,
                   maxiter=25):
    """The Bragg solve of every (s, plane) system of an instance, timed on
    the device: (v (n_s, n_y, Nx) complex128 before the phase restoration,
    info (n_s n_y, 4), ms)."""
    torch = _lib.torch_cuda()
    from .bragg import solve_scan
    cfg = inst["cfg"]
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    out, info = solve_scan(inst["segs"], inst["s"], cfg, inst["ys"],
                           inst["xtal"], inst["g"], tol=tol, restart=restart,
                           maxiter=maxiter, x0=x0, precision=precision)
    b.record()
    torch.cuda.synchronize()
    return out, info, a.elapsed_time(b)


def targets(v, h0, v0, col0, field):
    """Training target of an instance: v (phase-restored solution times
    e^{+iH(0)}) minus v0 over columns col0 .. col0 + field (mod Nx), as
    (n_s, n_y, field, 2) float32."""
    torch = _lib.torch_cuda()
    vv = v * torch.exp(1j * h0)[None]
    Nx = vv.shape[-1]
    cols = torch.arange(col0, col0 + field, device="cuda") % Nx
    d = vv.index_select(2, cols) - torch.as_tensor(v0, device="cuda")[
        :, None, None]
    return torch.view_as_real(d.to(torch.complex64)).contiguous()


def initial_guess(inst, v0, y=None, col0=None):
    """x0 of the solve: v0(s) on every column of every plane, plus the
    network's prediction y (n_s, n_y, width, 2) on columns col0 .. col0 +
    width (mod Nx; the field of interest by default).  A prediction of
    the full width (col0 = 0, width >= Nx) covers every column."""
    torch = _lib.torch_cuda()
    cfg = inst["cfg"]
    n_s, n_y = len(inst["s"]), len(inst["ys"])
    x0 = torch.as_tensor(v0, dtype=torch.complex128, device="cuda")[
        :, None, None].expand(n_s, n_y, cfg.Nx).clone()
    if y is not None:
        c0 = inst["col0"] if col0 is None else col0
        width = min(int(y.shape[2]), cfg.Nx)
        cols = torch.arange(c0, c0 + width, device="cuda") % cfg.Nx
        x0.index_add_(2, cols, torch.view_as_complex(
            y[:, :, :width].contiguous()).to(torch.complex128))
    return x0.contiguous()


def predict_full(net, inst, h=None, batch=None):
    """The network applied to the whole periodic lateral grid of an
    instance (a fully convolutional network trained on windows):
    (n_s, n_y, full_width(Nx), 2) float32.  ``net`` supplies the trained
    parameters; a network of the full width shares them."""
    cfg = inst["cfg"]
    W = full_width(cfg.Nx)
    key = (len(inst["ys"]), W)
    cache = getattr(net, "_full", {})
    wide = cache.get(key)
    if wide is None:
        wide = UNet(batch=batch or net.batch, H=len(inst["ys"]), W=W)
        cache[key] = wide
        net._full = cache
    wide.load(net.params)
    X, _, _ = instance_inputs(inst, col0=0, width=W, h=h)
    return wide.predict(X)
