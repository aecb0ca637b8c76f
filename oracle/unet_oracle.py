"""ORACLE -- test infrastructure only.  NumPy FP64 forward and backward of
the learned shooting-guess U-Net, written from the layer definitions
(DYFOX has no learned part; this oracle is pinned by finite differences in
tests/test_unet_oracle_cpu.py and is the checker of the CUDA kernels).

Network (NHWC; every 3x3 convolution is zero-padded, stride 1, followed by
bias and ReLU):

    input  (N, H, W, 32)    17 used channels, 15 zero
    enc0   conv 32->32, conv 32->32           (H, W)
    enc1   avgpool 2, conv 32->64, conv 64->64
    enc2   avgpool 2, conv 64->128, conv 128->128
    bott   avgpool 2, conv 128->256, conv 256->256   (H/8, W/8)
    dec2   concat(up2(bott), enc2) 384 -> conv 128, conv 128->128
    dec1   concat(up2(dec2), enc1) 192 -> conv 64, conv 64->64
    dec0   concat(up2(dec1), enc0) 96 -> conv 32, conv 32->32
    head   1x1 conv 32 -> 2 (+ bias, no activation)
    loss   L = sum((y - t)^2) / (2 * y.size)

``bf16=True`` rounds to bfloat16 (round to nearest even) exactly where the
CUDA kernels store bfloat16: the weights of every convolution, each ReLU
output, each pooled / concatenated tensor, and each masked gradient G =
dL/dY * (Y > 0) that feeds the backward products.  Accumulations and the
head stay in FP64 here (FP32 on the GPU).
"""

import numpy as np

C_IN = 32
LEVELS = (32, 64, 128, 256)

# (name, Cin, Cout) of the 3x3 convolutions in forward order.
CONVS = [("e0a", C_IN, 32), ("e0b", 32, 32),
         ("e1a", 32, 64), ("e1b", 64, 64),
         ("e2a", 64, 128), ("e2b", 128, 128),
         ("ba", 128, 256), ("bb", 256, 256),
         ("d2a", 384, 128), ("d2b", 128, 128),
         ("d1a", 192, 64), ("d1b", 64, 64),
         ("d0a", 96, 32), ("d0b", 32, 32)]
HEAD = ("head", 32, 2)


def param_layout():
    """[(name, shape)] of the flat FP32 parameter vector, in order: per 3x3
    convolution W (Cout, 3, 3, Cin) then b (Cout); then the head's W (2, 32)
    and b (2)."""
    out = []
    for name, ci, co in CONVS:
        out.append((name + ".W", (co, 3, 3, ci)))
        out.append((name + ".b", (co,)))
    out.append(("head.W", (2, 32)))
    out.append(("head.b", (2,)))
    return out


def n_params():
    return sum(int(np.prod(s)) for _, s in param_layout())


def unflatten(flat):
    p, o = {}, 0
    for name, shape in param_layout():
        n = int(np.prod(shape))
        p[name] = np.asarray(flat[o:o + n], np.float64).reshape(shape)
        o += n
    return p


def flatten(p):
    return np.concatenate([np.asarray(p[n], np.float64).ravel()
                           for n, _ in param_layout()])


def bf16(a):
    """Round to bfloat16 (nearest, ties to even); returns float64."""
    a32 = np.asarray(a, np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def _shift(x, dy, dx):
    """x[:, y + dy, x + dx, :] with zeros outside."""
    N, H, W, C = x.shape
    out = np.zeros_like(x)
    ys = slice(max(0, -dy), min(H, H - dy))
    xs = slice(max(0, -dx), min(W, W - dx))
    yd = slice(max(0, dy), min(H, H + dy))
    xd = slice(max(0, dx), min(W, W + dx))
    out[:, ys, xs, :] = x[:, yd, xd, :]
    return out


def conv3(x, W, b):
    """out[n, y, x, co] = b[co] + sum W[co, ky, kx, ci] x[n, y+ky-1, x+kx-1, ci]."""
    out = np.zeros(x.shape[:3] + (W.shape[0],))
    for ky in range(3):
        for kx in range(3):
            out += _shift(x, ky - 1, kx - 1) @ W[:, ky, kx, :].T
    return out + b


def conv3_backward(x, W, G):
    """Gradients of conv3 for the output gradient G: (dx, dW, db)."""
    dW = np.zeros_like(W)
    dx = np.zeros_like(x)
    for ky in range(3):
        for kx in range(3):
            xs = _shift(x, ky - 1, kx - 1)
            dW[:, ky, kx, :] = np.einsum("nyxo,nyxi->oi", G, xs)
            dx += _shift(G @ W[:, ky, kx, :], 1 - ky, 1 - kx)
    return dx, dW, G.sum(axis=(0, 1, 2))


def pool(x):
    N, H, W, C = x.shape
    return x.reshape(N, H // 2, 2, W // 2, 2, C).mean(axis=(2, 4))


def pool_backward(g):
    return np.repeat(np.repeat(g, 2, axis=1), 2, axis=2) / 4.0


def up(x):
    return np.repeat(np.repeat(x, 2, axis=1), 2, axis=2)


def up_backward(g):
    N, H, W, C = g.shape
    return g.reshape(N, H // 2, 2, W // 2, 2, C).sum(axis=(2, 4))


def forward(p, x, bf16_storage=False):
    """(y, cache): head output (N, H, W, 2) and what backward needs."""
    r = bf16 if bf16_storage else (lambda a: a)
    Wr = {n: (r(p[n]) if n.endswith(".W") and not n.startswith("head")
              else p[n]) for n in p}
    cache = {"x": r(x)}

    def cv(name, inp):
        y = r(np.maximum(conv3(inp, Wr[name + ".W"], Wr[name + ".b"]), 0.0))
        cache[name] = (inp, y)
        return y

    e0 = cv("e0b", cv("e0a", cache["x"]))
    p0 = r(pool(e0))
    e1 = cv("e1b", cv("e1a", p0))
    p1 = r(pool(e1))
    e2 = cv("e2b", cv("e2a", p1))
    p2 = r(pool(e2))
    bt = cv("bb", cv("ba", p2))
    c2 = np.concatenate([up(bt), e2], axis=-1)
    d2 = cv("d2b", cv("d2a", c2))
    c1 = np.concatenate([up(d2), e1], axis=-1)
    d1 = cv("d1b", cv("d1a", c1))
    c0 = np.concatenate([up(d1), e0], axis=-1)
    d0 = cv("d0b", cv("d0a", c0))
    y = d0 @ p["head.W"].T + p["head.b"]
    cache.update(Wr=Wr, d0=d0)
    return y, cache


def loss(y, t):
    return float(np.sum((y - t) ** 2) / (2.0 * y.size))


def backward(p, cache, y, t, bf16_storage=False):
    """Gradient of ``loss`` with respect to every parameter (dict)."""
    r = bf16 if bf16_storage else (lambda a: a)
    Wr = cache["Wr"]
    g = {}
    dy = (y - t) / y.size
    d0 = cache["d0"]
    g["head.W"] = np.einsum("nyxc,nyxi->ci", dy, d0)
    g["head.b"] = dy.sum(axis=(0, 1, 2))
    d_out = dy @ p["head.W"]                 # dL/d d0

    def cvb(name, d_out):
        inp, yv = cache[name]
        G = r(d_out * (yv > 0))
        dx, dW, db = conv3_backward(inp, Wr[name + ".W"], G)
        g[name + ".W"], g[name + ".b"] = dW, db
        return dx

    def split(dc, cb):
        return up_backward(dc[..., :cb]), dc[..., cb:]

    d_c0 = cvb("d0a", cvb("d0b", d_out))
    d_d1, d_e0 = split(d_c0, 64)
    d_c1 = cvb("d1a", cvb("d1b", d_d1))
    d_d2, d_e1 = split(d_c1, 128)
    d_c2 = cvb("d2a", cvb("d2b", d_d2))
    d_bt, d_e2 = split(d_c2, 256)
    d_p2 = cvb("ba", cvb("bb", d_bt))
    d_e2 = d_e2 + pool_backward(d_p2)
    d_p1 = cvb("e2a", cvb("e2b", d_e2))
    d_e1 = d_e1 + pool_backward(d_p1)
    d_p0 = cvb("e1a", cvb("e1b", d_e1))
    d_e0 = d_e0 + pool_backward(d_p0)
    cvb("e0a", cvb("e0b", d_e0))
    return g


def init_params(seed=0):
    """He-normal weights, zero biases (FP64)."""
    rng = np.random.default_rng(seed)
    p = {}
    for name, shape in param_layout():
        if name.endswith(".b"):
            p[name] = np.zeros(shape)
        else:
            fan_in = int(np.prod(shape[1:]))
            p[name] = rng.normal(size=shape) * np.sqrt(2.0 / fan_in)
    return p
