"""The U-Net training and inference kernels against the NumPy oracle
(oracle/unet_oracle.py, pinned by finite differences).

Tight checks: each tensor-core product (forward, data gradient, weight
gradient of a 3x3 convolution) alone against FP64 on the same bfloat16
operands, and every layer of a full forward + backward pass against the
oracle evaluated on the GPU's own input to that layer.  Bfloat16 outputs
equal the correctly rounded FP64 value except where FP32 accumulation
lands on the other side of a rounding midpoint (<= 2e-3 of the elements,
never more than one unit in the last place); FP32 products agree to
<= 1e-5 relative L2.

Chained check: the whole network against the oracle run end to end.  An
isolated rounding flip in one layer moves that element by one bfloat16
unit, and a 14-layer ReLU network carries such perturbations forward
(measured: one flipped element of e1b grows to 2e-3 relative at the
output), so this integration check allows 2e-2 on the output and 0.15 on
the gradients.
"""

import numpy as np
import pytest

from conftest import rel_l2
from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu


def np_(t):
    return t.detach().cpu().numpy()


def _setup(rng, n=2, H=16, W=16, seed=2):
    p = U.init_params(seed=seed)
    for k in p:
        if k.endswith(".b"):
            p[k] = rng.normal(size=p[k].shape) * 0.05
    flat32 = U.flatten(p).astype(np.float32)
    p32 = U.unflatten(flat32.astype(np.float64))
    x = U.bf16(rng.normal(size=(n, H, W, U.C_IN)))
    x[..., 17:] = 0.0
    t = rng.normal(size=(n, H, W, 2)).astype(np.float32)
    return p32, flat32, x, t


@pytest.mark.parametrize("N,H,W,Cin,Cout", [(2, 16, 12, 32, 32),
                                            (1, 8, 8, 96, 64),
                                            (3, 12, 20, 64, 128)])
def test_single_conv_products(gpu, rng, N, H, W, Cin, Cout):
    from dyfox_gb300.learned import conv
    torch = gpu

    def dev_bf16(a):
        return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).cuda()
    X = U.bf16(rng.normal(size=(N, H, W, Cin)))
    G = U.bf16(rng.normal(size=(N, H, W, Cout)))
    Wt = U.bf16(rng.normal(size=(Cout, 3, 3, Cin)) * 0.1)
    b = rng.normal(size=Cout).astype(np.float32)
    # forward: one bfloat16 rounding of relu(conv + b)
    y = conv("fwd", X=dev_bf16(X), Wk=dev_bf16(Wt), bias=torch.tensor(b).cuda(),
             Cout=Cout).float().cpu().numpy()
    ref = np.maximum(U.conv3(X, Wt, b.astype(np.float64)), 0.0)
    # one unit in the last place, or FP32 accumulation error where the
    # output is within it of zero (the ReLU then clamps either way)
    assert np.all(np.abs(y - ref) <= 2.0 ** -7 * np.abs(ref) + 1e-5)
    assert np.mean(y != U.bf16(ref)) <= 2e-3
    # data and weight gradients: FP32 accumulation of exact products
    dx_ref, dw_ref, _ = U.conv3_backward(X, Wt, G)
    WtT = np.ascontiguousarray(np.transpose(Wt, (3, 1, 2, 0)))   # [ci][ky][kx][co]
    dx = conv("dgrad", G=dev_bf16(G), Wk=dev_bf16(WtT), Cin=Cin,
              Cout=Cout).cpu().numpy()
    assert rel_l2(dx, dx_ref) < 1e-5
    dw = conv("wgrad", X=dev_bf16(X), G=dev_bf16(G)).cpu().numpy()
    assert rel_l2(dw.reshape(Cout, 3, 3, Cin), dw_ref) < 1e-5


@pytest.mark.parametrize("N,H,W,Cin,Cout", [(2, 8, 128, 32, 32),
                                            (1, 6, 256, 32, 64),
                                            (2, 4, 64, 64, 128),
                                            (1, 8, 32, 128, 256),
                                            (1, 4, 32, 384, 128)])
def test_tcgen05_products_match_the_oracle_and_mma_sync(gpu, rng, N, H, W,
                                                        Cin, Cout):
    """The forward, data-gradient and weight-gradient products on the
    tcgen05 tensor cores (rows of 128 pixels or rows dividing 128; zero
    padding from the TMA bounds; N split above 128 channels; the weight
    gradient's MN-major operands and split-K partials) against FP64 on the
    same bfloat16 operands, with the tolerances of the mma.sync products,
    and against the mma.sync implicit GEMM itself.  No bounded wait
    expires."""
    from dyfox_gb300.learned import conv, tc_error
    torch = gpu
    tc_error(clear=True)

    def dev_bf16(a):
        return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).cuda()
    X = U.bf16(rng.normal(size=(N, H, W, Cin)))
    G = U.bf16(rng.normal(size=(N, H, W, Cout)))
    Wt = U.bf16(rng.normal(size=(Cout, 3, 3, Cin)) * 0.1)
    b = rng.normal(size=Cout).astype(np.float32)
    args = dict(X=dev_bf16(X), Wk=dev_bf16(Wt), bias=torch.tensor(b).cuda(),
                Cout=Cout)
    y = conv("fwd", **args).float().cpu().numpy()
    y_mma = conv("fwd", mma_sync=True, **args).float().cpu().numpy()
    ref = np.maximum(U.conv3(X, Wt, b.astype(np.float64)), 0.0)
    assert np.all(np.abs(y - ref) <= 2.0 ** -7 * np.abs(ref) + 1e-5)
    assert np.mean(y != U.bf16(ref)) <= 2e-3
    assert np.mean(y != y_mma) <= 2e-3
    dx_ref, _, _ = U.conv3_backward(X, Wt, G)
    WtT = dev_bf16(np.ascontiguousarray(np.transpose(Wt, (3, 1, 2, 0))))
    dx = conv("dgrad", G=dev_bf16(G), Wk=WtT, Cin=Cin,
              Cout=Cout).cpu().numpy()
    dx_mma = conv("dgrad", G=dev_bf16(G), Wk=WtT, Cin=Cin, Cout=Cout,
                  mma_sync=True).cpu().numpy()
    assert rel_l2(dx, dx_ref) < 1e-5
    assert rel_l2(dx, dx_mma) < 1e-5
    _, dw_ref, _ = U.conv3_backward(X, Wt, G)
    wargs = dict(X=dev_bf16(X), G=dev_bf16(G), Cin=Cin, Cout=Cout)
    dw = conv("wgrad", **wargs).cpu().numpy().reshape(Cout, 3, 3, Cin)
    dw_mma = conv("wgrad", mma_sync=True, **wargs).cpu().numpy().reshape(
        Cout, 3, 3, Cin)
    assert rel_l2(dw, dw_ref) < 1e-5
    assert rel_l2(dw, dw_mma) < 1e-5
    assert tc_error(clear=True) == 0


def _conv_in(net, i, x, n):
    if i == 0:
        return x
    if i in (2, 4, 6):
        return net.buffer("pool", i // 2 - 1, n).cpu().numpy()
    if i in (8, 10, 12):
        return net.buffer("cat", (i - 8) // 2, n).cpu().numpy()
    return net.buffer("act", i - 1, n).cpu().numpy()


def test_layerwise_against_the_oracle(gpu, rng):
    """Every layer of one forward and backward pass against the oracle
    evaluated on the GPU's own inputs to that layer (no error carried over
    from earlier layers): bfloat16 outputs within one rounding, FP32
    products within 1e-5."""
    from dyfox_gb300.learned import UNet
    torch = gpu
    n, H, W = 2, 16, 16
    p32, flat32, x, t = _setup(rng, n, H, W)
    net = UNet(batch=n, H=H, W=W)
    net.load(flat32)
    y = net.forward(torch.tensor(x, dtype=torch.float32).to(
        torch.bfloat16).cuda()).cpu().numpy()
    net.backward(torch.tensor(t).cuda())
    grads = U.unflatten(net.grads.cpu().numpy().astype(np.float64))
    names = [c[0] for c in U.CONVS]
    for i, name in enumerate(names):
        xin = _conv_in(net, i, x, n)
        Wr = U.bf16(p32[name + ".W"])
        ref = np.maximum(U.conv3(xin, Wr, p32[name + ".b"]), 0.0)
        got = net.buffer("act", i, n).cpu().numpy()
        assert np.all(np.abs(got - ref) <= 2.0 ** -7 * np.abs(ref) + 1e-5), \
            (name, float(np.abs(got - ref).max()))
        assert np.mean(got != U.bf16(ref)) <= 2e-3, name
    for l in range(3):
        src = net.buffer("act", 2 * l + 1, n).cpu().numpy()
        got = net.buffer("pool", l, n).cpu().numpy()
        assert np.array_equal(got, U.bf16(U.pool(src))), l
    for c, (lo, sk) in enumerate(((7, 5), (9, 3), (11, 1))):
        ref = np.concatenate([U.up(net.buffer("act", lo, n).cpu().numpy()),
                              net.buffer("act", sk, n).cpu().numpy()], -1)
        assert np.array_equal(net.buffer("cat", c, n).cpu().numpy(), ref), c
    d0 = net.buffer("act", 13, n).cpu().numpy()
    yref = d0 @ p32["head.W"].T + p32["head.b"]
    assert rel_l2(y, yref) < 1e-6
    dy = (y - t) / y.size
    assert rel_l2(net.buffer("dout", 13, n).cpu().numpy(),
                  dy @ p32["head.W"]) < 1e-5
    assert rel_l2(grads["head.W"], np.einsum("nyxc,nyxi->ci", dy, d0)) < 1e-5
    for i, name in enumerate(names):
        xin = _conv_in(net, i, x, n)
        act = net.buffer("act", i, n).cpu().numpy()
        G = U.bf16(net.buffer("dout", i, n).cpu().numpy() * (act > 0))
        dx, dW, db = U.conv3_backward(xin, U.bf16(p32[name + ".W"]), G)
        assert rel_l2(grads[name + ".W"], dW) < 1e-5, name
        assert rel_l2(grads[name + ".b"], db) < 1e-5, name
        if i > 0 and i not in (2, 4, 6, 8, 10, 12):
            assert rel_l2(net.buffer("dout", i - 1, n).cpu().numpy(),
                          dx) < 1e-5, name


@pytest.mark.parametrize("shape", [(2, 16, 16), (3, 32, 24)])
def test_forward_and_gradients_match_the_oracle(gpu, rng, shape):
    from dyfox_gb300.learned import UNet
    torch = gpu
    n, H, W = shape
    p32, flat32, x, t = _setup(rng, n, H, W)
    net = UNet(batch=4, H=H, W=W)
    assert net.n_params == U.n_params()
    net.load(flat32)
    xt = torch.tensor(x, dtype=torch.float32).to(torch.bfloat16).cuda()
    y = net.forward(xt)
    loss = net.backward(torch.tensor(t).cuda())
    yo, cache = U.forward(p32, x, bf16_storage=True)
    go = U.backward(p32, cache, yo, t.astype(np.float64), bf16_storage=True)
    assert rel_l2(y.cpu().numpy(), yo) < 2e-2
    assert float(loss) == pytest.approx(U.loss(yo, t), rel=2e-2)
    gg = U.unflatten(net.grads.cpu().numpy().astype(np.float64))
    for name, _ in U.param_layout():
        assert rel_l2(gg[name], go[name]) < 0.15, name


def test_adam_step_matches_numpy(gpu, rng):
    from dyfox_gb300.learned import UNet
    torch = gpu
    p32, flat32, x, t = _setup(rng)
    net = UNet(batch=2, H=16, W=16)
    net.load(flat32)
    net.forward(torch.tensor(x, dtype=torch.float32).to(torch.bfloat16).cuda())
    net.backward(torch.tensor(t).cuda())
    g = net.grads.cpu().numpy().astype(np.float64)
    net.step(lr=1e-3)
    m = 0.1 * g
    v = 0.001 * g * g
    want = flat32 - 1e-3 * (m / 0.1) / (np.sqrt(v / 0.001) + 1e-8)
    got = net.params.cpu().numpy()
    assert np.allclose(got, want, rtol=1e-5, atol=1e-7)


def test_training_reduces_the_loss(gpu, rng):
    """A learnable map (target = functions of the input channels): the
    loss falls by 5x within a few hundred Adam steps."""
    from dyfox_gb300.learned import UNet
    torch = gpu
    n, H, W = 16, 32, 32
    x = U.bf16(rng.normal(size=(n, H, W, U.C_IN)) * 0.5)
    x[..., 17:] = 0.0
    t = np.stack([x[..., 0] - 0.5 * x[..., 3],
                  np.tanh(x[..., 16]) * x[..., 1]], axis=-1)
    X = torch.tensor(x, dtype=torch.float32).to(torch.bfloat16).cuda()
    T = torch.tensor(t, dtype=torch.float32).cuda()
    net = UNet(batch=4, H=H, W=W, seed=5)
    hist = net.train(X, T, epochs=60, lr=2e-3)
    assert hist[-1] < 0.2 * hist[0]
    assert np.all(np.isfinite(hist))


def test_features(gpu, rng):
    from dyfox_gb300.learned import features
    torch = gpu
    h = rng.normal(size=(5, 8, 40)) * 4
    s = np.array([0.3, -1.2])
    got = features(torch.tensor(h).cuda(), 6, 24, s).float().cpu().numpy()
    assert got.shape == (2, 5, 24, 32)
    win = h[:, :, 6:30]
    for k in range(8):
        assert np.array_equal(got[..., 2 * k],
                              np.broadcast_to(U.bf16(np.cos(win[:, k])),
                                              (2, 5, 24)))
        assert np.array_equal(got[..., 2 * k + 1],
                              np.broadcast_to(U.bf16(np.sin(win[:, k])),
                                              (2, 5, 24)))
    assert np.array_equal(got[0, ..., 16], np.full((5, 24), U.bf16(0.3)))
    assert np.all(got[..., 17:] == 0)
    # columns wrap around the periodic lateral grid
    wrap = features(torch.tensor(h).cuda(), 30, 24, s).float().cpu().numpy()
    cols = np.arange(30, 54) % 40
    assert np.array_equal(wrap[0, ..., 0], U.bf16(np.cos(h[:, 0, cols])))


def test_bad_shapes(gpu):
    from dyfox_gb300.learned import UNet
    torch = gpu
    with pytest.raises(ValueError):
        UNet(batch=1, H=20, W=16)
    net = UNet(batch=1, H=16, W=16)
    with pytest.raises(ValueError):
        net.forward(torch.zeros((2, 16, 16, 32), dtype=torch.bfloat16,
                                device="cuda"))


def test_learned_guess_lowers_the_initial_residual(gpu):
    """End to end on a small configuration (64 planes x 64 px field, 64
    deviation parameters, t 10-14 um): train on the plain solves of 8
    instances (3 lateral windows each), then on a held-out instance the
    network's full-width guess lowers the initial shooting residual
    |A x0 + d| / |d| below the zero start's 1, and the solve from it still
    meets its tolerance."""
    from dyfox_gb300 import learned as Lm
    from dyfox_gb300.bragg import apply_operator
    from dyfox_gb300.workloads import learned_guess_instances
    torch = gpu
    inst = learned_guess_instances(9, seed=11, t_range=(10e-6, 14e-6),
                                   n_planes=64, field=64, n_s=64)
    Xs, Ts = [], []
    for w in inst[:8]:
        h = Lm.instance_h(w)
        v, info, _ = Lm.solve_instance(w, tol=1e-6)
        Nx = w["cfg"].Nx
        for c0 in (w["col0"], (w["col0"] + Nx // 3) % Nx,
                   (w["col0"] + 2 * Nx // 3) % Nx):
            X, h0, v0 = Lm.instance_inputs(w, col0=c0, h=h)
            Xs.append(X)
            Ts.append(Lm.targets(v, h0, v0, c0, w["field"]))
    X, T = torch.cat(Xs), torch.cat(Ts)
    # A training run from one initialisation can stall on this small set
    # (the loss flat over 12 epochs); a second initialisation is tried
    # before the test requires the loss to fall.
    for seed in (2, 5):
        net = Lm.UNet(batch=8, H=64, W=64, seed=seed)
        hist = net.train(X, T, epochs=12, lr=1e-3, decay_every=4)
        if hist[-1] < 0.7 * hist[0]:
            break
    assert hist[-1] < 0.7 * hist[0], hist
    w = inst[8]
    h = Lm.instance_h(w)
    _, h0, v0 = Lm.instance_inputs(w, h=h)
    x0 = Lm.initial_guess(w, v0, Lm.predict_full(net, w, h=h), col0=0)
    inc = torch.ones((len(w["s"]), len(w["ys"]), w["cfg"].Nx),
                     dtype=torch.complex128, device="cuda")
    d = apply_operator(w["segs"], w["s"], w["cfg"], w["ys"], w["xtal"],
                       w["g"], "march", in0=inc)
    Ax = apply_operator(w["segs"], w["s"], w["cfg"], w["ys"], w["xtal"],
                        w["g"], "march", in1=x0)
    r0 = float(torch.linalg.vector_norm(Ax + d) / torch.linalg.vector_norm(d))
    assert r0 < 0.95
    _, info, _ = Lm.solve_instance(w, x0=x0, tol=1e-8)
    info = np_(info) if hasattr(info, "cpu") else info
    assert info[:, 0].max() < 1e-8 and np.all(info[:, 2] == 0)


def test_a_guess_pays_only_at_percent_level_accuracy(gpu):
    """How accurate a starting vector must be to save GMRES work.  On one
    instance (t 10-14 um, 16 planes, 8 deviation parameters), the solve
    from the exact answer perturbed by smooth relative noise eps (harmonics
    1-8 across the width, the kind of error a network makes) needs at most
    0.85 of the zero start's inner iterations at eps = 1e-2 and at most
    0.65 at eps = 1e-4, while eps = 0.5 (the accuracy the trained network
    reaches: r0 0.43-0.47) saves at most a few iterations.  Over 15-60 um
    the same measurement gave 0.64-0.82 at 1e-2 and 0.45-0.67 at 1e-4."""
    from dyfox_gb300 import learned as Lm
    from dyfox_gb300.workloads import learned_guess_instances
    torch = gpu
    rng = np.random.default_rng(5)
    w = learned_guess_instances(1, seed=103, t_range=(10e-6, 14e-6),
                                n_planes=16, field=64, n_s=8)[0]
    v, info, _ = Lm.solve_instance(w, tol=1e-8)
    its0 = float(np_(info)[:, 1].mean())
    h0 = Lm.instance_h(w)[:, 0, :]
    xs = (v * torch.exp(1j * h0)[None]).contiguous()
    Nx = w["cfg"].Nx
    xg = np.arange(Nx)
    noise = np.zeros((len(w["s"]), len(w["ys"]), Nx), complex)
    for k in range(1, 9):
        a = rng.normal(size=noise.shape[:2]) + \
            1j * rng.normal(size=noise.shape[:2])
        ph = rng.uniform(0, 2 * np.pi, size=noise.shape[:2])
        noise += (a[..., None] / k) * np.exp(
            1j * (2 * np.pi * k * xg[None, None] / Nx + ph[..., None]))
    nt = torch.from_numpy(noise).cuda()
    nt = nt * (torch.linalg.vector_norm(xs, dim=-1, keepdim=True) /
               torch.linalg.vector_norm(nt, dim=-1, keepdim=True))
    its = {}
    for eps in (0.5, 1e-2, 1e-4):
        _, inf, _ = Lm.solve_instance(w, x0=(xs + eps * nt).contiguous(),
                                      tol=1e-8)
        inf = np_(inf)
        assert inf[:, 0].max() < 1e-8 and np.all(inf[:, 2] == 0)
        its[eps] = float(inf[:, 1].mean())
    assert its[1e-2] <= 0.85 * its0, (its, its0)
    assert its[1e-4] <= 0.65 * its0, (its, its0)
    assert its[0.5] >= 0.7 * its0, (its, its0)
