"""The single-precision building blocks of the fused Volterra phase against
CUDA's correctly rounded operations, through dyfox_arith_probe:

* the Newton-refined hardware reciprocal (rcp_nr) against __frcp_rn over
  normal x in [2^-100, 2^100], including the core clamp r2c >= a2 (pixel
  units) of the edge terms: within 1 ulp;
* the residual-corrected quotient (div_nr) against __fdiv_rn for
  0 <= a <= b, the folded arguments of the atan2 polynomial: within 1 ulp;
* the integer-built float-to-double widening of the FP64 segment sum
  against the hardware conversion: equal bit for bit, zeros, infinities,
  NaN and subnormals included;
* the FP64 segment sum itself (exact on the 2^-66 grid, or in double in
  order past its range) against the same sums formed exactly on the host.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _probe(torch, op, a, b=None, out_dtype=None):
    from dyfox_gb300 import _lib
    L = _lib.lib()
    f = L.dyfox_arith_probe
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    at = torch.from_numpy(np.ascontiguousarray(a, np.float32)).cuda()
    bt = (torch.from_numpy(np.ascontiguousarray(b, np.float32)).cuda()
          if b is not None else None)
    out = torch.empty(len(a), dtype=out_dtype or torch.float32,
                      device="cuda")
    _lib.check(f(op, at.data_ptr(), bt.data_ptr() if bt is not None else
                 None, out.data_ptr(), len(a),
                 torch.cuda.current_stream().cuda_stream),
               "dyfox_arith_probe")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _ulps(x, y):
    """Distance in units in the last place between float32 arrays of the
    same sign (ordered integer representations)."""
    xi = x.view(np.int32).astype(np.int64)
    yi = y.view(np.int32).astype(np.int64)
    return np.abs(xi - yi)


def test_reciprocal_within_one_ulp(gpu):
    rng = np.random.default_rng(5)
    x = np.exp2(rng.uniform(-100, 100, 1 << 20)).astype(np.float32)
    # the core clamp of the edge terms: r2c >= (a_core / dx)^2, with
    # a_core = |b| = 0.89 A and dx from 0.05 to 0.5 um
    x[:1000] = np.float32((0.8918e-10 / 0.25e-6) ** 2) * \
        (1 + rng.uniform(0, 4, 1000)).astype(np.float32)
    mine = _probe(gpu, 0, x)
    want = _probe(gpu, 1, x)
    d = _ulps(mine, want)
    assert d.max() <= 1
    assert np.mean(d == 0) > 0.9


def test_division_within_one_ulp(gpu):
    rng = np.random.default_rng(6)
    b = np.exp2(rng.uniform(-100, 100, 1 << 20)).astype(np.float32)
    a = (b * rng.uniform(0, 1, b.size)).astype(np.float32)
    a[:100] = 0.0
    a[100:200] = b[100:200]
    mine = _probe(gpu, 2, a, b)
    want = _probe(gpu, 3, a, b)
    d = _ulps(mine, want)
    assert d.max() <= 1
    assert np.mean(d == 0) > 0.9


def test_widening_is_the_hardware_conversion(gpu):
    torch = gpu
    rng = np.random.default_rng(7)
    bits = rng.integers(0, 1 << 32, 1 << 20, dtype=np.uint64).astype(
        np.uint32)
    special = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-40, -3e-45,
                        1.17549435e-38, 3.4028235e38, 1.0, -2.5],
                       dtype=np.float32)
    x = np.concatenate([special, bits.view(np.float32)])
    mine = _probe(torch, 4, x, out_dtype=torch.float64)
    want = _probe(torch, 5, x, out_dtype=torch.float64)
    nan = np.isnan(want)
    assert np.array_equal(np.isnan(mine), nan)
    assert np.array_equal(mine[~nan].view(np.uint64),
                          want[~nan].view(np.uint64))


def _probe64(torch, op, a, b=None):
    from dyfox_gb300 import _lib
    f = _lib.lib().dyfox_arith_probe64
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
    at = torch.from_numpy(np.ascontiguousarray(a, np.float64)).cuda()
    bt = (torch.from_numpy(np.ascontiguousarray(b, np.float64)).cuda()
          if b is not None else None)
    out = torch.empty(len(a), dtype=torch.float64, device="cuda")
    _lib.check(f(op, at.data_ptr(), bt.data_ptr() if bt is not None else
                 None, out.data_ptr(), len(a),
                 torch.cuda.current_stream().cuda_stream),
               "dyfox_arith_probe64")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_double_log_atan2_reciprocal_of_the_fp64_field(gpu):
    """The table-driven log and atan2 and the Newton-refined reciprocal of
    the FP64 Volterra field against CUDA's log, atan2 and __drcp_rn over
    the ranges the field meets (offsets from a line of 1e-12 to 1e-2 m,
    any quadrant, axes and signed zeros; r^2 from 1e-24 to 1 m^2):
    atan2 within 4 ulp of the result (both are about an ulp from the exact
    value), log within 3 ulp or 2e-16 absolute, the reciprocal within 1
    ulp.  (log_d itself, emulated exactly on the host, is within 1.2 ulp
    of ln x where |ln x| >= 1 and within 5e-17 absolute elsewhere: just
    below x = 1 the table term ln(1 + j/128) - ln 2 cancels; CUDA's log is
    within 1 ulp.)"""
    torch = gpu
    rng = np.random.default_rng(8)
    n = 1 << 20
    y = rng.normal(size=n) * 10.0 ** rng.uniform(-12, -2, n)
    x = rng.normal(size=n) * 10.0 ** rng.uniform(-12, -2, n)
    y[:8] = [0.0, -0.0, 0.0, -0.0, 1e-9, -1e-9, 0.0, 3e-6]
    x[:8] = [0.0, 0.0, -0.0, -0.0, 0.0, 0.0, 2e-9, -3e-6]
    mine = _probe64(torch, 0, y, x)
    want = _probe64(torch, 1, y, x)
    assert np.array_equal(np.signbit(mine), np.signbit(want))
    assert np.all(np.abs(mine - want) <= 4 * np.spacing(np.abs(want)) + 1e-300)
    r2 = 10.0 ** rng.uniform(-24, 0, n)
    r2[:4] = [1.0, 2.0, 0.5, 0.7071067811865476]
    lm = _probe64(torch, 2, r2)
    lw = _probe64(torch, 3, r2)
    assert np.all(np.abs(lm - lw) <= 3 * np.spacing(np.abs(lw)) + 2e-16)
    rm = _probe64(torch, 4, r2)
    rw = _probe64(torch, 5, r2)
    assert np.all(np.abs(rm - rw) <= np.spacing(np.abs(rw)))


def _seg_sum(torch, terms):
    from dyfox_gb300 import _lib
    f = _lib.lib().dyfox_seg_sum_probe
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p]
    n, m = terms.shape
    t = torch.from_numpy(np.ascontiguousarray(terms, np.float32)).cuda()
    out = torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.check(f(t.data_ptr(), m, out.data_ptr(), n,
                 torch.cuda.current_stream().cuda_stream),
               "dyfox_seg_sum_probe")
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _exact_grid_sum(row):
    """Each float32 term split exactly into integers on the grids 1, 2^-22,
    2^-44 and 2^-66 (each rounded to nearest, ties to even, from the
    remainder of the coarser ones; float64 holds every remainder exactly),
    the 1 and 2^-22 parts gathered in units of 2^-22, the others in units
    of 2^-66, each total converted to double and the two added."""
    hi = lo = 0
    for h in row.astype(np.float64):
        q = []
        r = h
        for k in (0, 22, 44, 66):
            qi = float(np.rint(r * 2.0 ** k))
            q.append(int(qi))
            r = r - qi * 2.0 ** -k
        hi += q[0] * 2 ** 22 + q[1]
        lo += q[2] * 2 ** 22 + q[3]
    return 0.0 + (float(hi) * 2.0 ** -22 + float(lo) * 2.0 ** -66)


def _ordered_double_sum(row):
    acc = 0.0
    for h in row.astype(np.float64):
        acc += h
    return acc


@pytest.mark.parametrize("m", [1, 7, 64, 700])
def test_exact_segment_sum(gpu, m):
    """seg_sum64 over groups of m terms of the sizes the Volterra phase
    meets (magnitudes from 1e-9 to 1e3 rad, mixed signs, cancelling pairs,
    exact ties of the grids): bit for bit the exact sum of the terms
    rounded to the 2^-66 grid, rounded to double; groups whose magnitudes
    sum to 2^17 rad or more, or with an infinity or a NaN, and single
    terms: bit for bit the in-order double sum."""
    rng = np.random.default_rng(11 + m)
    n = 512
    mag = 10.0 ** rng.uniform(-9, 3, (n, m))
    t = (rng.choice([-1.0, 1.0], (n, m)) * mag).astype(np.float32)
    cap = np.float32(2.0 ** 16 / m)                 # sum of |h| below 2^16
    t = np.clip(t, -cap, cap)
    t[1, :] = np.float32(1e-30)
    if m >= 2:
        t[2, 1] = -t[2, 0]                          # cancelling pair
        t[3, :2] = [np.float32(2.0 ** -67), np.float32(3 * 2.0 ** -67)]
        t[4, :2] = [np.float32(1 + 2.0 ** -23), np.float32(0.5)]
    over = [5, 6, 7, 8]
    t[5, 0] = np.float32(2.0 ** 17)                 # at the limit
    t[6, -1] = np.float32(-2.0 ** 19)
    t[7, 0] = np.inf
    t[8, 0] = np.nan
    got = _seg_sum(gpu, t)
    for i in range(n):
        want = (_ordered_double_sum(t[i]) if i in over or m == 1
                else _exact_grid_sum(t[i]))
        if np.isnan(want):
            assert np.isnan(got[i]), i
        else:
            assert got[i] == want, (i, got[i], want)
