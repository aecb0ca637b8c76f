"""ORACLE -- test infrastructure only.  NumPy restatement of DYFOX's Bragg
shooting solve, pinned by tests/test_oracle_pins.py against the golden
vectors of tests/golden/bragg_small.npz (made from the reference):

    march_down        bragg/solver.py:28-35
    perfect_symbol    bragg/solver.py:38-60
    precondition      bragg/solver.py:164-168 (T22 floored at 1e-8 max|T22|)
    couplings         bragg/solver.py:256-261 (H from the C oracle)
    solve_plane       solve_bragg_stable's algorithm (135-179): SciPy GMRES
                      (scipy.sparse.linalg.gmres, left preconditioned)
    dense_solve       the same shooting system solved directly (Nx matvecs
                      build A; numpy.linalg.solve) -- free of GMRES tolerance
"""

import numpy as np

from oracle import oracle as O


def march_down(D0, Dg, Ch, Cb, e0, eg, ds, Nz):
    for k in range(Nz - 1):
        D0n = e0 * np.roll(D0 + ds * Cb[k] * Dg, 1, axis=-1)
        Dgn = np.roll((Dg - ds * Ch[k] * D0) / eg, -1, axis=-1)
        D0, Dg = D0n, Dgn
    return Dg


def step_factors(xtal, s_dev, ds):
    s0 = complex(xtal.sig0)
    alpha = -2.0 * np.pi * float(s_dev)
    return complex(np.exp(s0 * ds)), complex(np.exp((s0 + 1j * alpha) * ds))


def perfect_symbol(e0, eg, ds, Nz, Nx, xtal):
    sh, sb = complex(xtal.sig_h), complex(xtal.sig_hbar)
    m = np.fft.fftfreq(Nx) * Nx
    p = np.exp(-2j * np.pi * m / Nx)
    pi = np.conj(p)
    T11 = np.ones(Nx, complex)
    T12 = np.zeros(Nx, complex)
    T21 = np.zeros(Nx, complex)
    T22 = np.ones(Nx, complex)
    for _ in range(Nz - 1):
        a11 = e0 * p
        a12 = e0 * p * ds * sb
        a21 = -pi * ds * sh / eg
        a22 = pi / eg
        T11, T12, T21, T22 = (a11 * T11 + a12 * T21, a11 * T12 + a12 * T22,
                              a21 * T11 + a22 * T21, a21 * T12 + a22 * T22)
    return T21, T22


def floored(T22):
    floor = 1e-8 * np.abs(T22).max()
    return np.where(np.abs(T22) < floor, floor, T22)


def precondition(w, T22s):
    return np.fft.ifft(np.fft.fft(w, axis=-1) / T22s, axis=-1)


def plane_H(seg_list, cfg, g_vec, xtal, y):
    if not seg_list:
        return np.zeros((cfg.Nz, cfg.Nx))
    return O.h_rows(seg_list, g_vec, xtal.nu, xtal.a_core, cfg.Nx, cfg.Nz,
                    cfg.dx, cfg.dz, [y])[0]


def couplings(H, xtal):
    Ch = (complex(xtal.sig_h) * np.exp(-1j * H)).astype(np.complex128)
    Cb = (complex(xtal.sig_hbar) * np.exp(+1j * H)).astype(np.complex128)
    return Ch, Cb


def system(seg_list, s_dev, cfg, xtal, g_vec, y=0.0):
    """(matvec, d, H, T22s) of one plane's shooting system."""
    H = plane_H(seg_list, cfg, g_vec, xtal, y)
    Ch, Cb = couplings(H, xtal)
    e0, eg = step_factors(xtal, s_dev, cfg.ds)
    zero = np.zeros(cfg.Nx, complex)
    d = march_down(cfg.incident(n=1)[0], zero, Ch, Cb, e0, eg, cfg.ds,
                   cfg.Nz)

    def matvec(v):
        return march_down(zero, np.asarray(v, complex), Ch, Cb, e0, eg,
                          cfg.ds, cfg.Nz)
    _, T22 = perfect_symbol(e0, eg, cfg.ds, cfg.Nz, cfg.Nx, xtal)
    return matvec, d, H, floored(T22)


def solve_plane(seg_list, s_dev, cfg, xtal, g_vec, y=0.0, tol=1e-10,
                restart=40, maxiter=20):
    """SciPy GMRES on A v = -d with the perfect-crystal preconditioner;
    returns (exit wave v e^{-iH(0)}, v, true relative residual, code)."""
    from scipy.sparse.linalg import LinearOperator, gmres
    matvec, d, H, T22s = system(seg_list, s_dev, cfg, xtal, g_vec, y)
    N = cfg.Nx
    A = LinearOperator((N, N), matvec=matvec, dtype=np.complex128)
    M = LinearOperator((N, N), matvec=lambda w: precondition(w, T22s),
                       dtype=np.complex128)
    v, code = gmres(A, -d, M=M, rtol=tol, restart=restart, maxiter=maxiter)
    res = np.linalg.norm(matvec(v) + d) / np.linalg.norm(d)
    return v * np.exp(-1j * H[0]), v, float(res), code


def dense_solve(seg_list, s_dev, cfg, xtal, g_vec, y=0.0):
    """Direct solve of the shooting system: exit wave and v.  The columns
    A e_j are marched together (row j of one (Nx, Nx) march)."""
    matvec, d, H, _ = system(seg_list, s_dev, cfg, xtal, g_vec, y)
    N = cfg.Nx
    A = matvec(np.eye(N, dtype=complex)).T
    v = np.linalg.solve(A, -d)
    return v * np.exp(-1j * H[0]), v


def solve_surface(seg_list, s_dev, cfg, y_values, xtal, g_vec, chunk=32,
                  tol=1e-10, restart=40, maxiter=25, accept=1e-7, grow=4,
                  tries=3, restart_cap=256, max_depth=6, per_plane=6,
                  chunk_cap=32):
    """The CPU branch of solve_surface_batch (bragg/solver.py:182-379): the
    planes of a chunk share one SciPy GMRES; true-residual retries with a
    larger Krylov space, then splitting.  Returns (out, info)."""
    from scipy.sparse.linalg import LinearOperator, gmres
    e0, eg = step_factors(xtal, s_dev, cfg.ds)
    _, T22 = perfect_symbol(e0, eg, cfg.ds, cfg.Nz, cfg.Nx, xtal)
    T22s = floored(T22)
    ny = len(y_values)
    out = np.zeros((ny, cfg.Nx), dtype=np.complex128)
    st = dict(worst=0.0, its=0, retries=0, splits=0, unconverged=0)
    chunk = max(1, min(chunk, chunk_cap))

    def block(j0, j1, depth=0):
        nyc = j1 - j0
        H = np.stack([plane_H(seg_list, cfg, g_vec, xtal, float(y))
                      for y in y_values[j0:j1]], axis=1)
        Ch, Cb = couplings(H, xtal)
        zero = np.zeros((nyc, cfg.Nx), complex)
        d = march_down(cfg.incident(n=nyc), zero, Ch, Cb, e0, eg, cfg.ds,
                       cfg.Nz).ravel()

        def mv(v):
            return march_down(zero, v.reshape(nyc, cfg.Nx), Ch, Cb, e0, eg,
                              cfg.ds, cfg.Nz).ravel()

        def pc(w):
            return precondition(w.reshape(nyc, cfg.Nx), T22s[None]).ravel()
        N = nyc * cfg.Nx
        A = LinearOperator((N, N), matvec=mv, dtype=np.complex128)
        M = LinearOperator((N, N), matvec=pc, dtype=np.complex128)
        cap = max(restart, min(restart_cap, 8 * nyc))
        r = max(restart, min(cap, per_plane * nyc))
        cnt = [0]
        nb = np.linalg.norm(d) + 1e-300
        v, x0 = None, None
        for _ in range(tries):
            v, _ = gmres(A, -d, x0=x0, M=M, rtol=tol, restart=r,
                         maxiter=maxiter,
                         callback=lambda _: cnt.__setitem__(0, cnt[0] + 1),
                         callback_type="pr_norm")
            res = float(np.linalg.norm(mv(v) + d) / nb)
            if res <= accept or r >= cap:
                break
            st["retries"] += 1
            x0, r = v, min(r * grow, cap)
        if res > accept and nyc > 1 and depth < max_depth:
            st["splits"] += 1
            mid = j0 + nyc // 2
            block(j0, mid, depth + 1)
            block(mid, j1, depth + 1)
            return
        st["unconverged"] += res > accept
        st["worst"] = max(st["worst"], res)
        st["its"] = max(st["its"], cnt[0])
        out[j0:j1] = v.reshape(nyc, cfg.Nx) * np.exp(-1j * H[0])

    for j0 in range(0, ny, chunk):
        block(j0, min(j0 + chunk, ny))
    return out, {"residual": st["worst"], "iterations": st["its"],
                 "retries": st["retries"], "splits": st["splits"],
                 "unconverged_chunks": st["unconverged"],
                 "converged": st["unconverged"] == 0}
