"""Dislocation segments and their displacement phase H = 2 pi g.u.

Segments are ``[(r_start, r_end, b), ...]`` in lab-frame metres, as in DYFOX
``dislocations.py:1-11``.  The host helpers (``burgers_vector``,
``straight_segment``, ``volterra_frame``, ``analytic_line_params``, ...) keep
the reference's names and results.  The volume evaluators run on the GPU
through the C ABI:

    compute_H_grid   (Ny, Nz, Nx) over a Laue grid  (dislocations.py:113-168)
    H_plane          one (Nz, Nx) plane at y         (dislocations.py:171-211)
    H_rows           (n, Nz, Nx) planes at several y (device result)

In FP64 every product and sum of the Volterra expression is rounded as the
reference's element-wise GPU arithmetic rounds it, so the grid reproduces the
reference's values; segments are summed in list order from zero.
"""

import numpy as np

from . import _lib
from .backend import FP64, precision as as_precision


def rotate_about_z(v, deg):
    if not deg:
        return v
    c, s = np.cos(np.radians(deg)), np.sin(np.radians(deg))
    return np.array([c * v[0] - s * v[1], s * v[0] + c * v[1], v[2]])


def line_direction(U_lab, line_cryst, tilt_deg=0.0):
    xi = U_lab @ np.asarray(line_cryst, float)
    return rotate_about_z(xi / np.linalg.norm(xi), tilt_deg)


def burgers_vector(U_lab, b_cryst, b_mag, sign=+1):
    b_hat = U_lab @ np.asarray(b_cryst, float)
    return sign * b_mag * b_hat / np.linalg.norm(b_hat)


def g_dot_b(g_vec, b):
    """g.b, the topological charge of the exit-wave vortex."""
    return float(np.dot(np.asarray(g_vec, float), np.asarray(b, float)))


def beam_column_center(z0, y0, tan_tB):
    return np.array([-z0 * tan_tB, y0, z0])


def straight_segment(xi, b, center, half_length):
    """One segment from ``center - half_length xi`` to ``center +
    half_length xi``, as the one-element list the solvers take."""
    xi = np.asarray(xi, float)
    center = np.asarray(center, float)
    return [(center - half_length * xi, center + half_length * xi,
             np.asarray(b, float))]


def volterra_frame(xi, bv):
    """(b_screw, b_perp, e1, e2): screw component, edge magnitude, unit edge
    direction (for pure screw the lab axis furthest from the line) and
    e2 = xi x e1 (dislocations.py:68-90)."""
    xi = np.asarray(xi, float)
    bv = np.asarray(bv, float)
    b_screw = float(np.dot(bv, xi))
    bp = bv - b_screw * xi
    b_perp = np.linalg.norm(bp)
    if b_perp > 1e-20:
        e1 = bp / b_perp
    elif abs(xi[2]) > 0.9:
        e1 = np.array([1.0, 0.0, 0.0])
    else:
        axis = [1, 0, 0] if abs(xi[0]) < 0.9 else [0, 1, 0]
        e1 = np.cross(xi, axis)
        e1 = e1 / np.linalg.norm(e1)
    return b_screw, b_perp, e1, np.cross(xi, e1)


def analytic_line_params(seg_list, xtal):
    """Closed-form march arguments for a single line along x_lab whose frame
    has no x component, else None (dislocations.py:214-242)."""
    if len(seg_list) != 1:
        return None
    ra, rb, bv = (np.asarray(v, float) for v in seg_list[0])
    t = rb - ra
    L = np.linalg.norm(t)
    if L < 1e-20:
        return None
    xi = t / L
    if abs(abs(xi[0]) - 1.0) > 1e-9:
        return None
    core = (ra + rb) / 2.0
    g = np.asarray(xtal.g_vec, float)
    b_screw, b_perp, e1, e2 = volterra_frame(xi, bv)
    if abs(e1[0]) > 1e-9 or abs(e2[0]) > 1e-9:
        return None
    return dict(y0=core[1], z0=core[2], e1y=e1[1], e1z=e1[2], e2y=e2[1],
                e2z=e2[2], C_atan=np.dot(g, e1) * b_perp
                + np.dot(g, xi) * b_screw,
                ge1=np.dot(g, e1), ge2=np.dot(g, e2), b_perp=b_perp,
                nu=xtal.nu, a2=xtal.a_core ** 2)


def analytic_vector(ap):
    """The 12 closed-form scalars in the C ABI's order."""
    return [float(ap[k]) for k in ("y0", "z0", "e1y", "e1z", "e2y", "e2z",
                                   "C_atan", "ge1", "ge2", "b_perp", "nu",
                                   "a2")]


def compute_H_grid(seg_list, grid, xtal, precision=FP64, chunk_y=32):
    """H over the (Ny, Nz, Nx) volume of a Laue grid, on the GPU.

    ``chunk_y`` is accepted for signature compatibility; the kernel has no
    chunking, so the result is independent of it.  FP32 rounds each
    segment's double value before a single-precision sum (as the reference).
    """
    torch = _lib.torch_cuda()
    prec = as_precision(precision)
    Nx, Ny, dz, _, _ = grid.geometry()
    Nz = int(grid.Nz)
    need = Ny * Nz * Nx * prec.itemsize
    free = torch.cuda.mem_get_info()[0]
    if need > 0.9 * free:
        raise MemoryError(f"H grid needs {need / 1e9:.1f} GB, "
                          f"{free / 1e9:.1f} GB free")
    table = _lib.segment_table(seg_list, xtal.g_vec, xtal.nu, xtal.a_core,
                               grid.dx)
    dt = _lib.device_table(table)
    out = torch.empty((Ny, Nz, Nx), dtype=prec.torch_real, device="cuda")
    _lib.check(_lib.lib().dyfox_h_grid(
        _lib.ptr(dt), len(table), int(Nx), int(Ny), Nz, float(grid.dx),
        float(dz), float(xtal.nu), float(xtal.a_core), prec.code,
        _lib.ptr(out), _lib.stream_ptr()), "dyfox_h_grid")
    return out


def H_rows(seg_list, Nx, Nz, dx, dz, g_vec, nu, a_core, y_values):
    """H (FP64) on planes of constant y: a (len(y), Nz, Nx) CUDA tensor."""
    torch = _lib.torch_cuda()
    y = torch.as_tensor(np.atleast_1d(np.asarray(y_values, float)),
                        dtype=torch.float64).to("cuda")
    out = torch.empty((len(y), int(Nz), int(Nx)), dtype=torch.float64,
                      device="cuda")
    table = _lib.segment_table(seg_list, g_vec, nu, a_core, dx)
    dt = _lib.device_table(table)
    _lib.check(_lib.lib().dyfox_h_rows(
        _lib.ptr(dt), len(table), int(Nx), int(Nz), float(dx), float(dz),
        float(nu), float(a_core), _lib.ptr(y), len(y), _lib.ptr(out),
        _lib.stream_ptr()), "dyfox_h_rows")
    return out


def H_plane(seg_list, cfg, g_vec, nu, a_core, xp=np, y_plane=0.0):
    """H on the (Nz, Nx) plane at ``y_plane`` of a grid with ``Nx``, ``Nz``,
    ``dx``, ``dz`` attributes.  NumPy result when ``xp`` is NumPy, else a
    CUDA tensor."""
    h = H_rows(seg_list, cfg.Nx, cfg.Nz, cfg.dx, cfg.dz, g_vec, nu, a_core,
               [y_plane])[0]
    return h.cpu().numpy() if xp is np else h
