"""ORACLE -- test infrastructure only (tests/, __graft_entry__.smoke() and the
CPU legs of bench.py use it as the checker; the product never imports it).

ctypes front-end of the C restatement ``oracle/dyfox_oracle.c`` and of the
reference kernels compiled from the DYFOX sources into ``oracle/_ref`` by
``oracle/make_ref.py``.  ``build()`` compiles both with gcc/g++ (no CUDA).

Parity is pinned: ``tests/test_oracle_pins.py`` checks this module against
the golden vectors of ``tests/golden`` (generated from the reference by
``tests/golden/make_golden.py``) and against ``oracle/_ref``.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.path.join(HERE, "_ref")
LIB = os.path.join(HERE, "liboracle.so")
REF_CPU = os.path.join(REF, "libref_cpu.so")
OSEG = 16

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def build(force=False):
    """Compile the oracle (and the reference CPU harness when its generated
    source is present).  Same flags on x86 and aarch64."""
    flags = ["-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared"]
    src = os.path.join(HERE, "dyfox_oracle.c")
    if force or not _fresh(LIB, [src]):
        subprocess.check_call(["gcc", *flags, "-o", LIB, src, "-lm"])
    ref_src = os.path.join(REF, "ref_cpu.cpp")
    if os.path.exists(ref_src):
        deps = [ref_src, os.path.join(REF, "ref_kernels.inc"),
                os.path.join(HERE, "ref_cpu_shim.h"),
                os.path.join(HERE, "ref_launch_cpu.inc")]
        if force or not _fresh(REF_CPU, deps):
            subprocess.check_call(["g++", *flags, "-w", "-o", REF_CPU,
                                   ref_src])


def _fresh(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps if os.path.exists(d))


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _lib.oracle_num_threads.restype = ctypes.c_int
    return _lib


def ref_cpu():
    """The reference kernels compiled for the CPU, or None if not built."""
    global _ref
    if _ref is None and os.path.exists(os.path.join(REF, "ref_cpu.cpp")):
        build()
        _ref = ctypes.CDLL(REF_CPU)
    return _ref


def _d(a):
    return a.ctypes.data_as(_dp)


def num_threads():
    return lib().oracle_num_threads()


# ------------------------------------------------------------------ Volterra
def segment_array(seg_list):
    """Segments as an (n, 9) float64 array of (r_start, r_end, b)."""
    if len(seg_list) == 0:
        return np.zeros((0, 9))
    return np.array([np.concatenate([np.asarray(v, float).ravel()
                                     for v in s]) for s in seg_list],
                    dtype=np.float64).reshape(-1, 9)


def segment_frames(seg_list, g_vec):
    segs = np.ascontiguousarray(segment_array(seg_list))
    out = np.zeros((max(len(segs), 1), OSEG))
    g = np.ascontiguousarray(np.asarray(g_vec, float))
    n = lib().oracle_segment_frames(_d(segs), ctypes.c_int(len(segs)), _d(g),
                                    _d(out))
    return out[:n]


def h_rows(seg_list, g_vec, nu, a_core, Nx, Nz, dx, dz, y_values,
           cast_fp32=False):
    """H (len(y), Nz, Nx) in FP64 at the given y (dislocations.py:113-211)."""
    fr = np.ascontiguousarray(segment_frames(seg_list, g_vec))
    y = np.ascontiguousarray(np.atleast_1d(np.asarray(y_values, float)))
    out = np.zeros((len(y), Nz, Nx))
    lib().oracle_h_rows(_d(fr), ctypes.c_int(len(fr)), ctypes.c_double(nu),
                        ctypes.c_double(a_core), ctypes.c_int(Nx),
                        ctypes.c_int(Nz), ctypes.c_double(dx),
                        ctypes.c_double(dz), _d(y), ctypes.c_int(len(y)),
                        ctypes.c_int(int(bool(cast_fp32))), _d(out))
    return out


def grid_y(Ny, dx, rows=None):
    """y of grid rows as compute_H_grid samples them: (iy - Ny/2) dx."""
    iy = np.arange(Ny) if rows is None else np.asarray(rows)
    return (iy - Ny / 2) * dx


# ---------------------------------------------------------------- Laue march
def _xtal6(xtal):
    return [float(v) for v in (xtal.sig0.real, xtal.sig0.imag,
                               xtal.sig_h.real, xtal.sig_h.imag,
                               xtal.sig_hbar.real, xtal.sig_hbar.imag)]


def laue_march(mode, xtal, s_dev, geo, H_rows=None, an=None, rows=None):
    """Exit waves (n_e, len(rows), Nx) complex128 of the reference march.

    mode: "pristine", "fullfield" (H_rows indexed like rows), "analytic".
    geo: dict with Nx, Ny, Nz, dz, ds, shift_px, dx, sheet_hw, fov_hy.
    """
    m = {"pristine": 0, "fullfield": 1, "analytic": 2}[mode]
    s = np.ascontiguousarray(np.atleast_1d(np.asarray(s_dev, float)))
    Nx, Ny, Nz = geo["Nx"], geo["Ny"], geo["Nz"]
    rws = np.arange(Ny, dtype=np.int32) if rows is None else \
        np.ascontiguousarray(np.asarray(rows, dtype=np.int32))
    out = np.zeros((len(s), len(rws), Nx), dtype=np.complex128)
    Hp = None
    if m == 1:
        H = np.ascontiguousarray(np.asarray(H_rows, dtype=np.float64))
        assert H.shape == (len(rws), Nz, Nx)
        Hp = _d(H)
    anp = None
    if m == 2:
        A = np.ascontiguousarray(np.asarray(an, float))
        anp = _d(A)
    c = ctypes.c_double
    lib().oracle_laue_march(
        ctypes.c_int(m), *[c(v) for v in _xtal6(xtal)], _d(s),
        ctypes.c_int(len(s)), c(geo["dz"]), c(geo["shift_px"]), c(geo["ds"]),
        c(geo["dx"]), ctypes.c_int(Nz), ctypes.c_int(Nx), ctypes.c_int(Ny),
        c(geo["sheet_hw"]), c(geo["fov_hy"]), Hp, anp,
        rws.ctypes.data_as(_ip), ctypes.c_int(len(rws)),
        out.ctypes.data_as(_dp))
    return out


def analytic_vector(ap):
    """The 12 closed-form scalars in tt3d_analytic_batch's argument order."""
    return np.array([ap[k] for k in ("y0", "z0", "e1y", "e1z", "e2y", "e2z",
                                     "C_atan", "ge1", "ge2", "b_perp", "nu",
                                     "a2")], dtype=np.float64)


def ref_laue_march(mode, xtal, s_dev, geo, H_grid=None, an=None, rows=None,
                   fp32=False):
    """The DYFOX reference kernel itself, run on the CPU (oracle/_ref).

    H_grid is the (Ny, Nz, Nx) grid the reference kernel indexes; it may
    stop after the last row computed, since no other row is read.
    Returns (n_e, len(rows), Nx) complex, or None when _ref is absent.
    """
    r = ref_cpu()
    if r is None:
        return None
    T = np.float32 if fp32 else np.float64
    ct = ctypes.c_float if fp32 else ctypes.c_double
    pt = ctypes.POINTER(ct)
    sfx = "_f32" if fp32 else "_f64"
    s = np.ascontiguousarray(np.atleast_1d(np.asarray(s_dev)).astype(T))
    n_e = len(s)
    Nx, Ny, Nz = geo["Nx"], geo["Ny"], geo["Nz"]
    rws = np.arange(Ny) if rows is None else np.asarray(rows)
    blocks = np.ascontiguousarray(
        (rws[None, :] * n_e + np.arange(n_e)[:, None]).ravel().astype(
            np.int32))
    re = np.zeros(n_e * Ny * Nx, dtype=T)
    im = np.zeros(n_e * Ny * Nx, dtype=T)
    common = [re.ctypes.data_as(pt), im.ctypes.data_as(pt),
              *[ct(v) for v in _xtal6(xtal)], s.ctypes.data_as(pt),
              ctypes.c_int(n_e), ct(geo["dz"]), ct(geo["shift_px"]),
              ct(geo["ds"]), ct(geo["dx"]), ctypes.c_int(Nz),
              ctypes.c_int(Nx), ctypes.c_int(Ny), ct(geo["sheet_hw"]),
              ct(geo["fov_hy"])]
    tail = [blocks.ctypes.data_as(_ip), ctypes.c_int(len(blocks))]
    if mode == "fullfield":
        H = np.ascontiguousarray(np.asarray(H_grid).astype(T))
        assert H.shape[1:] == (Nz, Nx) and H.shape[0] > int(np.max(rws))
        getattr(r, "ref_cpu_fullfield" + sfx)(*common, H.ctypes.data_as(pt),
                                              *tail)
    elif mode == "pristine":
        getattr(r, "ref_cpu_pristine" + sfx)(*common, *tail)
    else:
        A = np.ascontiguousarray(np.asarray(an).astype(T))
        getattr(r, "ref_cpu_analytic" + sfx)(*common, A.ctypes.data_as(pt),
                                             *tail)
    # The kernel's blocks are (iy, ie) with out offset ie*Ny*Nx + iy*Nx.
    out = (re + 1j * im).reshape(n_e, Ny, Nx)
    return out[:, rws, :]


# ------------------------------------------------ reference kernel, on GPU
REF_GPU = os.path.join(REF, "libref_gpu.so")
_ref_gpu = None


def build_ref_gpu(force=False):
    """Compile oracle/_ref/ref_gpu.cu (the reference kernel text plus
    ref_launch_gpu.cuh) with nvcc when its generated source is present."""
    src = os.path.join(REF, "ref_gpu.cu")
    if not os.path.exists(src):
        return None
    deps = [src, os.path.join(REF, "ref_kernels.inc"),
            os.path.join(HERE, "ref_launch_gpu.cuh")]
    if force or not _fresh(REF_GPU, deps):
        import shutil
        nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
        subprocess.check_call([nvcc, "-gencode",
                               "arch=compute_103a,code=sm_103a", "-O3",
                               "-shared", "-Xcompiler", "-fPIC", "-w",
                               "-o", REF_GPU, src])
    return REF_GPU


def ref_gpu():
    """The reference kernels compiled for the GPU, or None if not built."""
    global _ref_gpu
    if _ref_gpu is None and os.path.exists(REF_GPU):
        _ref_gpu = ctypes.CDLL(REF_GPU)
    return _ref_gpu


def ref_gpu_laue_march(mode, xtal, s_dev, geo, H_grid=None, an=None,
                       fp32=False):
    """Run the DYFOX reference kernel on the GPU with solver.py's launch
    (grid Ny * n_e, block 256).  H_grid: a torch CUDA (Ny, Nz, Nx) tensor.
    Returns the (n_e, Ny, Nx) exit waves as a torch complex tensor."""
    import torch
    r = ref_gpu()
    if r is None:
        return None
    T = torch.float32 if fp32 else torch.float64
    ct = ctypes.c_float if fp32 else ctypes.c_double
    sfx = "_f32" if fp32 else "_f64"
    s = torch.as_tensor(np.atleast_1d(np.asarray(s_dev, float))).to(
        "cuda", T)
    n_e = len(s)
    Nx, Ny, Nz = geo["Nx"], geo["Ny"], geo["Nz"]
    re = torch.empty(n_e * Ny * Nx, dtype=T, device="cuda")
    im = torch.empty_like(re)
    vp = ctypes.c_void_p
    common = [vp(re.data_ptr()), vp(im.data_ptr()),
              *[ct(v) for v in _xtal6(xtal)], vp(s.data_ptr()),
              ctypes.c_int(n_e), ct(geo["dz"]), ct(geo["shift_px"]),
              ct(geo["ds"]), ct(geo["dx"]), ctypes.c_int(Nz),
              ctypes.c_int(Nx), ctypes.c_int(Ny), ct(geo["sheet_hw"]),
              ct(geo["fov_hy"])]
    stream = vp(torch.cuda.current_stream().cuda_stream)
    if mode == "fullfield":
        H = H_grid.to(T).contiguous()
        st = getattr(r, "ref_gpu_fullfield" + sfx)(*common, vp(H.data_ptr()),
                                                   stream)
    elif mode == "pristine":
        st = getattr(r, "ref_gpu_pristine" + sfx)(*common, stream)
    else:
        A = np.ascontiguousarray(np.asarray(an, dtype=np.float32 if fp32
                                            else np.float64))
        st = getattr(r, "ref_gpu_analytic" + sfx)(
            *common, A.ctypes.data_as(ctypes.POINTER(ct)), stream)
    if st != 0:
        raise RuntimeError(f"reference kernel launch failed: cudaError {st}")
    return torch.complex(re, im).reshape(n_e, Ny, Nx)
