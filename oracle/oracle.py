"""ctypes binding of the oracle (CPU restatement of miniFE's path).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference legs of bench.py.  The product path never imports
this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_CPUB = None

_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_u8p = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


def build() -> None:
    """Compile liboracle.so / libcpubase.so with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def lib():
    global _LIB
    if _LIB is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.orc_num_rows.restype = ctypes.c_int64
        L.orc_num_rows.argtypes = [ctypes.c_int] * 3
        L.orc_num_nonzeros.restype = ctypes.c_int64
        L.orc_num_nonzeros.argtypes = [ctypes.c_int] * 3
        L.orc_structure.argtypes = [ctypes.c_int] * 3 + [_i32p, _i32p]
        L.orc_gradient_values.argtypes = [_f64p]
        L.orc_elem_nodes_and_coords.argtypes = [ctypes.c_int] * 6 + [_i32p, _f64p]
        L.orc_diffusion_matrix_symm.argtypes = [_f64p, _f64p, ctypes.c_double, _f64p]
        L.orc_source_vector.argtypes = [_f64p, _f64p, _f64p]
        L.orc_assemble.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, _i32p, _i32p, _f64p, _f64p]
        L.orc_bc_masks.argtypes = [ctypes.c_int] * 3 + [_u8p, _u8p]
        L.orc_impose_dirichlet.argtypes = [ctypes.c_double, ctypes.c_int64, _i32p, _i32p,
                                           _f64p, _f64p, _u8p]
        L.orc_matvec.argtypes = [ctypes.c_int64, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.orc_dot.restype = ctypes.c_double
        L.orc_dot.argtypes = [ctypes.c_int64, _f64p, _f64p]
        L.orc_waxpby.argtypes = [ctypes.c_int64, ctypes.c_double, _f64p, ctypes.c_double,
                                 _f64p, _f64p]
        L.orc_cg_solve.argtypes = [ctypes.c_int64, _i32p, _i32p, _f64p, _f64p, _f64p,
                                   ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                   ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double),
                                   ctypes.c_void_p]
        L.orc_analytic_soln.restype = ctypes.c_double
        L.orc_analytic_soln.argtypes = [ctypes.c_double] * 3 + [ctypes.c_int] * 2
        L.orc_verify_solution.argtypes = [ctypes.c_int] * 3 + [_f64p, ctypes.c_double,
                                          ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.orc_build_system.argtypes = [ctypes.c_int] * 3 + [ctypes.c_void_p, _i32p, _i32p,
                                       _f64p, _f64p]
        L.orc_element_gradient.argtypes = [ctypes.c_int] * 3 + [_f64p, _f64p, _f64p]
        _LIB = L
    return _LIB


def cpubase():
    """The OpenMP CPU baseline library (libcpubase.so)."""
    global _CPUB
    if _CPUB is None:
        path = os.path.join(HERE, "libcpubase.so")
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.cpub_num_threads.restype = ctypes.c_int
        L.cpub_cg_solve.restype = ctypes.c_int
        L.cpub_cg_solve.argtypes = [ctypes.c_int64, _i32p, _i32p, _f64p, _f64p, _f64p,
                                    ctypes.c_int, ctypes.c_double, ctypes.c_int,
                                    ctypes.POINTER(ctypes.c_double)]
        _CPUB = L
    return _CPUB


def dims_rows_nnz(nx, ny, nz):
    L = lib()
    return int(L.orc_num_rows(nx, ny, nz)), int(L.orc_num_nonzeros(nx, ny, nz))


def structure(nx, ny, nz):
    n, nnz = dims_rows_nnz(nx, ny, nz)
    ro = np.zeros(n + 1, np.int32)
    cols = np.zeros(nnz, np.int32)
    lib().orc_structure(nx, ny, nz, ro, cols)
    return ro, cols


def assemble(nx, ny, nz, kappa=None):
    """Structure + element loop (before boundary conditions)."""
    ro, cols = structure(nx, ny, nz)
    vals = np.zeros(cols.size, np.float64)
    b = np.zeros(ro.size - 1, np.float64)
    kp = None
    if kappa is not None:
        kappa = np.ascontiguousarray(kappa, np.float64)
        kp = kappa.ctypes.data
    lib().orc_assemble(nx, ny, nz, kp, ro, cols, vals, b)
    return ro, cols, vals, b


def bc_masks(nx, ny, nz):
    n, _ = dims_rows_nnz(nx, ny, nz)
    m0 = np.zeros(n, np.uint8)
    m1 = np.zeros(n, np.uint8)
    lib().orc_bc_masks(nx, ny, nz, m0, m1)
    return m0, m1


def impose_dirichlet(value, ro, cols, vals, b, mask):
    lib().orc_impose_dirichlet(float(value), ro.size - 1, ro, cols, vals, b,
                               np.ascontiguousarray(mask, np.uint8))


def build_system(nx, ny, nz, kappa=None):
    """Full reference pipeline: structure, assembly, both Dirichlet passes."""
    n, nnz = dims_rows_nnz(nx, ny, nz)
    ro = np.zeros(n + 1, np.int32)
    cols = np.zeros(nnz, np.int32)
    vals = np.zeros(nnz, np.float64)
    b = np.zeros(n, np.float64)
    kp = None
    if kappa is not None:
        kappa = np.ascontiguousarray(kappa, np.float64)
        kp = kappa.ctypes.data
    rc = lib().orc_build_system(nx, ny, nz, kp, ro, cols, vals, b)
    if rc:
        raise MemoryError("orc_build_system failed")
    return ro, cols, vals, b


def matvec(ro, cols, vals, x):
    y = np.zeros(ro.size - 1, np.float64)
    lib().orc_matvec(ro.size - 1, ro, cols, vals, np.ascontiguousarray(x, np.float64), y)
    return y


def dot(x, y):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    return float(lib().orc_dot(x.size, x, y))


def waxpby(alpha, x, beta, y):
    x = np.ascontiguousarray(x, np.float64)
    y = np.ascontiguousarray(y, np.float64)
    w = np.zeros_like(x)
    lib().orc_waxpby(x.size, float(alpha), x, float(beta), y, w)
    return w


def cg_solve(ro, cols, vals, b, x0=None, max_iter=200, tol=2.220446049250313e-16,
             tol_mode=0, history=False):
    """Reference cg_solve; returns (x, num_iters, normr, status[, history])."""
    n = ro.size - 1
    x = np.zeros(n, np.float64) if x0 is None else np.array(x0, np.float64)
    it = ctypes.c_int(0)
    nr = ctypes.c_double(0.0)
    hist = np.zeros(max_iter + 1, np.float64) if history else None
    st = lib().orc_cg_solve(n, ro, cols, vals, np.ascontiguousarray(b, np.float64), x,
                            int(max_iter), float(tol), int(tol_mode),
                            ctypes.byref(it), ctypes.byref(nr),
                            hist.ctypes.data if history else None)
    out = (x, it.value, nr.value, st)
    if history:
        out = out + (hist[: it.value + 1],)
    return out


def verify_solution(nx, ny, nz, x, tolerance=0.06, whole=False):
    err = ctypes.c_double(0.0)
    rc = lib().orc_verify_solution(nx, ny, nz, np.ascontiguousarray(x, np.float64),
                                   float(tolerance), int(whole), ctypes.byref(err))
    return rc, err.value


def element_matrix(coords, k=1.0):
    g = np.zeros(192, np.float64)
    lib().orc_gradient_values(g)
    em = np.zeros(36, np.float64)
    lib().orc_diffusion_matrix_symm(np.ascontiguousarray(coords, np.float64), g, float(k), em)
    ev = np.zeros(8, np.float64)
    lib().orc_source_vector(np.ascontiguousarray(coords, np.float64), g, ev)
    return em, ev


def gradient_values():
    g = np.zeros(192, np.float64)
    lib().orc_gradient_values(g)
    return g


def element_gradient(nx, ny, nz, u, lam):
    g = np.zeros(nx * ny * nz, np.float64)
    lib().orc_element_gradient(nx, ny, nz, np.ascontiguousarray(u, np.float64),
                               np.ascontiguousarray(lam, np.float64), g)
    return g
