"""minife_gb300: miniFE's assemble-and-solve path on one GB300 GPU.

Python mirror of the reference's operator interface (Mantevo miniFE, ref/
variant) over the C ABI of libminife_gb300.so (include/minife_gb300.h):

  reference (C++ templates)                     here
  ---------------------------------------------  ---------------------------------
  CSRMatrix<S,LO,GO> (ref/src/CSRMatrix.hpp)      CSRMatrix (device arrays)
  Vector<S,LO,GO>    (ref/src/Vector.hpp)         torch CUDA tensor of float64
  generate_matrix_structure(mesh, A)              generate_matrix_structure(nx,ny,nz)
  assemble_FE_data(mesh, A, b, params)            assemble_FE_data(nx,ny,nz, A, b)
  impose_dirichlet(value, A, b, nx,ny,nz, rows)   impose_dirichlet(value, A, b, rows)
  matvec_std<M,V>()(A, x, y)                      matvec(A, x, y)
  matvec_and_dot(A, x, y)                         matvec_and_dot(A, x, y)
  dot(x, y), waxpby(a, x, b, y, w)                dot(x, y), waxpby(a, x, b, y, w)
  cg_solve(A, b, x, matvec, max_iter, tol, ...)   cg_solve(A, b, x, max_iter, tol, ...)
  verify_solution(mesh, x, tol)                   verify_solution(nx,ny,nz, x, tol)

Torch is used for device memory and streams only; every computation runs in
the library's CUDA kernels.  Errors raise MiniFEError carrying the C status.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

from . import _abi
from ._abi import (MFE_F32, MFE_F64, MFE_PREC_F64, MFE_PREC_MIXED, MFE_TOL_ABSOLUTE,
                   MFE_TOL_RELATIVE, MfeCgOpts, MfeCgResult, MfeCsr)

__all__ = [
    "MiniFEError", "Context", "CSRMatrix", "CGResult", "default_context", "box_dims",
    "generate_matrix_structure", "assemble_FE_data", "impose_dirichlet", "box_bc_rows",
    "build_system", "matvec", "matvec_and_dot", "dot", "dot_f32", "waxpby", "fused_waxpby",
    "inject_wait_timeout", "Stencil64", "matvec_stencil64", "set_multi_tuning", "cg_solve",
    "cg_solve_host", "cg_solve_multi", "Batch", "batch_solve_boxes", "verify_solution",
    "element_gradient", "to_f32", "spmm", "ELLMatrix", "matvec_ell", "cg_solve_ell",
]

DBL_EPSILON = 2.220446049250313e-16


class MiniFEError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__("minife_gb300 status %d (%s): %s" % (status, _status_name(status), msg))
        self.status = status


def _status_name(s: int) -> str:
    try:
        return _abi.load().mfe_status_string(s).decode()
    except Exception:  # pragma: no cover - load failure path
        return str(s)


def _torch():
    import torch
    return torch


class Context:
    """One mfe_ctx: a device and a stream.  Work is issued on torch's current
    CUDA stream at call time, so it orders with surrounding torch work."""

    def __init__(self, device: int = 0):
        self.lib = _abi.load()
        h = ctypes.c_void_p()
        st = self.lib.mfe_ctx_create(int(device), ctypes.byref(h))
        if st != 0:
            raise MiniFEError(st, "mfe_ctx_create(device=%d) failed" % device)
        self.h = h
        self.device = int(device)
        self._bound_stream = -1

    def close(self):
        if getattr(self, "h", None):
            self.lib.mfe_ctx_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover - interpreter teardown order varies
        try:
            self.close()
        except Exception:
            pass

    def bind_torch_stream(self):
        torch = _torch()
        s = torch.cuda.current_stream(self.device).cuda_stream
        if s != self._bound_stream:
            self.check(self.lib.mfe_set_stream(self.h, ctypes.c_void_p(s)), "mfe_set_stream")
            self._bound_stream = s

    def check(self, st: int, what: str):
        if st != 0:
            msg = self.lib.mfe_last_error_string(self.h)
            raise MiniFEError(st, "%s: %s" % (what, msg.decode() if msg else ""))

    @property
    def sm_count(self) -> int:
        return int(self.lib.mfe_device_sm_count(self.h))

    def synchronize(self):
        self.check(self.lib.mfe_synchronize(self.h), "mfe_synchronize")


_DEFAULT = {}


def default_context(device: int | None = None) -> Context:
    torch = _torch()
    if device is None:
        device = torch.cuda.current_device()
    ctx = _DEFAULT.get(device)
    if ctx is None:
        ctx = Context(device)
        _DEFAULT[device] = ctx
    ctx.bind_torch_stream()
    return ctx


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


def box_dims(nx: int, ny: int, nz: int):
    """(rows, nonzeros) of the nx*ny*nz element box."""
    n = ctypes.c_int64()
    nnz = ctypes.c_int64()
    st = _abi.load().mfe_box_dims(nx, ny, nz, ctypes.byref(n), ctypes.byref(nnz))
    if st != 0:
        raise MiniFEError(st, "bad box dimensions %dx%dx%d" % (nx, ny, nz))
    return n.value, nnz.value


class CSRMatrix:
    """Device CSR with the reference CSRMatrix's fields (one rank:
    rows[i] == i, has_local_indices true, num_cols == nrows; a rank's local
    matrix of a multi-rank decomposition has num_cols = owned rows plus
    externals, minife_gb300.halo)."""

    def __init__(self, row_offsets, packed_cols, packed_coefs, box=(0, 0, 0), max_row_len=0,
                 num_cols=None):
        torch = _torch()
        assert row_offsets.dtype == torch.int32 and packed_cols.dtype == torch.int32
        assert packed_coefs.dtype in (torch.float64, torch.float32)
        self.row_offsets = row_offsets
        self.packed_cols = packed_cols
        self.packed_coefs = packed_coefs
        self.box = tuple(box)
        self.max_row_len = int(max_row_len)
        self.has_local_indices = True
        self._num_cols = None if num_cols is None else int(num_cols)

    @property
    def nrows(self) -> int:
        return self.row_offsets.numel() - 1

    @property
    def num_cols(self) -> int:
        return self.nrows if self._num_cols is None else self._num_cols

    @property
    def nnz(self) -> int:
        return self.packed_cols.numel()

    def num_nonzeros(self) -> int:
        return self.nnz

    @property
    def dtype(self):
        return self.packed_coefs.dtype

    def c(self) -> MfeCsr:
        torch = _torch()
        m = MfeCsr()
        m.nrows = self.nrows
        m.ncols = self.num_cols
        m.nnz = self.nnz
        m.row_offsets = self.row_offsets.data_ptr()
        m.cols = self.packed_cols.data_ptr()
        m.vals = self.packed_coefs.data_ptr()
        m.dtype = MFE_F64 if self.packed_coefs.dtype == torch.float64 else MFE_F32
        m.max_row_len = self.max_row_len
        m.box_nx, m.box_ny, m.box_nz = self.box
        m.owned = 0
        return m

    @staticmethod
    def empty_box(nx, ny, nz, device=None, dtype=None):
        torch = _torch()
        n, nnz = box_dims(nx, ny, nz)
        dev = torch.device("cuda", torch.cuda.current_device() if device is None else device)
        # +4 elements of padding: the bulk-copy granule is 16 bytes
        ro = torch.empty(n + 1, dtype=torch.int32, device=dev)
        cols = torch.empty(nnz + 4, dtype=torch.int32, device=dev)[:nnz]
        vals = torch.empty(nnz + 4, dtype=dtype or torch.float64, device=dev)[:nnz]
        return CSRMatrix(ro, cols, vals, box=(nx, ny, nz), max_row_len=27)


class ELLMatrix:
    """The reference's ELLMatrix (ref/src/ELLMatrix.hpp) on the device:
    ncols_per_row entries per row, row-major, the row's columns first and
    then padding (column 0, value 0)."""

    def __init__(self, cols, coefs, ncols_per_row: int):
        self.cols = cols
        self.coefs = coefs
        self.num_cols_per_row = int(ncols_per_row)
        self.has_local_indices = True

    @property
    def nrows(self) -> int:
        return self.cols.numel() // self.num_cols_per_row

    def num_nonzeros(self) -> int:
        return self.cols.numel()

    def c(self):
        torch = _torch()
        e = _abi.MfeEll()
        e.nrows = self.nrows
        e.ncols_per_row = self.num_cols_per_row
        e.dtype = MFE_F64 if self.coefs.dtype == torch.float64 else MFE_F32
        e.cols = self.cols.data_ptr()
        e.vals = self.coefs.data_ptr()
        return e

    @staticmethod
    def from_csr(A: "CSRMatrix", ncols_per_row: int = 27, ctx: Context | None = None):
        torch = _torch()
        ctx = ctx or default_context()
        n = A.nrows
        E = ELLMatrix(torch.empty(n * ncols_per_row + 4, dtype=torch.int32,
                                  device=A.packed_cols.device)[: n * ncols_per_row],
                      torch.empty(n * ncols_per_row + 4, dtype=A.packed_coefs.dtype,
                                  device=A.packed_cols.device)[: n * ncols_per_row],
                      ncols_per_row)
        e = E.c()
        m = A.c()
        ctx.check(ctx.lib.mfe_csr_to_ell(ctx.h, ctypes.byref(m), ctypes.byref(e)), "mfe_csr_to_ell")
        return E


class SELLMatrix:
    """A sliced copy of an FP64 ELLMatrix (mfe_sell): rows in slices of 32,
    column-major inside a slice -- entry k of row r at ((r // 32) *
    ncols_per_row + k) * 32 + r % 32 -- so the entries k of 32 consecutive
    rows are one coalesced line.  The ELL CG runs its iterations on such a
    copy."""

    SLICE = 32

    def __init__(self, cols, coefs, nrows: int, ncols_per_row: int):
        self.cols = cols
        self.coefs = coefs
        self.nrows = int(nrows)
        self.num_cols_per_row = int(ncols_per_row)

    @staticmethod
    def entries(nrows: int, ncols_per_row: int) -> int:
        s = SELLMatrix.SLICE
        return (nrows + s - 1) // s * s * ncols_per_row

    def c(self):
        e = _abi.MfeSell()
        e.nrows = self.nrows
        e.ncols_per_row = self.num_cols_per_row
        e.cols = self.cols.data_ptr()
        e.vals = self.coefs.data_ptr()
        return e

    @staticmethod
    def from_ell(E: "ELLMatrix", ctx: Context | None = None):
        torch = _torch()
        ctx = ctx or default_context()
        m = SELLMatrix.entries(E.nrows, E.num_cols_per_row)
        S = SELLMatrix(torch.empty(m, dtype=torch.int32, device=E.cols.device),
                       torch.empty(m, dtype=torch.float64, device=E.cols.device),
                       E.nrows, E.num_cols_per_row)
        s = S.c()
        e = E.c()
        ctx.check(ctx.lib.mfe_ell_to_sell(ctx.h, ctypes.byref(e), ctypes.byref(s)), "mfe_ell_to_sell")
        return S


def matvec_sell(S: SELLMatrix, x, y, ctx: Context | None = None):
    """y = A x with the sliced ELL copy (every stored entry summed)."""
    ctx = ctx or default_context()
    s = S.c()
    ctx.check(ctx.lib.mfe_spmv_sell(ctx.h, ctypes.byref(s), _ptr(x), _ptr(y)), "mfe_spmv_sell")
    return y


def matvec_ell(E: ELLMatrix, x, y, ctx: Context | None = None):
    """matvec_std<ELLMatrix> (ref/src/SparseMatrix_functions.hpp:579-611)."""
    ctx = ctx or default_context()
    e = E.c()
    ctx.check(ctx.lib.mfe_spmv_ell(ctx.h, ctypes.byref(e), _ptr(x), _ptr(y)), "mfe_spmv_ell")
    return y


def cg_solve_ell(E: ELLMatrix, b, x, max_iter: int = 200, tol: float = DBL_EPSILON,
                 tol_mode: str = "absolute", ctx: Context | None = None) -> CGResult:
    """cg_solve with the ELL matvec (FP64)."""
    ctx = ctx or default_context()
    e = E.c()
    o, _ = _opts(max_iter, tol, tol_mode, "f64")
    r = MfeCgResult()
    st = ctx.lib.mfe_cg_solve_ell(ctx.h, ctypes.byref(e), _ptr(b), _ptr(x), ctypes.byref(o),
                                  ctypes.byref(r))
    if st not in (0, _abi.MFE_BREAKDOWN, _abi.MFE_MAXITER):
        ctx.check(st, "mfe_cg_solve_ell")
    return _result(ctx, r, False)


def generate_matrix_structure(nx, ny, nz, ctx: Context | None = None) -> CSRMatrix:
    """generate_matrix_structure (ref/src/generate_matrix_structure.hpp:47):
    27-point sparsity with zero coefficients."""
    ctx = ctx or default_context()
    A = CSRMatrix.empty_box(nx, ny, nz, device=ctx.device)
    m = A.c()
    ctx.check(ctx.lib.mfe_generate_structure(ctx.h, nx, ny, nz, ctypes.byref(m)),
              "mfe_generate_structure")
    return A


def assemble_FE_data(nx, ny, nz, A: CSRMatrix, b, kappa=None, impose_bc: bool = False,
                     ctx: Context | None = None):
    """assemble_FE_data (ref/src/assemble_FE_data.hpp:38): element loop into
    A and b (overwritten).  kappa: optional per-element conductivity (CUDA
    float64 tensor of nx*ny*nz).  impose_bc also applies both Dirichlet passes
    of driver.hpp:214-218 in the same kernel."""
    ctx = ctx or default_context()
    m = A.c()
    ctx.check(ctx.lib.mfe_assemble(ctx.h, nx, ny, nz, _ptr(kappa), ctypes.byref(m), _ptr(b),
                                   1 if impose_bc else 0), "mfe_assemble")
    A.max_row_len = 27
    A.box = (nx, ny, nz)
    return A, b


def box_bc_rows(nx, ny, nz, which: int, ctx: Context | None = None):
    """The bc_rows_0 (which=0) / bc_rows_1 (which=1) sets of
    simple_mesh_description as an ascending int32 CUDA tensor."""
    torch = _torch()
    ctx = ctx or default_context()
    cnt = ctypes.c_int64()
    ctx.check(ctx.lib.mfe_box_bc_rows(ctx.h, nx, ny, nz, which, None, ctypes.byref(cnt)),
              "mfe_box_bc_rows")
    rows = torch.empty(max(cnt.value, 1), dtype=torch.int32, device="cuda:%d" % ctx.device)
    ctx.check(ctx.lib.mfe_box_bc_rows(ctx.h, nx, ny, nz, which, _ptr(rows), ctypes.byref(cnt)),
              "mfe_box_bc_rows")
    return rows[: cnt.value]


def impose_dirichlet(value: float, A: CSRMatrix, b, bc_rows, ctx: Context | None = None):
    """impose_dirichlet (ref/src/SparseMatrix_functions.hpp:434) with bc_rows
    an ascending int32 CUDA tensor."""
    ctx = ctx or default_context()
    m = A.c()
    ctx.check(ctx.lib.mfe_impose_dirichlet(ctx.h, ctypes.byref(m), _ptr(b), float(value),
                                           _ptr(bc_rows), bc_rows.numel()),
              "mfe_impose_dirichlet")


def build_system(nx, ny, nz, kappa=None, ctx: Context | None = None):
    """driver.hpp:159-218 for one rank: structure, assembly, both Dirichlet
    passes.  Returns (A, b) on the device."""
    torch = _torch()
    ctx = ctx or default_context()
    A = CSRMatrix.empty_box(nx, ny, nz, device=ctx.device)
    b = torch.empty(A.nrows, dtype=torch.float64, device="cuda:%d" % ctx.device)
    assemble_FE_data(nx, ny, nz, A, b, kappa=kappa, impose_bc=True, ctx=ctx)
    return A, b


def to_f32(A: CSRMatrix, ctx: Context | None = None) -> CSRMatrix:
    """FP32 copy of A's values sharing A's structure arrays."""
    torch = _torch()
    ctx = ctx or default_context()
    vals = torch.empty(A.nnz + 4, dtype=torch.float32, device=A.packed_coefs.device)[: A.nnz]
    B = CSRMatrix(A.row_offsets, A.packed_cols, vals, box=A.box, max_row_len=A.max_row_len)
    ms, md = A.c(), B.c()
    ctx.check(ctx.lib.mfe_csr_convert_f32(ctx.h, ctypes.byref(ms), ctypes.byref(md)),
              "mfe_csr_convert_f32")
    return B


def matvec(A: CSRMatrix, x, y, ctx: Context | None = None):
    """matvec_std (ref/src/SparseMatrix_functions.hpp:545): y = A x."""
    ctx = ctx or default_context()
    m = A.c()
    ctx.check(ctx.lib.mfe_spmv(ctx.h, ctypes.byref(m), _ptr(x), _ptr(y)), "mfe_spmv")
    return y


def matvec_and_dot(A: CSRMatrix, x, y, ctx: Context | None = None) -> float:
    ctx = ctx or default_context()
    m = A.c()
    out = ctypes.c_double()
    ctx.check(ctx.lib.mfe_matvec_and_dot(ctx.h, ctypes.byref(m), _ptr(x), _ptr(y),
                                         ctypes.byref(out)), "mfe_matvec_and_dot")
    return out.value


def spmm(A: CSRMatrix, X, Y, ctx: Context | None = None):
    """Y = A X for row-major X, Y of shape (nrows, nrhs)."""
    ctx = ctx or default_context()
    m = A.c()
    ctx.check(ctx.lib.mfe_spmm(ctx.h, ctypes.byref(m), X.shape[1], _ptr(X), _ptr(Y)), "mfe_spmm")
    return Y


def dot(x, y, ctx: Context | None = None) -> float:
    ctx = ctx or default_context()
    out = ctypes.c_double()
    ctx.check(ctx.lib.mfe_dot(ctx.h, x.numel(), _ptr(x), _ptr(y), ctypes.byref(out)), "mfe_dot")
    return out.value


def waxpby(alpha, x, beta, y, w, ctx: Context | None = None):
    ctx = ctx or default_context()
    ctx.check(ctx.lib.mfe_waxpby(ctx.h, x.numel(), float(alpha), _ptr(x), float(beta), _ptr(y),
                                 _ptr(w)), "mfe_waxpby")
    return w


class Stencil64:
    """The verified FP64 stencil operator of a miniFE box matrix
    (mfe_stencil64_from_csr): checked once against every entry of A, then
    applied by matvec_stencil64 with 12.5 FP64 operations per row on average."""

    def __init__(self, A: "CSRMatrix", ctx: Context | None = None):
        ctx = ctx or default_context()
        self.s = _abi.MfeStencil64()
        m = A.c()
        ctx.check(ctx.lib.mfe_stencil64_from_csr(ctx.h, ctypes.byref(m), ctypes.byref(self.s)),
                  "mfe_stencil64_from_csr")

    @property
    def weights(self):
        return list(self.s.w), self.s.dd


def matvec_stencil64(S: Stencil64, x, y, ctx: Context | None = None):
    """y = S x through the verified FP64 stencil operator."""
    ctx = ctx or default_context()
    ctx.check(ctx.lib.mfe_spmv_stencil64(ctx.h, ctypes.byref(S.s), _ptr(x), _ptr(y)),
              "mfe_spmv_stencil64")
    return y


def gather(x, idx, out=None, ctx: Context | None = None):
    """out[i] = x[idx[i]] on the device (mfe_gather; idx int32)."""
    torch = _torch()
    ctx = ctx or default_context()
    if out is None:
        out = torch.empty(idx.numel(), dtype=torch.float64, device=x.device)
    ctx.check(ctx.lib.mfe_gather(ctx.h, idx.numel(), _ptr(idx), _ptr(x), _ptr(out)), "mfe_gather")
    return out


def dot_f32(x, y, ctx: Context | None = None) -> float:
    """x.y of FP32 device vectors, accumulated in double-float as the mixed
    solvers' reductions are (mfe_dot_f32)."""
    ctx = ctx or default_context()
    out = ctypes.c_double()
    ctx.check(ctx.lib.mfe_dot_f32(ctx.h, x.numel(), _ptr(x), _ptr(y), ctypes.byref(out)),
              "mfe_dot_f32")
    return out.value


def inject_wait_timeout(wait_ns: int = 20_000_000, ctx: Context | None = None):
    """Test hook: the next box-structured SpMV on the context withholds its
    copies, so its bounded waits run out after wait_ns (mfe_inject_wait_timeout)."""
    ctx = ctx or default_context()
    ctx.check(ctx.lib.mfe_inject_wait_timeout(ctx.h, int(wait_ns)), "mfe_inject_wait_timeout")


def fused_waxpby(alpha, x, beta, y, w, alpha2, x2, beta2, y2, w2, ctx: Context | None = None):
    ctx = ctx or default_context()
    ctx.check(ctx.lib.mfe_fused_waxpby(ctx.h, x.numel(), float(alpha), _ptr(x), float(beta),
                                       _ptr(y), _ptr(w), float(alpha2), _ptr(x2), float(beta2),
                                       _ptr(y2), _ptr(w2)), "mfe_fused_waxpby")


@dataclass
class CGResult:
    num_iters: int
    normr: float
    normr0: float
    final_resid: float
    status: int
    times: tuple
    refinements: int
    history: list | None = None
    # the operator of the CG iteration: for mixed solves the FP32 one
    # ("stencil", "values" or "padded"); for FP64 solves "stencil64" (the
    # verified FP64 stencil operator) or "none" (the CSR values)
    inner_operator: str = "none"
    # products with the FP64 CSR values (initial and true residuals of a
    # stencil solve; every iteration's product otherwise)
    fp64_spmvs: int = 0

    @property
    def total_time(self) -> float:
        return self.times[4]


def _opts(max_iter, tol, tol_mode, precision, refine_k=0, inner_tol=0.0, max_refine=0,
          record_history=False, A32=None, precond="none", mixed_operator="auto",
          f64_operator="auto"):
    o = MfeCgOpts()
    _abi.load().mfe_cg_opts_default(ctypes.byref(o))
    o.max_iter = int(max_iter)
    o.tol = float(tol)
    o.tol_mode = {"absolute": MFE_TOL_ABSOLUTE, "relative": MFE_TOL_RELATIVE}[tol_mode]
    o.precision = {"f64": MFE_PREC_F64, "mixed": MFE_PREC_MIXED}[precision]
    o.refine_k = int(refine_k)
    o.inner_tol = float(inner_tol)
    o.max_refine = int(max_refine)
    o.record_history = 1 if record_history else 0
    o.precond = {"none": 0, "jacobi": 1}[precond]
    o.mixed_operator = {"auto": 0, "values": 1}[mixed_operator]
    o.f64_operator = {"auto": 0, "csr": 1}[f64_operator]
    keep = None
    if A32 is not None:
        keep = A32.c()
        o.A32 = ctypes.pointer(keep)
    return o, keep


def _result(ctx, r: MfeCgResult, record_history: bool) -> CGResult:
    hist = None
    if record_history:
        cnt = ctypes.c_int32()
        ctx.lib.mfe_cg_history(ctx.h, None, 0, ctypes.byref(cnt))
        buf = (ctypes.c_double * max(cnt.value, 1))()
        ctx.lib.mfe_cg_history(ctx.h, buf, cnt.value, ctypes.byref(cnt))
        hist = list(buf[: cnt.value])
    return _cg_result(r, hist)


_INNER = {0: "none", 1: "stencil", 2: "values", 3: "padded", 4: "stencil64"}


def _cg_result(r: MfeCgResult, hist=None) -> CGResult:
    return CGResult(r.num_iters, r.normr, r.normr0, r.final_resid, r.status, tuple(r.times),
                    r.refinements, hist, _INNER.get(r.inner_operator, "none"), r.fp64_spmvs)


def cg_solve(A: CSRMatrix, b, x, max_iter: int = 200, tol: float = DBL_EPSILON,
             tol_mode: str = "absolute", precision: str = "f64", refine_k: int = 0,
             inner_tol: float = 0.0, max_refine: int = 0, record_history: bool = False,
             A32: CSRMatrix | None = None, allow_breakdown: bool = True,
             precond: str = "none", mixed_operator: str = "auto",
             f64_operator: str = "auto", ctx: Context | None = None) -> CGResult:
    """cg_solve (ref/src/cg_solve.hpp:69) on device vectors; x holds the
    initial guess and receives the solution.  Breakdown (the reference prints
    an error and returns) is reported in CGResult.status unless
    allow_breakdown is False.  precond="jacobi" runs the Jacobi-preconditioned
    CG (FP64, stops on ||r|| after the update).  mixed_operator="values"
    makes the mixed solver use the FP32 copy of the values even where the
    verified FP32 stencil operator applies ("auto").  f64_operator="csr"
    makes the FP64 solver use the CSR values (matvec_std) even where the
    verified FP64 stencil operator applies ("auto")."""
    ctx = ctx or default_context()
    m = A.c()
    o, keep = _opts(max_iter, tol, tol_mode, precision, refine_k, inner_tol, max_refine,
                    record_history, A32, precond, mixed_operator, f64_operator)
    r = MfeCgResult()
    st = ctx.lib.mfe_cg_solve(ctx.h, ctypes.byref(m), _ptr(b), _ptr(x), ctypes.byref(o),
                              ctypes.byref(r))
    del keep
    if not (st == 0 or (allow_breakdown and st in (_abi.MFE_BREAKDOWN, _abi.MFE_MAXITER))):
        ctx.check(st, "mfe_cg_solve")
    return _result(ctx, r, record_history)


def cg_solve_multi(A: CSRMatrix, B, X, max_iter: int = 200, tol: float = DBL_EPSILON,
                   tol_mode: str = "absolute", precision: str = "mixed", refine_k: int = 0,
                   ctx: Context | None = None, inner_tol: float = 0.0,
                   max_refine: int = 0, mixed_operator: str = "auto") -> list:
    """nrhs independent CG solves on one box matrix advanced together (one
    matrix read per iteration for all of them).  B, X: device (n, nrhs) FP64,
    contiguous; X holds the initial guesses and receives the solutions.
    nrhs divides 32.  precision "f64" runs the reference's CG per column
    (ref/src/cg_solve.hpp:69); "mixed" runs FP32 products with FP64 reliable
    updates: with 32 columns on the verified FP32 stencil operator where it
    applies (mixed_operator "auto"), else on the FP32 values ("values").
    Returns one CGResult per right-hand side."""
    ctx = ctx or default_context()
    if B.dim() != 2 or tuple(X.shape) != tuple(B.shape):
        raise ValueError("B and X must be (n, nrhs) with the same shape")
    nrhs = B.shape[1]
    m = A.c()
    o, _ = _opts(max_iter, tol, tol_mode, precision, refine_k, inner_tol, max_refine,
                 mixed_operator=mixed_operator)
    res = (MfeCgResult * nrhs)()
    st = ctx.lib.mfe_cg_solve_multi(ctx.h, ctypes.byref(m), nrhs, _ptr(B), _ptr(X),
                                    ctypes.byref(o), res)
    if st not in (0, _abi.MFE_BREAKDOWN, _abi.MFE_MAXITER):
        ctx.check(st, "mfe_cg_solve_multi")
    return [_cg_result(r) for r in res]


def set_multi_tuning(z_chunk: int = 0, ctx: Context | None = None):
    """Launch shape of the multi-RHS solver on the context
    (mfe_multi_set_tuning): z steps per work item of the 32-column stencil
    SpMM (0: the default)."""
    ctx = ctx or default_context()
    t = _abi.MfeMultiTuning(int(z_chunk))
    ctx.check(ctx.lib.mfe_multi_set_tuning(ctx.h, ctypes.byref(t)), "mfe_multi_set_tuning")


class Batch:
    """nbox independent miniFE boxes (k = 1, the reference's boundary
    conditions) assembled once into one device store (mfe_batch_create) and
    solved together any number of times.  Box i's solution is
    x[offsets[i]:offsets[i+1]] of the vector solve() returns."""

    def __init__(self, dims, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.dims = [tuple(int(v) for v in d) for d in dims]
        self.offsets = [0]
        for d in self.dims:
            self.offsets.append(self.offsets[-1] + box_dims(*d)[0])
        flat = (ctypes.c_int32 * (3 * len(self.dims)))(*[v for d in self.dims for v in d])
        h = ctypes.c_void_p()
        self.ctx.check(self.ctx.lib.mfe_batch_create(self.ctx.h, len(self.dims), flat,
                                                     ctypes.byref(h)), "mfe_batch_create")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.mfe_batch_destroy(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover - interpreter teardown order varies
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        """(rows, nonzeros, assembly seconds, tuning dict)."""
        rows, nnz, t = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_double()
        tu = _abi.MfeBatchTuning()
        self.ctx.lib.mfe_batch_info(self.h, ctypes.byref(rows), ctypes.byref(nnz),
                                    ctypes.byref(t), ctypes.byref(tu))
        return rows.value, nnz.value, t.value, {"spmv_rows": tu.spmv_rows,
                                                "spmv_stages": tu.spmv_stages,
                                                "chunk_rows": tu.chunk_rows}

    def set_tuning(self, spmv_rows: int = 256, spmv_stages: int = 2, chunk_rows: int = 8192):
        tu = _abi.MfeBatchTuning(int(spmv_rows), int(spmv_stages), int(chunk_rows))
        self.ctx.check(self.ctx.lib.mfe_batch_set_tuning(self.ctx.h, self.h, ctypes.byref(tu)),
                       "mfe_batch_set_tuning")

    def solve(self, max_iter: int = 200, tol: float = DBL_EPSILON, tol_mode: str = "absolute",
              precision: str = "mixed", refine_k: int = 0, x=None, mixed_operator: str = "auto",
              inner_tol: float = 0.0, max_refine: int = 0):
        """Returns (x, results): results holds one CGResult per box (times[0] =
        assembly of the batch, times[4] = the batched solve, in seconds).
        Mixed precision: mixed_operator "auto" uses the verified FP32 stencil
        when every box passes its check (else the padded FP32 values),
        "values" always the padded FP32 values."""
        torch = _torch()
        ctx = self.ctx
        ctx.bind_torch_stream()
        if x is None:
            x = torch.empty(max(self.offsets[-1], 1), dtype=torch.float64, device="cuda")
        o, _ = _opts(max_iter, tol, tol_mode, precision, refine_k, inner_tol, max_refine,
                     mixed_operator=mixed_operator)
        res = (MfeCgResult * len(self.dims))()
        st = ctx.lib.mfe_batch_solve(ctx.h, self.h, ctypes.byref(o), _ptr(x), res)
        if st not in (0, _abi.MFE_BREAKDOWN, _abi.MFE_MAXITER):
            ctx.check(st, "mfe_batch_solve")
        return x, [_cg_result(r) for r in res]


def batch_solve_boxes(dims, max_iter: int = 200, tol: float = DBL_EPSILON,
                      tol_mode: str = "absolute", precision: str = "mixed", refine_k: int = 0,
                      tuning: dict | None = None, ctx: Context | None = None,
                      mixed_operator: str = "auto", inner_tol: float = 0.0, max_refine: int = 0):
    """Assemble and solve len(dims) independent miniFE boxes together
    (mfe_batch_solve_boxes).  Returns (x, offsets, results); box i's rows are
    x[offsets[i]:offsets[i+1]]."""
    b = Batch(dims, ctx)
    try:
        if tuning:
            b.set_tuning(**tuning)
        x, res = b.solve(max_iter, tol, tol_mode, precision, refine_k,
                         mixed_operator=mixed_operator, inner_tol=inner_tol,
                         max_refine=max_refine)
        return x, b.offsets, res
    finally:
        b.close()


def cg_solve_host(row_offsets, cols, vals, b, x, max_iter=200, tol=DBL_EPSILON,
                  tol_mode="absolute", precision="f64", f64_operator="auto",
                  ctx: Context | None = None) -> CGResult:
    """Drop-in host call: CSR and vectors in host memory (numpy arrays or CPU
    tensors, int32 / float64); x is updated in place."""
    import numpy as np
    ctx = ctx or default_context()

    def hp(a):
        if hasattr(a, "data_ptr"):
            return ctypes.c_void_p(a.data_ptr())
        return a.ctypes.data_as(ctypes.c_void_p)

    n = (row_offsets.shape[0] if hasattr(row_offsets, "shape") else len(row_offsets)) - 1
    nnz = cols.shape[0]
    o, _ = _opts(max_iter, tol, tol_mode, precision, f64_operator=f64_operator)
    r = MfeCgResult()
    st = ctx.lib.mfe_cg_solve_host(ctx.h, n, nnz, hp(row_offsets), hp(cols), hp(vals), hp(b),
                                   hp(x), ctypes.byref(o), ctypes.byref(r))
    if st not in (0, _abi.MFE_BREAKDOWN, _abi.MFE_MAXITER):
        ctx.check(st, "mfe_cg_solve_host")
    del np
    return _result(ctx, r, False)


def verify_solution(nx, ny, nz, x, tolerance=0.06, whole_domain=False,
                    ctx: Context | None = None):
    """verify_solution (ref/fem/verify_solution.hpp:55): returns (return_code,
    max_abs_error); return_code 0 = within tolerance, as in the reference."""
    ctx = ctx or default_context()
    err = ctypes.c_double()
    ok = ctypes.c_int()
    ctx.check(ctx.lib.mfe_verify_solution(ctx.h, nx, ny, nz, _ptr(x), float(tolerance),
                                          1 if whole_domain else 0, ctypes.byref(err),
                                          ctypes.byref(ok)), "mfe_verify_solution")
    return (0 if ok.value else 1), err.value


def element_gradient(nx, ny, nz, u, lam, g=None, ctx: Context | None = None):
    """g[e] = -lambda_e^T Khat_e u_e for every element (adjoint contraction)."""
    torch = _torch()
    ctx = ctx or default_context()
    if g is None:
        g = torch.empty(nx * ny * nz, dtype=torch.float64, device=u.device)
    ctx.check(ctx.lib.mfe_element_gradient(ctx.h, nx, ny, nz, _ptr(u), _ptr(lam), _ptr(g)),
              "mfe_element_gradient")
    return g


def box_zero_boundary(nx, ny, nz, v, ctx: Context | None = None):
    """v[r] = 0 on every Dirichlet row of the box (in place)."""
    ctx = ctx or default_context()
    ctx.check(ctx.lib.mfe_box_zero_boundary(ctx.h, nx, ny, nz, _ptr(v)), "mfe_box_zero_boundary")
    return v
