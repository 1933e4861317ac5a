"""ctypes declarations of the C ABI in include/minife_gb300.h.

Loads the in-tree libminife_gb300.so (built by minife_gb300.build).  There is
no fallback: if the library cannot be built or loaded, importing the package's
compute entry points raises.
"""
from __future__ import annotations

import ctypes
import os
import shutil

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libminife_gb300.so")

MFE_OK, MFE_BAD_ARG, MFE_OOM, MFE_CUDA_ERR, MFE_BREAKDOWN, MFE_MAXITER, MFE_TIMEOUT, \
    MFE_NOT_SUPPORTED = range(8)
MFE_F64, MFE_F32 = 0, 1
MFE_PREC_F64, MFE_PREC_MIXED = 0, 1
MFE_TOL_ABSOLUTE, MFE_TOL_RELATIVE = 0, 1

c_int32 = ctypes.c_int32
c_int64 = ctypes.c_int64
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p


class MfeCsr(ctypes.Structure):
    _fields_ = [
        ("nrows", c_int64), ("ncols", c_int64), ("nnz", c_int64),
        ("row_offsets", c_void_p), ("cols", c_void_p), ("vals", c_void_p),
        ("dtype", c_int32), ("max_row_len", c_int32),
        ("box_nx", c_int32), ("box_ny", c_int32), ("box_nz", c_int32),
        ("owned", c_int32),
    ]


class MfeCgOpts(ctypes.Structure):
    _fields_ = [
        ("max_iter", c_int32), ("tol_mode", c_int32), ("tol", c_double),
        ("precision", c_int32), ("refine_k", c_int32), ("inner_tol", c_double),
        ("max_refine", c_int32), ("record_history", c_int32),
        ("A32", ctypes.POINTER(MfeCsr)), ("precond", c_int32), ("mixed_operator", c_int32),
        ("f64_operator", c_int32),
    ]


class MfeCgResult(ctypes.Structure):
    _fields_ = [
        ("num_iters", c_int32), ("status", c_int32), ("normr", c_double),
        ("normr0", c_double), ("final_resid", c_double), ("times", c_double * 5),
        ("refinements", c_int32), ("fp64_spmvs", c_int32), ("inner_operator", c_int32),
    ]


class MfeStencil64(ctypes.Structure):
    _fields_ = [("box_nx", c_int32), ("box_ny", c_int32), ("box_nz", c_int32),
                ("reserved", c_int32), ("w", c_double * 8), ("dd", c_double)]


class MfeMultiTuning(ctypes.Structure):
    _fields_ = [("z_chunk", c_int32)]


class MfeEll(ctypes.Structure):
    _fields_ = [("nrows", c_int64), ("ncols_per_row", c_int32), ("dtype", c_int32),
                ("cols", c_void_p), ("vals", c_void_p)]


class MfeSell(ctypes.Structure):
    _fields_ = [("nrows", c_int64), ("ncols_per_row", c_int32), ("reserved", c_int32),
                ("cols", c_void_p), ("vals", c_void_p)]


class MfeBatchTuning(ctypes.Structure):
    _fields_ = [("spmv_rows", c_int32), ("spmv_stages", c_int32), ("chunk_rows", c_int32)]


_P = ctypes.POINTER
# name -> (restype, argtypes)
SIGNATURES = {
    "mfe_abi_version": (ctypes.c_int, []),
    "mfe_ctx_create": (ctypes.c_int, [ctypes.c_int, _P(c_void_p)]),
    "mfe_ctx_destroy": (ctypes.c_int, [c_void_p]),
    "mfe_set_stream": (ctypes.c_int, [c_void_p, c_void_p]),
    "mfe_use_own_stream": (ctypes.c_int, [c_void_p]),
    "mfe_synchronize": (ctypes.c_int, [c_void_p]),
    "mfe_last_error_string": (ctypes.c_char_p, [c_void_p]),
    "mfe_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "mfe_device_sm_count": (ctypes.c_int, [c_void_p]),
    "mfe_device_alloc": (ctypes.c_int, [c_void_p, ctypes.c_size_t, _P(c_void_p)]),
    "mfe_device_free": (ctypes.c_int, [c_void_p, c_void_p]),
    "mfe_memcpy_h2d": (ctypes.c_int, [c_void_p, c_void_p, c_void_p, ctypes.c_size_t]),
    "mfe_memcpy_d2h": (ctypes.c_int, [c_void_p, c_void_p, c_void_p, ctypes.c_size_t]),
    "mfe_csr_alloc": (ctypes.c_int, [c_void_p, c_int64, c_int64, ctypes.c_int, _P(MfeCsr)]),
    "mfe_csr_free": (ctypes.c_int, [c_void_p, _P(MfeCsr)]),
    "mfe_box_dims": (ctypes.c_int, [ctypes.c_int] * 3 + [_P(c_int64), _P(c_int64)]),
    "mfe_generate_structure": (ctypes.c_int, [c_void_p] + [ctypes.c_int] * 3 + [_P(MfeCsr)]),
    "mfe_assemble": (ctypes.c_int, [c_void_p] + [ctypes.c_int] * 3 +
                     [c_void_p, _P(MfeCsr), c_void_p, ctypes.c_int]),
    "mfe_impose_dirichlet": (ctypes.c_int, [c_void_p, _P(MfeCsr), c_void_p, c_double,
                                            c_void_p, c_int64]),
    "mfe_box_bc_rows": (ctypes.c_int, [c_void_p] + [ctypes.c_int] * 4 + [c_void_p, _P(c_int64)]),
    "mfe_csr_convert_f32": (ctypes.c_int, [c_void_p, _P(MfeCsr), _P(MfeCsr)]),
    "mfe_spmv": (ctypes.c_int, [c_void_p, _P(MfeCsr), c_void_p, c_void_p]),
    "mfe_matvec_and_dot": (ctypes.c_int, [c_void_p, _P(MfeCsr), c_void_p, c_void_p,
                                          _P(c_double)]),
    "mfe_dot": (ctypes.c_int, [c_void_p, c_int64, c_void_p, c_void_p, _P(c_double)]),
    "mfe_dot_noalloc": (ctypes.c_int, [c_int64, c_void_p, c_void_p, c_void_p, c_void_p]),
    "mfe_stencil64_from_csr": (ctypes.c_int, [c_void_p, _P(MfeCsr), _P(MfeStencil64)]),
    "mfe_spmv_stencil64": (ctypes.c_int, [c_void_p, _P(MfeStencil64), c_void_p, c_void_p]),
    "mfe_gather": (ctypes.c_int, [c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "mfe_dot_f32": (ctypes.c_int, [c_void_p, c_int64, c_void_p, c_void_p, _P(c_double)]),
    "mfe_inject_wait_timeout": (ctypes.c_int, [c_void_p, c_int64]),
    "mfe_waxpby": (ctypes.c_int, [c_void_p, c_int64, c_double, c_void_p, c_double, c_void_p,
                                  c_void_p]),
    "mfe_fused_waxpby": (ctypes.c_int, [c_void_p, c_int64, c_double, c_void_p, c_double,
                                        c_void_p, c_void_p, c_double, c_void_p, c_double,
                                        c_void_p, c_void_p]),
    "mfe_cg_opts_default": (None, [_P(MfeCgOpts)]),
    "mfe_cg_solve": (ctypes.c_int, [c_void_p, _P(MfeCsr), c_void_p, c_void_p, _P(MfeCgOpts),
                                    _P(MfeCgResult)]),
    "mfe_cg_solve_host": (ctypes.c_int, [c_void_p, c_int64, c_int64, c_void_p, c_void_p,
                                         c_void_p, c_void_p, c_void_p, _P(MfeCgOpts),
                                         _P(MfeCgResult)]),
    "mfe_cg_history": (ctypes.c_int, [c_void_p, _P(c_double), c_int32, _P(c_int32)]),
    "mfe_verify_solution": (ctypes.c_int, [c_void_p] + [ctypes.c_int] * 3 +
                            [c_void_p, c_double, ctypes.c_int, _P(c_double),
                             _P(ctypes.c_int)]),
    "mfe_element_gradient": (ctypes.c_int, [c_void_p] + [ctypes.c_int] * 3 +
                             [c_void_p, c_void_p, c_void_p]),
    "mfe_box_zero_boundary": (ctypes.c_int, [c_void_p] + [ctypes.c_int] * 3 + [c_void_p]),
    "mfe_adjoint_grad": (ctypes.c_int, [c_void_p] + [ctypes.c_int] * 3 +
                         [c_void_p, c_void_p, _P(MfeCgOpts), c_void_p, c_void_p, _P(c_double),
                          _P(MfeCgResult), _P(MfeCgResult)]),
    "mfe_spmm": (ctypes.c_int, [c_void_p, _P(MfeCsr), c_int32, c_void_p, c_void_p]),
    "mfe_multi_set_tuning": (ctypes.c_int, [c_void_p, _P(MfeMultiTuning)]),
    "mfe_cg_solve_multi": (ctypes.c_int, [c_void_p, _P(MfeCsr), c_int32, c_void_p, c_void_p,
                                          _P(MfeCgOpts), _P(MfeCgResult)]),
    "mfe_batch_solve_boxes": (ctypes.c_int, [c_void_p, c_int32, c_void_p, _P(MfeCgOpts),
                                             c_void_p, _P(MfeCgResult)]),
    "mfe_batch_create": (ctypes.c_int, [c_void_p, c_int32, c_void_p, _P(c_void_p)]),
    "mfe_batch_set_tuning": (ctypes.c_int, [c_void_p, c_void_p, _P(MfeBatchTuning)]),
    "mfe_batch_info": (ctypes.c_int, [c_void_p, _P(c_int64), _P(c_int64), _P(c_double),
                                      _P(MfeBatchTuning)]),
    "mfe_batch_solve": (ctypes.c_int, [c_void_p, c_void_p, _P(MfeCgOpts), c_void_p,
                                       _P(MfeCgResult)]),
    "mfe_batch_destroy": (None, [c_void_p]),
    "mfe_write_matrix": (ctypes.c_int, [c_void_p, _P(MfeCsr), ctypes.c_char_p]),
    "mfe_csr_to_ell": (ctypes.c_int, [c_void_p, _P(MfeCsr), _P(MfeEll)]),
    "mfe_spmv_ell": (ctypes.c_int, [c_void_p, _P(MfeEll), c_void_p, c_void_p]),
    "mfe_ell_to_sell": (ctypes.c_int, [c_void_p, _P(MfeEll), _P(MfeSell)]),
    "mfe_spmv_sell": (ctypes.c_int, [c_void_p, _P(MfeSell), c_void_p, c_void_p]),
    "mfe_cg_solve_ell": (ctypes.c_int, [c_void_p, _P(MfeEll), c_void_p, c_void_p, _P(MfeCgOpts),
                                        _P(MfeCgResult)]),
    "mfe_write_vector": (ctypes.c_int, [c_void_p, c_int64, c_void_p, c_int64, ctypes.c_char_p]),
}

_LIB = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libminife_gb300.so, building it first when it is missing or stale
    and nvcc is available."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if build_if_missing and (shutil.which("nvcc") or os.path.exists("/usr/local/cuda/bin/nvcc")):
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libminife_gb300.so is missing; build it with "
                           "`python -m minife_gb300.build` (needs nvcc)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib
