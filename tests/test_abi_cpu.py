"""CPU-side checks of the C ABI library: it builds for sm_103a, loads, and
exports every entry point that include/minife_gb300.h declares.  No compute
call is made (there is no GPU here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    text = open(os.path.join(ROOT, "include", "minife_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mfe_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from minife_gb300 import _abi
    lib = _abi.load()
    names = _declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each of them
    assert set(names) <= set(_abi.SIGNATURES), set(names) - set(_abi.SIGNATURES)


def test_box_dims_without_gpu():
    from minife_gb300 import box_dims
    assert box_dims(30, 30, 30) == (29791, 753571)
    assert box_dims(256, 256, 256) == (16974593, 454756609)
    assert box_dims(1, 1, 2) == (12, 112)


def test_bad_box_rejected():
    from minife_gb300 import MiniFEError, box_dims
    with pytest.raises(MiniFEError):
        box_dims(0, 5, 5)
    with pytest.raises(MiniFEError):
        box_dims(1000, 1000, 1000)  # >= 2^31 nonzeros


def test_status_strings_and_version():
    from minife_gb300 import _abi
    lib = _abi.load()
    assert lib.mfe_abi_version() == 3
    assert lib.mfe_status_string(0) == b"ok"
    assert lib.mfe_status_string(4) == b"numerical breakdown"


def test_ctx_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from minife_gb300 import _abi
    lib = _abi.load()
    h = ctypes.c_void_p()
    assert lib.mfe_ctx_create(0, ctypes.byref(h)) == _abi.MFE_CUDA_ERR


def test_cg_opts_default_matches_reference():
    from minife_gb300 import _abi
    o = _abi.MfeCgOpts()
    _abi.load().mfe_cg_opts_default(ctypes.byref(o))
    assert o.max_iter == 200          # driver.hpp:241
    assert o.tol == 2.220446049250313e-16  # driver.hpp:245
    assert o.tol_mode == 0 and o.precision == 0
