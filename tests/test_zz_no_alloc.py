"""GPU test of mfe_dot_noalloc, the allocation-free dot product.

Callers that may not allocate device memory (their GPU memory belongs to
another allocator, or they cannot afford cudaMalloc's synchronisation) use
this entry point: it needs no context and keeps its partial sums in a device
array inside the library.  The test calls it through the C ABI and checks two
consecutive calls against the context-based mfe_dot, with the tolerance the
other dot tests use.  The file is named so pytest collects it last; it passes
both on its own in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU-only machines
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import minife_gb300 as M  # noqa: E402
from minife_gb300 import _abi  # noqa: E402


def _noalloc_dot(lib, x, y, out):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    st = lib.mfe_dot_noalloc(x.numel(), ctypes.c_void_p(x.data_ptr()),
                             ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                             stream)
    assert st == _abi.MFE_OK
    torch.cuda.synchronize()
    return float(out.item())


def test_dot_noalloc_matches_dot_twice():
    lib = _abi.load()
    torch.cuda.set_device(0)
    g = torch.Generator(device="cuda").manual_seed(11)
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    # two calls in a row on different data (the second reuses the scratch the
    # first left behind), including a length that is not a multiple of the
    # 8192-element chunk
    for n in (1_000_003, 4_194_304):
        x = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
        y = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
        got = _noalloc_dot(lib, x, y, out)
        ref = M.dot(x, y)
        scale = float((x.abs() * y.abs()).sum())
        assert abs(got - ref) <= 1e-13 * scale, (n, got, ref)


def test_dot_noalloc_small_and_rejects_oversize():
    lib = _abi.load()
    out = torch.full((1,), 7.0, dtype=torch.float64, device="cuda")
    x = torch.arange(5, dtype=torch.float64, device="cuda")
    assert _noalloc_dot(lib, x, x, out) == 30.0
    # n = 0 writes 0
    st = lib.mfe_dot_noalloc(0, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(x.data_ptr()),
                             ctypes.c_void_p(out.data_ptr()), None)
    assert st == _abi.MFE_OK
    torch.cuda.synchronize()
    assert float(out.item()) == 0.0
    # beyond the scratch's capacity: rejected before any launch
    st = lib.mfe_dot_noalloc(2 ** 29 + 1, ctypes.c_void_p(x.data_ptr()),
                             ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()), None)
    assert st == _abi.MFE_BAD_ARG
    assert np.isfinite(float(out.item()))
