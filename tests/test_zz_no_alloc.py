"""GPU test of mfe_dot_noalloc, the allocation-free dot product.

Callers that may not allocate device memory (their GPU memory belongs to
another allocator, or they cannot afford cudaMalloc's synchronisation) use
this entry point: it needs no context and keeps its partial sums in a device
array inside the library.  The test calls it through the C ABI and checks two
consecutive calls against the oracle's FP64 dot (the reference's sequential
sum) and the context-based mfe_dot, with the tolerance the other dot tests
use, also back to back on one non-default stream with no synchronisation
between the calls.  The file is named so pytest collects it last; it passes
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
from oracle import oracle as O  # noqa: E402


def _launch(lib, x, y, out, stream=None):
    s = torch.cuda.current_stream() if stream is None else stream
    st = lib.mfe_dot_noalloc(x.numel(), ctypes.c_void_p(x.data_ptr()),
                             ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                             ctypes.c_void_p(s.cuda_stream))
    assert st == _abi.MFE_OK


def _noalloc_dot(lib, x, y, out):
    _launch(lib, x, y, out)
    torch.cuda.synchronize()
    return float(out.item())


def _check(got, x, y):
    """Against the oracle's FP64 dot of the host copies, and the library's
    context-based dot, within 1e-13 of sum |x_i y_i|."""
    xh, yh = x.cpu().numpy(), y.cpu().numpy()
    scale = float(np.abs(xh) @ np.abs(yh))
    ref = O.dot(xh, yh)
    assert abs(got - ref) <= 1e-13 * scale, (x.numel(), got, ref)
    assert abs(got - M.dot(x, y)) <= 1e-13 * scale


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
        _check(_noalloc_dot(lib, x, y, out), x, y)


def test_dot_noalloc_back_to_back_on_one_stream():
    """Two calls queued on one non-default stream with no synchronisation
    between them: stream order keeps them from racing on the shared scratch,
    and each result lands in its own output."""
    lib = _abi.load()
    g = torch.Generator(device="cuda").manual_seed(12)
    s = torch.cuda.Stream()
    xs = [torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
          for n in (3_000_001, 8192)]
    ys = [torch.randn_like(x) for x in xs]
    outs = [torch.empty(1, dtype=torch.float64, device="cuda") for _ in xs]
    torch.cuda.synchronize()
    for x, y, out in zip(xs, ys, outs):
        _launch(lib, x, y, out, stream=s)
    s.synchronize()
    for x, y, out in zip(xs, ys, outs):
        _check(float(out.item()), x, y)


@pytest.mark.skipif(torch.cuda.device_count() < 2, reason="needs a second GPU")
def test_dot_noalloc_second_device():
    """The per-device scratch address on another device."""
    lib = _abi.load()
    with torch.cuda.device(1):
        x = torch.randn(100_003, dtype=torch.float64, device="cuda:1")
        y = torch.randn_like(x)
        out = torch.empty(1, dtype=torch.float64, device="cuda:1")
        _launch(lib, x, y, out)
        torch.cuda.synchronize(1)
        xh, yh = x.cpu().numpy(), y.cpu().numpy()
        assert abs(float(out.item()) - O.dot(xh, yh)) <= 1e-13 * float(np.abs(xh) @ np.abs(yh))


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
