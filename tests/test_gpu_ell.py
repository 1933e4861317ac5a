"""The reference's ELLMatrix layout (ref/src/ELLMatrix.hpp, MatrixInitOp.hpp:
160-220): conversion from the CSR bit for bit against the same conversion of
the oracle's system in numpy, the ELL matvec within the FMA-reordering bound,
and CG on the ELL matrix against the oracle."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import minife_gb300 as M  # noqa: E402


def np_ell(ro, cols, vals, K):
    n = ro.size - 1
    ec = np.zeros(n * K, np.int32)
    ev = np.zeros(n * K, np.float64)
    for i in range(n):
        a, b = ro[i], ro[i + 1]
        ec[i * K:i * K + b - a] = cols[a:b]
        ev[i * K:i * K + b - a] = vals[a:b]
    return ec, ev


@pytest.mark.parametrize("dims", [(4, 5, 6), (10, 10, 10)])
def test_ell_conversion_matvec_cg(dims):
    A, b = M.build_system(*dims)
    E = M.ELLMatrix.from_csr(A, 27)
    ro, cols, vals, bo = O.build_system(*dims)
    ec, ev = np_ell(ro, cols, vals, 27)
    assert np.array_equal(E.cols.cpu().numpy(), ec)
    assert np.array_equal(E.coefs.cpu().numpy(), ev)
    rng = np.random.default_rng(2)
    x = rng.standard_normal(ro.size - 1)
    y = torch.empty_like(b)
    M.matvec_ell(E, torch.from_numpy(x).to(b.device), y)
    yo = O.matvec(ro, cols, vals, x)
    bound = 30 * 2.0 ** -53 * O.matvec(ro, cols, np.abs(vals), np.abs(x)) + 1e-300
    assert np.all(np.abs(y.cpu().numpy() - yo) <= bound)
    xg = torch.zeros_like(b)
    res = M.cg_solve_ell(E, b, xg)
    xo, it, nr, st = O.cg_solve(ro, cols, vals, bo)
    assert abs(res.num_iters - it) <= 2
    assert np.abs(xg.cpu().numpy() - xo).max() <= 1e-12


@pytest.mark.parametrize("K", [27, 30, 64])
def test_ell_conversion_padding(K):
    """The conversion with more columns per row than the longest row (every
    row padded with column 0, value 0) on 210 rows (a partial 32-row group),
    bit for bit against numpy."""
    A, b = M.build_system(4, 5, 6)
    E = M.ELLMatrix.from_csr(A, K)
    ro, cols, vals, bo = O.build_system(4, 5, 6)
    ec, ev = np_ell(ro, cols, vals, K)
    assert np.array_equal(E.cols.cpu().numpy(), ec)
    assert np.array_equal(E.coefs.cpu().numpy(), ev)


def test_ell_rejects_short_rows():
    A, b = M.build_system(5, 5, 5)
    with pytest.raises(M.MiniFEError) as ei:
        M.ELLMatrix.from_csr(A, 20)
    assert ei.value.status == 1


def np_sell(ec, ev, n, K):
    """The sliced layout in numpy: entry k of row r at ((r // 32) * K + k) * 32
    + r % 32, rows past n padded with column 0, value 0."""
    ns = (n + 31) // 32
    sc = np.zeros(ns * 32 * K, np.int32)
    sv = np.zeros(ns * 32 * K, np.float64)
    for r in range(n):
        s, l = divmod(r, 32)
        idx = (s * K + np.arange(K)) * 32 + l
        sc[idx] = ec[r * K:(r + 1) * K]
        sv[idx] = ev[r * K:(r + 1) * K]
    return sc, sv


@pytest.mark.parametrize("dims,K", [((4, 5, 6), 27), ((6, 3, 4), 100)])
def test_sell_layout_and_matvec(dims, K):
    """The sliced copy against its layout built in numpy (a partial last
    slice; K = 100 takes the transpose's column chunks), and its matvec
    within the FMA-reordering bound of the oracle's."""
    A, b = M.build_system(*dims)
    E = M.ELLMatrix.from_csr(A, K)
    S = M.SELLMatrix.from_ell(E)
    ro, cols, vals, bo = O.build_system(*dims)
    n = ro.size - 1
    assert n % 32 != 0
    ec, ev = np_ell(ro, cols, vals, K)
    sc, sv = np_sell(ec, ev, n, K)
    assert np.array_equal(S.cols.cpu().numpy(), sc)
    assert np.array_equal(S.coefs.cpu().numpy(), sv)
    x = np.random.default_rng(4).standard_normal(n)
    y = torch.empty_like(b)
    M.matvec_sell(S, torch.from_numpy(x).to(b.device), y)
    yo = O.matvec(ro, cols, vals, x)
    bound = 30 * 2.0 ** -53 * O.matvec(ro, cols, np.abs(vals), np.abs(x)) + 1e-300
    assert np.all(np.abs(y.cpu().numpy() - yo) <= bound)


def test_ell_cg_relative_and_jacobi():
    """The ELL CG to 1e-10 relative (its iterations on the sliced copy) and
    with the Jacobi preconditioner (the ELL matrix's own products), both
    against the oracle's solution."""
    dims = (12, 9, 10)
    A, b = M.build_system(*dims)
    E = M.ELLMatrix.from_csr(A, 27)
    ro, cols, vals, bo = O.build_system(*dims)
    xo, it, nr, st = O.cg_solve(ro, cols, vals, bo, max_iter=1000, tol=1e-10, tol_mode=1)
    xg = torch.zeros_like(b)
    res = M.cg_solve_ell(E, b, xg, max_iter=1000, tol=1e-10, tol_mode="relative")
    assert res.status == 0 and abs(res.num_iters - it) <= 1
    assert np.linalg.norm(xg.cpu().numpy() - xo) <= 1e-9 * np.linalg.norm(xo)
    xj = torch.zeros_like(b)
    ctx = M.default_context()
    o, _ = M._opts(1000, 1e-10, "relative", "f64", precond="jacobi")
    r = M._abi.MfeCgResult()
    e = E.c()
    st = ctx.lib.mfe_cg_solve_ell(ctx.h, M.ctypes.byref(e), M._ptr(b), M._ptr(xj),
                                  M.ctypes.byref(o), M.ctypes.byref(r))
    assert st == 0
    assert np.linalg.norm(xj.cpu().numpy() - xo) <= 1e-8 * np.linalg.norm(xo)


@pytest.mark.parametrize("dtype", [torch.float64, torch.float32])
@pytest.mark.parametrize("n,K", [(1, 27), (31, 27), (33, 8), (1000, 27), (4099, 27), (4099, 28),
                                 (777, 1), (2049, 64), (513, 65)])
def test_ell_matvec_shapes(n, K, dtype):
    """The row-major ELL product on random rows (columns anywhere, a quarter
    of the entries padding: column 0, value 0) for partial 32-row groups,
    odd and even K, K = 64 (the largest on the warp-staged kernel) and 65
    (through the CSR view), against an FP64 numpy product within the
    reordering bound of the two partial sums per row."""
    rng = np.random.default_rng(n * 131 + K)
    c = rng.integers(0, n, size=(n, K)).astype(np.int32)
    v = rng.standard_normal((n, K))
    pad = rng.random((n, K)) < 0.25
    c[pad] = 0
    v[pad] = 0.0
    if dtype == torch.float32:
        v = v.astype(np.float32).astype(np.float64)
    x = rng.standard_normal(n)
    if dtype == torch.float32:
        x = x.astype(np.float32).astype(np.float64)
    yo = (v * x[c]).sum(axis=1)
    u = 2.0 ** -53 if dtype == torch.float64 else 2.0 ** -24
    bound = (K + 4) * u * (np.abs(v) * np.abs(x[c])).sum(axis=1) + 1e-300
    E = M.ELLMatrix(torch.from_numpy(c.ravel()).cuda(), torch.from_numpy(v.ravel()).to("cuda", dtype), K)
    xd = torch.from_numpy(x).to("cuda", dtype)
    y = torch.full((n,), float("nan"), dtype=dtype, device="cuda")
    M.matvec_ell(E, xd, y)
    assert np.all(np.abs(y.cpu().double().numpy() - yo) <= bound)


def test_ell_matvec_unaligned_arrays():
    """Arrays that do not start on a 16-byte boundary take the CSR view and
    give the same result."""
    n, K = 1000, 27
    rng = np.random.default_rng(5)
    c = rng.integers(0, n, size=n * K).astype(np.int32)
    v = rng.standard_normal(n * K)
    x = rng.standard_normal(n)
    cb = torch.zeros(n * K + 1, dtype=torch.int32, device="cuda")
    vb = torch.zeros(n * K + 1, dtype=torch.float64, device="cuda")
    cb[1:] = torch.from_numpy(c).cuda()
    vb[1:] = torch.from_numpy(v).cuda()
    E1 = M.ELLMatrix(cb[1:], vb[1:], K)
    E0 = M.ELLMatrix(torch.from_numpy(c).cuda(), torch.from_numpy(v).cuda(), K)
    xd = torch.from_numpy(x).cuda()
    y1 = torch.empty(n, dtype=torch.float64, device="cuda")
    y0 = torch.empty_like(y1)
    M.matvec_ell(E1, xd, y1)
    M.matvec_ell(E0, xd, y0)
    yo = (v.reshape(n, K) * x[c.reshape(n, K)]).sum(axis=1)
    bound = (K + 4) * 2.0 ** -53 * (np.abs(v.reshape(n, K)) * np.abs(x[c.reshape(n, K)])).sum(axis=1)
    assert np.all(np.abs(y1.cpu().numpy() - yo) <= bound)
    assert np.all(np.abs(y0.cpu().numpy() - yo) <= bound)
