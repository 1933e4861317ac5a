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


def test_ell_rejects_short_rows():
    A, b = M.build_system(5, 5, 5)
    with pytest.raises(M.MiniFEError) as ei:
        M.ELLMatrix.from_csr(A, 20)
    assert ei.value.status == 1
