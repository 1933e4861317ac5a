"""Jacobi-preconditioned CG against the same algorithm in numpy on the
oracle's system (FP64): iteration count within 1, solution within 1e-10
relative, true residual at the tolerance; fewer iterations than plain CG on
miniFE's matrix (its Dirichlet rows carry 1 on the diagonal, the interior
rows about 8h/3)."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import minife_gb300 as M  # noqa: E402


def csr_matvec(ro, cols, vals, x):
    return O.matvec(ro, cols, vals, x)


def jacobi_pcg(ro, cols, vals, b, tol, max_iter):
    n = b.size
    d = np.ones(n)
    for i in range(n):
        for k in range(ro[i], ro[i + 1]):
            if cols[k] == i and vals[k] != 0.0:
                d[i] = vals[k]
    x = np.zeros(n)
    r = b.copy()
    z = r / d
    p = z.copy()
    rz = r @ z
    tol_abs = tol * np.linalg.norm(r)
    k = 0
    while k < max_iter and np.linalg.norm(r) > tol_abs:
        Ap = csr_matvec(ro, cols, vals, p)
        alpha = rz / (p @ Ap)
        x += alpha * p
        r -= alpha * Ap
        z = r / d
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
        k += 1
    return x, k


@pytest.mark.parametrize("dims", [(10, 10, 10), (17, 9, 6), (24, 20, 16)])
def test_jacobi_pcg_matches_numpy(dims):
    A, b = M.build_system(*dims)
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=5000, tol=1e-10, tol_mode="relative", precond="jacobi")
    assert res.status == 0
    ro, cols, vals, bo = O.build_system(*dims)
    xo, ko = jacobi_pcg(ro, cols, vals, bo, 1e-10, 5000)
    assert abs(res.num_iters - ko) <= 1, (res.num_iters, ko)
    xg = x.cpu().numpy()
    assert np.linalg.norm(xg - xo) <= 1e-10 * np.linalg.norm(xo) * 100
    rel = np.linalg.norm(bo - csr_matvec(ro, cols, vals, xg)) / np.linalg.norm(bo)
    assert rel <= 1.01e-10
    xp = torch.zeros_like(b)
    plain = M.cg_solve(A, b, xp, max_iter=5000, tol=1e-10, tol_mode="relative")
    assert res.num_iters < plain.num_iters


def test_jacobi_pcg_generic_csr_and_errors():
    """A CSR without box dimensions (generic SpMV) and the option checks."""
    dims = (9, 8, 7)
    A, b = M.build_system(*dims)
    G = M.CSRMatrix(A.row_offsets, A.packed_cols, A.packed_coefs, box=(0, 0, 0), max_row_len=27)
    x1, x2 = torch.zeros_like(b), torch.zeros_like(b)
    r1 = M.cg_solve(A, b, x1, max_iter=2000, tol=1e-10, tol_mode="relative", precond="jacobi")
    r2 = M.cg_solve(G, b, x2, max_iter=2000, tol=1e-10, tol_mode="relative", precond="jacobi")
    assert abs(r1.num_iters - r2.num_iters) <= 1
    assert torch.allclose(x1, x2, rtol=0, atol=1e-9)
    with pytest.raises(M.MiniFEError):
        M.cg_solve(A, b, torch.zeros_like(b), precision="mixed", precond="jacobi",
                   allow_breakdown=False)
    r3 = M.cg_solve(A, b, torch.zeros_like(b), max_iter=3, tol=1e-12, tol_mode="relative",
                    precond="jacobi")
    assert r3.num_iters == 3 and r3.status == 5
