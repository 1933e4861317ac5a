"""Multi-right-hand-side CG (one matrix, nrhs columns advanced together)
against the oracle's single-vector CG run column by column.

Bars: FP64 mode follows the reference's loop per column, so each column's
iteration count is within 2 of the oracle's (dot products are summed in a
different order) and its solution within 1e-8 relative L2 at a 1e-12
relative tolerance (1e-8: two solutions stopped at 1e-12 relative residual
one iteration apart differ by up to cond(A) * 1e-12); mixed mode stops on the TRUE FP64 residual, so
||b_j - A x_j|| / ||b_j|| <= 1e-8 is checked with the oracle's matvec and the
solution is within 1e-6 of the oracle's FP64 solution solved to 1e-12.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import minife_gb300 as M  # noqa: E402


def host(t):
    return t.detach().cpu().numpy()


def rhs_block(b, nrhs, seed):
    """Column 0: the assembled miniFE right-hand side; others: seeded normal."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    B = torch.randn(b.numel(), nrhs, generator=g, dtype=torch.float64)
    B[:, 0] = b.cpu()
    return B.to(b.device).contiguous()


@pytest.mark.parametrize("dims,nrhs", [((10, 10, 10), 4), ((12, 7, 9), 1), ((9, 11, 6), 8),
                                       ((8, 8, 8), 32), ((13, 5, 7), 2)])
def test_multi_f64_matches_oracle_per_column(dims, nrhs):
    A, b = M.build_system(*dims)
    B = rhs_block(b, nrhs, seed=nrhs)
    X = torch.zeros_like(B)
    res = M.cg_solve_multi(A, B, X, max_iter=2000, tol=1e-12, tol_mode="relative",
                           precision="f64")
    ro, cols, vals, _ = O.build_system(*dims)
    Bh, Xh = host(B), host(X)
    for j in range(nrhs):
        xo, it, nr, st = O.cg_solve(ro, cols, vals, Bh[:, j], max_iter=2000, tol=1e-12,
                                    tol_mode=1)
        assert res[j].status == 0
        assert abs(res[j].num_iters - it) <= 2, (j, res[j].num_iters, it)
        rel = np.linalg.norm(Xh[:, j] - xo) / np.linalg.norm(xo)
        assert rel <= 1e-8, (j, rel)
        assert abs(res[j].normr0 - np.linalg.norm(Bh[:, j])) <= 1e-12 * np.linalg.norm(Bh[:, j])


def test_multi_f64_reference_defaults_column0():
    """Column 0 with the reference's defaults (200 iterations, absolute
    DBL_EPSILON) reproduces the single-vector GPU solve."""
    dims = (10, 10, 10)
    A, b = M.build_system(*dims)
    B = rhs_block(b, 4, seed=7)
    X = torch.zeros_like(B)
    res = M.cg_solve_multi(A, B, X, precision="f64")
    x1 = torch.zeros_like(b)
    r1 = M.cg_solve(A, b, x1)
    assert abs(res[0].num_iters - r1.num_iters) <= 2
    assert torch.allclose(X[:, 0], x1, rtol=0, atol=1e-12)


@pytest.mark.parametrize("dims,nrhs,refine_k", [((16, 16, 16), 32, 0), ((20, 14, 9), 8, 10),
                                               ((11, 13, 17), 16, 25)])
def test_multi_mixed_reaches_fp64_tolerance(dims, nrhs, refine_k):
    A, b = M.build_system(*dims)
    B = rhs_block(b, nrhs, seed=3 + nrhs)
    X = torch.zeros_like(B)
    res = M.cg_solve_multi(A, B, X, max_iter=3000, tol=1e-8, tol_mode="relative",
                           precision="mixed", refine_k=refine_k)
    ro, cols, vals, _ = O.build_system(*dims)
    Bh, Xh = host(B), host(X)
    for j in range(nrhs):
        assert res[j].status == 0, (j, res[j])
        rel_res = np.linalg.norm(Bh[:, j] - O.matvec(ro, cols, vals, Xh[:, j])) / \
            np.linalg.norm(Bh[:, j])
        assert rel_res <= 1e-8, (j, rel_res)
        assert abs(res[j].final_resid / res[j].normr0 - rel_res) <= 1e-3 * rel_res + 1e-15
    for j in (0, nrhs - 1):
        xo, it, nr, st = O.cg_solve(ro, cols, vals, Bh[:, j], max_iter=5000, tol=1e-12,
                                    tol_mode=1)
        rel_err = np.linalg.norm(Xh[:, j] - xo) / np.linalg.norm(xo)
        assert rel_err <= 1e-6, (j, rel_err)


def test_multi_inner_tol_and_max_refine():
    A, b = M.build_system(12, 12, 12)
    B = rhs_block(b, 4, seed=2)
    ro, cols, vals, _ = O.build_system(12, 12, 12)
    X = torch.zeros_like(B)
    res = M.cg_solve_multi(A, B, X, max_iter=3000, tol=1e-8, tol_mode="relative",
                           precision="mixed", refine_k=1000, inner_tol=1e-3)
    Bh, Xh = host(B), host(X)
    for j in range(4):
        rel = np.linalg.norm(Bh[:, j] - O.matvec(ro, cols, vals, Xh[:, j])) / \
            np.linalg.norm(Bh[:, j])
        assert res[j].status == 0 and rel <= 1e-8, (j, res[j].status, rel)
    res = M.cg_solve_multi(A, B, torch.zeros_like(B), max_iter=3000, tol=1e-8,
                           tol_mode="relative", precision="mixed", max_refine=1)
    assert all(r.status == 5 and r.refinements == 1 for r in res)
    with pytest.raises(M.MiniFEError) as ei:
        M.cg_solve_multi(A, B, torch.zeros_like(B), tol=1e-8, tol_mode="relative",
                         precision="mixed", max_refine=-2)
    assert ei.value.status == 1


def test_multi_zero_column_and_nonzero_guess():
    """A zero right-hand side with a zero guess is converged at entry (0
    iterations, untouched); a nonzero initial guess is honoured."""
    dims = (9, 9, 9)
    A, b = M.build_system(*dims)
    B = rhs_block(b, 4, seed=11)
    B[:, 2] = 0.0
    X = torch.zeros_like(B)
    g = torch.Generator(device="cpu").manual_seed(5)
    X[:, 3] = torch.randn(b.numel(), generator=g, dtype=torch.float64).to(b.device)
    x3 = X[:, 3].clone()
    res = M.cg_solve_multi(A, B, X, max_iter=1000, tol=1e-10, tol_mode="relative",
                           precision="f64")
    assert res[2].num_iters == 0 and res[2].status == 0
    assert torch.count_nonzero(X[:, 2]).item() == 0
    ro, cols, vals, _ = O.build_system(*dims)
    xo, it, nr, st = O.cg_solve(ro, cols, vals, host(B[:, 3]), x0=host(x3), max_iter=1000,
                                tol=1e-10, tol_mode=1)
    assert abs(res[3].num_iters - it) <= 2
    assert np.linalg.norm(host(X[:, 3]) - xo) <= 1e-9 * np.linalg.norm(xo)


def test_multi_maxiter_and_bad_arguments():
    A, b = M.build_system(12, 12, 12)
    B = rhs_block(b, 4, seed=1)
    X = torch.zeros_like(B)
    res = M.cg_solve_multi(A, B, X, max_iter=3, tol=1e-12, tol_mode="relative",
                           precision="f64")
    assert all(r.status == 5 and r.num_iters == 3 for r in res)
    resm = M.cg_solve_multi(A, B, torch.zeros_like(B), max_iter=3, tol=1e-12,
                            tol_mode="relative", precision="mixed")
    assert all(r.status == 5 for r in resm)
    B3 = rhs_block(b, 3, seed=1)
    with pytest.raises(M.MiniFEError) as ei:
        M.cg_solve_multi(A, B3, torch.zeros_like(B3))
    assert ei.value.status == 1  # MFE_BAD_ARG: nrhs must divide 32


def test_multi_rejects_non_box_matrix():
    A, b = M.build_system(6, 5, 4)
    cols = A.packed_cols.clone()
    cols[40] = cols[41]  # no longer the box's closed-form columns
    A2 = M.CSRMatrix(A.row_offsets, cols, A.packed_coefs, box=(0, 0, 0), max_row_len=27)
    B = rhs_block(b, 2, seed=2)
    with pytest.raises(M.MiniFEError) as ei:
        M.cg_solve_multi(A2, B, torch.zeros_like(B), precision="f64")
    assert ei.value.status == 7  # MFE_NOT_SUPPORTED


@pytest.mark.parametrize("dims,nrhs", [((10, 10, 10), 32), ((17, 3, 5), 8), ((7, 9, 4), 1),
                                       ((12, 11, 10), 3)])
def test_spmm_matches_oracle_per_column(dims, nrhs):
    """Y = A X column by column against the oracle's matvec: the box kernel
    (nrhs dividing 32) and the CSR kernel (nrhs = 3) within the FMA
    reordering bound of a 27-term row sum."""
    A, b = M.build_system(*dims)
    ro, cols, vals, _ = O.build_system(*dims)
    rng = np.random.default_rng(nrhs)
    X = rng.standard_normal((A.nrows, nrhs))
    Y = torch.empty(A.nrows, nrhs, dtype=torch.float64, device=b.device)
    M.spmm(A, torch.from_numpy(X).to(b.device), Y)
    M.default_context().synchronize()
    Yh = host(Y)
    for j in range(nrhs):
        yo = O.matvec(ro, cols, vals, X[:, j])
        bound = 30 * 2.0 ** -53 * O.matvec(ro, cols, np.abs(vals), np.abs(X[:, j])) + 1e-300
        assert np.all(np.abs(Yh[:, j] - yo) <= bound), j


def test_spmm_fp32_box_and_generic_agree():
    dims = (14, 9, 11)
    A, b = M.build_system(*dims)
    A32 = M.to_f32(A)
    X = torch.randn(A.nrows, 16, dtype=torch.float32, device=b.device)
    Y = torch.empty_like(X)
    M.spmm(A32, X, Y)
    Yref = torch.empty(A.nrows, 16, dtype=torch.float64, device=b.device)
    M.spmm(A, X.double().contiguous(), Yref)
    err = (Y.double() - Yref).abs().max().item()
    assert err <= 1e-5 * Yref.abs().max().item()


def test_multi_column_breakdown_is_local():
    """A right-hand side that CG solves exactly in one iteration (a unit
    vector on a Dirichlet row) meets p.Ap = 0 next; FP64 mode stops that
    column alone with the reference's breakdown (one completed iteration),
    mixed mode finishes it on its true residual; the other columns converge
    as usual."""
    dims = (9, 8, 7)
    A, b = M.build_system(*dims)
    B = rhs_block(b, 4, seed=21)
    B[:, 1] = 0.0
    B[0, 1] = 1.0  # row 0 (node (0,0,0)) is a Dirichlet row
    ro, cols, vals, _ = O.build_system(*dims)
    Bh = host(B)
    for prec in ("f64", "mixed"):
        X = torch.zeros_like(B)
        res = M.cg_solve_multi(A, B, X, max_iter=1000, tol=1e-10, tol_mode="relative",
                               precision=prec)
        Xh = host(X)
        assert np.all(np.isfinite(Xh))
        assert np.allclose(Xh[:, 1], Bh[:, 1], rtol=0, atol=1e-15)
        if prec == "f64":
            assert res[1].status == 4 and res[1].num_iters == 1
        else:
            assert res[1].status == 0
        for j in (0, 2, 3):
            assert res[j].status == 0, (prec, j, res[j])
            rel = np.linalg.norm(Bh[:, j] - O.matvec(ro, cols, vals, Xh[:, j])) / \
                np.linalg.norm(Bh[:, j])
            assert rel <= 1e-9, (prec, j, rel)


@pytest.mark.parametrize("dims", [(16, 16, 16), (23, 9, 14), (4, 6, 5)])
def test_multi_mixed_stencil_and_padded_values_agree(dims):
    """32 right-hand sides in mixed precision with the stencil SpMM (the
    verified FP32 stencil) and with the padded FP32 values: both reach the
    1e-8 relative residual checked in FP64 with the oracle's matvec, their
    iteration counts agree within 10 %, and one product of each (two inner
    iterations from x = 0 differ only by the operator's FP32 rounding)
    gives the same solutions to FP32 accuracy."""
    A, b = M.build_system(*dims)
    B = rhs_block(b, 32, seed=41)
    ro, cols, vals, _ = O.build_system(*dims)
    Bh = host(B)
    its = {}
    for op, name in (("auto", "stencil"), ("values", "padded")):
        X = torch.zeros_like(B)
        res = M.cg_solve_multi(A, B, X, max_iter=3000, tol=1e-8, tol_mode="relative",
                               precision="mixed", mixed_operator=op)
        assert all(r.status == 0 for r in res)
        assert res[0].inner_operator == name
        Xh = host(X)
        for j in range(32):
            rel = np.linalg.norm(Bh[:, j] - O.matvec(ro, cols, vals, Xh[:, j])) / np.linalg.norm(Bh[:, j])
            assert rel <= 1e-8, (op, j, rel)
        its[op] = max(r.num_iters for r in res)
        X2 = torch.zeros_like(B)
        M.cg_solve_multi(A, B, X2, max_iter=2, tol=1e-8, tol_mode="relative", precision="mixed",
                         mixed_operator=op, refine_k=1000)
        its[op + "_x2"] = host(X2)
    assert abs(its["auto"] - its["values"]) <= 0.1 * its["values"] + 2
    d = np.abs(its["auto_x2"] - its["values_x2"]).max()
    assert d <= 1e-5 * np.abs(its["values_x2"]).max()
