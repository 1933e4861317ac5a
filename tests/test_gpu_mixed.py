"""Mixed-precision CG (FP32 matrix and vectors, FP64 dots, FP64 reliable
updates) against the FP64 oracle.

Bars: the solver stops only on the TRUE FP64 residual, so ||b - A x|| / ||b||
<= tol is checked here with the oracle's own matvec on the host; the solution
is compared with the oracle's FP64 solution solved to 1e-12 (relative L2 and
max-abs error); the analytic check passes as in the reference.
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


@pytest.mark.parametrize("dims,refine_k", [((30, 30, 30), 0), ((24, 16, 8), 10),
                                           ((40, 30, 20), 50), ((17, 9, 11), 25)])
def test_mixed_reaches_fp64_verified_tolerance(dims, refine_k):
    A, b = M.build_system(*dims)
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=3000, tol=1e-8, tol_mode="relative",
                     precision="mixed", refine_k=refine_k)
    assert res.status == 0
    ro, cols, vals, bo = O.build_system(*dims)
    xg = host(x)
    rel_res = np.linalg.norm(bo - O.matvec(ro, cols, vals, xg)) / np.linalg.norm(bo)
    assert rel_res <= 1e-8, rel_res
    assert abs(res.final_resid / res.normr0 - rel_res) <= 1e-3 * rel_res + 1e-15
    xo, it, nr, st = O.cg_solve(ro, cols, vals, bo, max_iter=5000, tol=1e-12, tol_mode=1)
    rel_err = np.linalg.norm(xg - xo) / np.linalg.norm(xo)
    max_abs = np.abs(xg - xo).max()
    assert rel_err <= 1e-6, rel_err
    assert max_abs <= 1e-6, max_abs
    # iteration count stays close to the FP64 solver's
    x64 = torch.zeros_like(b)
    r64 = M.cg_solve(A, b, x64, max_iter=3000, tol=1e-8, tol_mode="relative")
    assert res.num_iters <= 1.35 * r64.num_iters + 10, (res.num_iters, r64.num_iters)
    rc, err = M.verify_solution(*dims, x)
    rco, erro = O.verify_solution(*dims, xo)
    assert rc == rco and abs(err - erro) <= 1e-5


def test_mixed_max_iter_reports_maxiter():
    A, b = M.build_system(20, 20, 20)
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=5, tol=1e-8, tol_mode="relative", precision="mixed")
    assert res.status == 5  # MFE_MAXITER
    assert res.num_iters == 5
    # the returned x is the reliably updated FP64 iterate: its residual is the
    # one reported
    ro, cols, vals, bo = O.build_system(20, 20, 20)
    r = np.linalg.norm(bo - O.matvec(ro, cols, vals, host(x)))
    assert abs(r - res.final_resid) <= 1e-9 * r


def test_mixed_inner_tol_and_max_refine():
    """inner_tol is the residual drop that makes a reliable update due (0:
    a hundredfold); max_refine caps the updates, after which an unconverged
    solve reports MFE_MAXITER with the reliably updated iterate."""
    A, b = M.build_system(30, 30, 30)
    ro, cols, vals, bo = O.build_system(30, 30, 30)
    updates, iters = {}, {}
    for t in (0.0, 1e-1, 1e-2, 1e-3):
        x = torch.zeros_like(b)
        res = M.cg_solve(A, b, x, max_iter=3000, tol=1e-8, tol_mode="relative",
                         precision="mixed", refine_k=1000, inner_tol=t)
        assert res.status == 0, (t, res.status)
        rel = np.linalg.norm(bo - O.matvec(ro, cols, vals, host(x))) / np.linalg.norm(bo)
        assert rel <= 1e-8, (t, rel)
        updates[t], iters[t] = res.refinements, res.num_iters
    assert updates[1e-3] <= updates[1e-2] <= updates[1e-1], updates
    assert updates[1e-3] < updates[1e-1], updates
    # the default is 1e-2: the same run
    assert (updates[0.0], iters[0.0]) == (updates[1e-2], iters[1e-2])
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=3000, tol=1e-8, tol_mode="relative",
                     precision="mixed", max_refine=2)
    assert res.status == 5 and res.refinements == 2, (res.status, res.refinements)
    r = np.linalg.norm(bo - O.matvec(ro, cols, vals, host(x)))
    assert abs(r - res.final_resid) <= 1e-9 * r
    assert r > 1e-8 * np.linalg.norm(bo)
    for bad in ({"inner_tol": 1.0}, {"inner_tol": -0.5}, {"inner_tol": float("nan")},
                {"max_refine": -1}):
        with pytest.raises(M.MiniFEError) as ei:
            M.cg_solve(A, b, torch.zeros_like(b), tol=1e-8, tol_mode="relative",
                       precision="mixed", **bad)
        assert ei.value.status == 1, bad  # MFE_BAD_ARG


def test_mixed_with_prepared_f32_copy_and_history():
    A, b = M.build_system(16, 16, 16)
    A32 = M.to_f32(A)
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=2000, tol=1e-9, tol_mode="relative", precision="mixed",
                     A32=A32, record_history=True)
    assert res.status == 0 and res.final_resid <= 1e-9 * res.normr0
    assert len(res.history) == res.num_iters + 1
    assert res.refinements >= 1


@pytest.mark.parametrize("dims", [(30, 30, 30), (17, 9, 11), (4, 4, 4), (3, 4, 2), (40, 5, 6),
                                  (11, 6, 7), (14, 8, 4)])
def test_mixed_stencil_operator_and_values_copy(dims):
    """The verified FP32 stencil operator (default on a k = 1 box with an
    interior node, i.e. at least 4 elements along each dimension) and the
    FP32 copy of the values both reach the FP64-verified tolerance with about
    the same number of inner iterations.  The x pitch of the stencil's
    vectors is Nx rounded up to 4: the cases cover padding 0 (11: Nx = 12),
    1, 2 and 3, and nz = 4 (one interior plane)."""
    A, b = M.build_system(*dims)
    ro, cols, vals, bo = O.build_system(*dims)
    its = {}
    for op in ("auto", "values"):
        x = torch.zeros_like(b)
        res = M.cg_solve(A, b, x, max_iter=3000, tol=1e-8, tol_mode="relative", precision="mixed",
                         mixed_operator=op)
        assert res.status == 0, (op, res)
        want = "stencil" if op == "auto" and min(dims) >= 4 else "values"
        assert res.inner_operator == want, (op, res.inner_operator)
        rel = np.linalg.norm(bo - O.matvec(ro, cols, vals, host(x))) / np.linalg.norm(bo)
        assert rel <= 1e-8, (op, rel)
        its[op] = res.num_iters
    assert abs(its["auto"] - its["values"]) <= max(3, 0.1 * its["values"]), its


def test_mixed_stencil_without_mirror_symmetry():
    """A verified stencil that is not mirror-symmetric per axis takes the
    27-coefficient stencil kernel: the (+-1, +-1, 0) entries scaled by 1.001
    keep A symmetric positive definite and every interior row one stencil,
    but coef(1, 1, 0) != coef(1, -1, 0)."""
    dims = (20, 18, 16)
    A, b = M.build_system(*dims)
    N = [d + 1 for d in dims]
    off = N[0] * N[1] + N[0]  # (dz, dy, dx) = (1, 1, 0)
    n = A.nrows
    lens = (A.row_offsets[1:] - A.row_offsets[:-1]).long()
    rows = torch.repeat_interleave(torch.arange(n, device=lens.device), lens)
    d = A.packed_cols.long() - rows
    scale = torch.ones_like(A.packed_coefs)
    scale[(d == off) | (d == -off)] = 1.001
    A.packed_coefs.mul_(scale)
    torch.cuda.synchronize()
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=3000, tol=1e-8, tol_mode="relative", precision="mixed")
    assert res.status == 0 and res.inner_operator == "stencil", (res.status, res.inner_operator)
    ro, cols, vals = host(A.row_offsets), host(A.packed_cols), host(A.packed_coefs)
    bo = host(b)
    rel = np.linalg.norm(bo - O.matvec(ro, cols, vals, host(x))) / np.linalg.norm(bo)
    assert rel <= 1e-8, rel
    xv = torch.zeros_like(b)
    rv = M.cg_solve(A, b, xv, max_iter=3000, tol=1e-8, tol_mode="relative", precision="mixed",
                    mixed_operator="values")
    assert rv.inner_operator == "values"
    assert abs(res.num_iters - rv.num_iters) <= max(3, rv.num_iters // 10)


def test_mixed_stencil_first_iterations_match_values():
    """Two inner iterations from x = 0 with each FP32 operator: the residual
    norms agree to FP32 accuracy, so the stencil applies the same operator as
    the matrix (Dirichlet rows, masked neighbours of rows beside them, z
    boundaries) and not merely one that converges."""
    dims = (13, 6, 9)
    A, b = M.build_system(*dims)
    out = {}
    for op in ("auto", "values"):
        x = torch.zeros_like(b)
        res = M.cg_solve(A, b, x, max_iter=2, tol=0.0, tol_mode="relative", precision="mixed",
                         refine_k=1, mixed_operator=op, record_history=True)
        out[op] = (res, host(x))
    ra, xa = out["auto"]
    rv, xv = out["values"]
    assert ra.inner_operator == "stencil" and rv.inner_operator == "values"
    assert np.abs(xa - xv).max() <= 1e-5 * np.abs(xv).max()
    assert abs(ra.final_resid - rv.final_resid) <= 1e-5 * rv.normr0


def test_mixed_falls_back_for_per_element_conductivity():
    """With random per-element conductivity no class stencil fits the rows, so
    the solver uses the FP32 copy of the values and still converges."""
    dims = (10, 9, 8)
    rng = np.random.default_rng(5)
    kappa = np.exp(rng.normal(0.0, 0.5, size=dims[0] * dims[1] * dims[2]))
    A, b = M.build_system(*dims, kappa=torch.from_numpy(kappa).cuda())
    ro, cols, vals, bo = O.build_system(*dims, kappa=kappa)
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=3000, tol=1e-8, tol_mode="relative", precision="mixed")
    assert res.status == 0 and res.inner_operator == "values"
    rel = np.linalg.norm(bo - O.matvec(ro, cols, vals, host(x))) / np.linalg.norm(bo)
    assert rel <= 1e-8


def test_mixed_stencil_check_rejects_non_finite_values():
    """A NaN in one interior entry fails the stencil check (the row's largest
    magnitude is not finite), so the solver keeps the FP32 values copy."""
    dims = (9, 8, 7)
    A, b = M.build_system(*dims)
    ro, cols, vals, bo = O.build_system(*dims)
    r = ((4 * 9) + 4) * 10 + 5  # an interior node
    A.packed_coefs[int(ro[r]) + 13] = float("nan")
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=3, tol=1e-8, tol_mode="relative", precision="mixed")
    assert res.inner_operator == "values"
