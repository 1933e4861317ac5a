"""Batched uneven boxes (assembled and solved together) against the oracle
box by box.

Bars: FP64 mode runs the reference's CG per box, so each box's iteration
count is within 2 of the oracle's (dot products are summed in a different
order) and its solution within 1e-8 relative L2 at a 1e-12 relative
tolerance (two solutions stopped one iteration apart differ by up to
cond(A) * 1e-12); mixed mode stops each box on its TRUE FP64 residual, so
||b - A x|| / ||b|| <= 1e-8 is checked with the oracle's matvec, and the
analytic check of the reference passes for every box.
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import minife_gb300 as M  # noqa: E402

DIMS = [(4, 5, 6), (7, 3, 9), (10, 10, 10), (12, 7, 5), (2, 2, 2), (9, 11, 6), (16, 3, 4)]


def host(t):
    return t.detach().cpu().numpy()


def test_batch_f64_matches_oracle_per_box():
    x, off, res = M.batch_solve_boxes(DIMS, max_iter=2000, tol=1e-12, tol_mode="relative",
                                      precision="f64")
    xh = host(x)
    for i, d in enumerate(DIMS):
        ro, cols, vals, b = O.build_system(*d)
        xo, it, nr, st = O.cg_solve(ro, cols, vals, b, max_iter=2000, tol=1e-12, tol_mode=1)
        xi = xh[off[i]:off[i + 1]]
        assert res[i].status == 0, (d, res[i])
        assert abs(res[i].num_iters - it) <= 2, (d, res[i].num_iters, it)
        assert np.linalg.norm(xi - xo) <= 1e-8 * np.linalg.norm(xo), d
        assert abs(res[i].normr0 - np.linalg.norm(b)) <= 1e-12 * np.linalg.norm(b)


def test_batch_f64_reference_defaults():
    """The reference's defaults (200 iterations, absolute DBL_EPSILON) give the
    oracle's iteration counts box by box."""
    dims = [(10, 10, 10), (6, 4, 8)]
    x, off, res = M.batch_solve_boxes(dims, precision="f64")
    xh = host(x)
    for i, d in enumerate(dims):
        ro, cols, vals, b = O.build_system(*d)
        xo, it, nr, st = O.cg_solve(ro, cols, vals, b)
        assert abs(res[i].num_iters - it) <= 2, (d, res[i].num_iters, it)
        assert np.abs(xh[off[i]:off[i + 1]] - xo).max() <= 1e-12


@pytest.mark.parametrize("refine_k", [0, 10])
def test_batch_mixed_reaches_fp64_tolerance(refine_k):
    x, off, res = M.batch_solve_boxes(DIMS, max_iter=3000, tol=1e-8, tol_mode="relative",
                                      precision="mixed", refine_k=refine_k)
    xh = host(x)
    for i, d in enumerate(DIMS):
        ro, cols, vals, b = O.build_system(*d)
        xi = xh[off[i]:off[i + 1]]
        rel = np.linalg.norm(b - O.matvec(ro, cols, vals, xi)) / np.linalg.norm(b)
        assert res[i].status == 0, (d, res[i])
        assert rel <= 1e-8, (d, rel)
        assert abs(res[i].final_resid / res[i].normr0 - rel) <= 1e-3 * rel + 1e-15
        rc, err = O.verify_solution(*d, xi)
        rco, erro = O.verify_solution(*d, O.cg_solve(ro, cols, vals, b, max_iter=5000, tol=1e-12,
                                                       tol_mode=1)[0])
        assert rc == rco and abs(err - erro) <= 1e-5


def test_batch_single_box_and_max_iter():
    x, off, res = M.batch_solve_boxes([(8, 9, 10)], max_iter=4, tol=1e-12, tol_mode="relative",
                                      precision="f64")
    assert res[0].num_iters == 4 and res[0].status == 5
    x, off, res = M.batch_solve_boxes([(8, 9, 10), (3, 3, 3)], max_iter=4, tol=1e-12,
                                      tol_mode="relative", precision="mixed")
    assert all(r.num_iters == 4 and r.status == 5 for r in res)


def test_batch_rejects_bad_dims():
    with pytest.raises(M.MiniFEError) as ei:
        M.batch_solve_boxes([(4, 4, 4), (0, 3, 3)])
    assert ei.value.status == 1
