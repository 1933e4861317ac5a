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


def test_batch_inner_tol_and_max_refine():
    dims = [(10, 10, 10), (12, 7, 5), (9, 11, 6)]
    x, off, res = M.batch_solve_boxes(dims, max_iter=3000, tol=1e-8, tol_mode="relative",
                                      precision="mixed", refine_k=1000, inner_tol=1e-3)
    xh = host(x)
    for i, d in enumerate(dims):
        ro, cols, vals, b = O.build_system(*d)
        rel = np.linalg.norm(b - O.matvec(ro, cols, vals, xh[off[i]:off[i + 1]])) / \
            np.linalg.norm(b)
        assert res[i].status == 0 and rel <= 1e-8, (d, res[i].status, rel)
    # one update each (at a tenfold drop): none has converged
    x, off, res = M.batch_solve_boxes(dims, max_iter=3000, tol=1e-8, tol_mode="relative",
                                      precision="mixed", max_refine=1)
    xh = host(x)
    for i, d in enumerate(dims):
        ro, cols, vals, b = O.build_system(*d)
        r = np.linalg.norm(b - O.matvec(ro, cols, vals, xh[off[i]:off[i + 1]]))
        assert res[i].status == 5, (d, res[i].status)
        assert abs(r - res[i].final_resid) <= 1e-9 * r
    with pytest.raises(M.MiniFEError) as ei:
        M.batch_solve_boxes(dims, tol=1e-8, tol_mode="relative", precision="mixed",
                            inner_tol=2.0)
    assert ei.value.status == 1


def test_batch_rejects_bad_dims():
    with pytest.raises(M.MiniFEError) as ei:
        M.batch_solve_boxes([(4, 4, 4), (0, 3, 3)])
    assert ei.value.status == 1


def test_batch_handle_shapes_agree():
    """One assembled batch solved at every launch shape: FP64 results are
    identical up to dot-product order (iterations within 1), and the C entry
    point mfe_batch_solve_boxes gives the handle's answer."""
    import ctypes
    from minife_gb300 import _abi
    dims = [(9, 7, 5), (3, 12, 6), (10, 4, 4)]
    b = M.Batch(dims)
    x0, r0 = b.solve(max_iter=500, tol=1e-10, tol_mode="relative", precision="f64")
    x0 = x0.clone()
    for rows, stages, chunk in [(128, 2, 1024), (128, 4, 4096), (256, 3, 1 << 20)]:
        b.set_tuning(rows, stages, chunk)
        for prec in ("f64", "mixed"):
            x, r = b.solve(max_iter=3000, tol=1e-10, tol_mode="relative", precision=prec)
            assert all(ri.status == 0 for ri in r)
            if prec == "f64":
                assert all(abs(ri.num_iters - rj.num_iters) <= 1 for ri, rj in zip(r, r0))
                assert torch.allclose(x, x0, rtol=0, atol=1e-9)
    assert b.info()[3] == {"spmv_rows": 256, "spmv_stages": 3, "chunk_rows": 1 << 20}
    with pytest.raises(M.MiniFEError):
        b.set_tuning(96, 2, 8192)
    b.close()
    ctx = M.default_context()
    flat = (ctypes.c_int32 * 9)(*[v for d in dims for v in d])
    o, _ = M._opts(500, 1e-10, "relative", "f64")
    res = (_abi.MfeCgResult * 3)()
    xc = torch.empty_like(x0)
    assert ctx.lib.mfe_batch_solve_boxes(ctx.h, 3, flat, ctypes.byref(o), M._ptr(xc), res) == 0
    assert torch.allclose(xc, x0, rtol=0, atol=1e-12)


def test_autotune_small_batch(tmp_path, monkeypatch):
    from minife_gb300 import autotune
    monkeypatch.setenv("MFE_TUNE_CACHE", str(tmp_path / "tune.json"))
    b = M.Batch([(12, 10, 8), (6, 6, 6), (16, 5, 7)])
    cfg = autotune.tune_batch(b, probe_iters=5, reps=1)
    assert (cfg["spmv_rows"], cfg["spmv_stages"]) in autotune.SHAPES
    assert cfg["chunk_rows"] in autotune.CHUNKS and cfg["refine_k"] in autotune.REFINE_K
    x, res = b.solve(max_iter=3000, tol=1e-8, tol_mode="relative", precision="mixed",
                     refine_k=cfg["refine_k"])
    assert all(r.status == 0 for r in res)
    assert autotune.tune_batch(b)["cached"]
    b.close()


def test_batch_tiny_boxes_and_breakdown():
    """Boxes of one to a few elements next to ordinary ones.  1x1x1, 1x1x2 and
    5x3x1 have only Dirichlet rows or nearly: CG solves them exactly in one
    iteration and the next meets p.Ap = 0, where the reference reports a
    breakdown and returns (cg_solve.hpp:186-198; the oracle does the same,
    with one completed iteration and normr 0).  The other boxes are not
    affected."""
    dims = [(1, 1, 1), (1, 1, 2), (5, 3, 1), (2, 2, 2), (6, 7, 8)]
    for prec in ("f64", "mixed"):
        x, off, res = M.batch_solve_boxes(dims, max_iter=500, tol=1e-10, tol_mode="relative",
                                          precision=prec)
        xh = host(x)
        for i, d in enumerate(dims):
            ro, cols, vals, b = O.build_system(*d)
            xo, it, nr, st = O.cg_solve(ro, cols, vals, b, max_iter=500, tol=1e-10, tol_mode=1)
            xi = xh[off[i]:off[i + 1]]
            assert np.all(np.isfinite(xi)), (prec, d)
            rel = np.linalg.norm(b - O.matvec(ro, cols, vals, xi)) / np.linalg.norm(b)
            assert rel <= 1e-9, (prec, d, rel)
            if st == 1:  # the oracle broke down after an exact solve
                assert res[i].status in (0, 4), (prec, d, res[i])
                if prec == "f64":
                    assert res[i].status == 4 and res[i].num_iters == it and res[i].normr == 0.0
            else:
                assert res[i].status == 0, (prec, d, res[i])


def test_batch_stencil_operator_matches_values():
    """Every box with an interior node (>= 4 elements per dimension): the
    batched mixed solver runs the verified FP32 stencil; each box reaches the
    FP64-verified tolerance with about as many iterations as with the padded
    FP32 values.  A batch holding a thinner box falls back to the values."""
    dims = [(4, 5, 6), (10, 10, 10), (12, 7, 5), (9, 11, 6), (16, 4, 4), (20, 13, 17)]
    b = M.Batch(dims)
    out = {}
    for op in ("auto", "values"):
        x, res = b.solve(max_iter=3000, tol=1e-8, tol_mode="relative", precision="mixed",
                         mixed_operator=op)
        out[op] = (host(x).copy(), res)
    b.close()
    xa, ra = out["auto"]
    xv, rv = out["values"]
    off = np.cumsum([0] + [(d[0] + 1) * (d[1] + 1) * (d[2] + 1) for d in dims])
    for i, d in enumerate(dims):
        assert ra[i].inner_operator == "stencil" and rv[i].inner_operator == "padded"
        assert ra[i].status == 0 and rv[i].status == 0, (d, ra[i], rv[i])
        ro, cols, vals, bo = O.build_system(*d)
        for xs in (xa, xv):
            xi = xs[off[i]:off[i + 1]]
            rel = np.linalg.norm(bo - O.matvec(ro, cols, vals, xi)) / np.linalg.norm(bo)
            assert rel <= 1e-8, (d, rel)
        assert abs(ra[i].num_iters - rv[i].num_iters) <= max(3, 0.1 * rv[i].num_iters)
    x, off2, res = M.batch_solve_boxes([(10, 10, 10), (3, 8, 8)], max_iter=3000, tol=1e-8,
                                       tol_mode="relative", precision="mixed")
    assert all(r.inner_operator == "padded" and r.status == 0 for r in res)


def test_batch_96_seeded_boxes_true_residuals():
    """The benchmark's batch (96 boxes, nx, ny, nz ~ U{32..160} seeded as in
    bench.batch_dims) solved together in mixed precision to 1e-8: every box
    converges, and for 12 boxes -- the smallest, the largest and ten drawn
    with a fixed seed -- the true FP64 residual ||b - A x|| / ||b|| computed
    with the oracle's assembly and CSR matvec meets 1e-8 and the reference's
    analytic check passes."""
    import os
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from bench import batch_dims
    dims = batch_dims()
    assert len(dims) == 96
    bt = M.Batch(dims)
    try:
        x, res = bt.solve(max_iter=5000, tol=1e-8, tol_mode="relative", precision="mixed",
                          refine_k=200)
        assert all(r.status == 0 for r in res)
        off = bt.offsets
        xh = host(x)
    finally:
        bt.close()
    del x
    sizes = [d[0] * d[1] * d[2] for d in dims]
    order = np.argsort(sizes)
    pick = {int(order[0]), int(order[-1])}
    pick |= {int(i) for i in np.random.default_rng(96).choice(96, 10, replace=False)}
    assert len(pick) == 12
    for i in sorted(pick):
        d = dims[i]
        ro, cols, vals, b = O.build_system(*d)
        xi = xh[off[i]:off[i + 1]]
        rel = np.linalg.norm(b - O.matvec(ro, cols, vals, xi)) / np.linalg.norm(b)
        assert rel <= 1e-8, (d, rel)
        rc, err = O.verify_solution(*d, xi)
        assert rc == 0, (d, err)
