"""GPU parity at the full 256^3 size (16,974,593 rows, 454,756,609 nonzeros)
against the reference itself: tests/golden/golden_256.json holds the sha256
of every array the unmodified reference (oracle/_ref/ref_harness, built from
ref/src) produced for this box, its CG iteration count and residual to a
1e-8 relative tolerance, and x256_strided.npy every 997th entry of its
solution (tests/golden/gen_golden.py --big 256).

* Assembly (structure, values and right-hand side, before and after the
  Dirichlet passes) must match bit for bit.
* CG: the iteration count to 1e-8 depends on rounding at this size (the
  serial reference takes 427 iterations, the OpenMP reference 99-100 % of
  that on a thread-dependent schedule), so the solve is checked by what
  does not: the true residual ||b - A x|| of the GPU's x computed by the
  oracle's CSR matvec (the reference's arithmetic) must meet 1e-8 ||b||,
  the iteration count must lie within 10 % of the reference's, x must agree
  with the reference's solution at the sampled entries within 1e-5 of
  max|x| (two CG iterates stopped at a 1e-8 residual differ by the
  residual's image under A^-1), and the analytic check must pass as the
  reference's did.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover - CPU-only machines
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import minife_gb300 as M  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
DIMS = (256, 256, 256)
X_TOL = 1e-5       # sampled |x - x_ref| / max|x_ref|
ITER_BAND = 0.10   # iteration count within 10 % of the reference's


@pytest.fixture(scope="module")
def golden():
    with open(os.path.join(HERE, "golden", "golden_256.json")) as f:
        g = json.load(f)
    g["x_samples"] = np.load(os.path.join(HERE, "golden", "x256_strided.npy"))
    return g


def sha(t):
    return hashlib.sha256(t.detach().cpu().numpy().tobytes()).hexdigest()


@pytest.fixture(scope="module")
def system():
    A, b = M.build_system(*DIMS)
    host = (A.row_offsets.cpu().numpy(), A.packed_cols.cpu().numpy(),
            A.packed_coefs.cpu().numpy(), b.cpu().numpy())
    yield A, b, host
    del A, b
    torch.cuda.empty_cache()


def test_256_assembly_hashes(golden, system):
    A, b, _ = system
    assert A.nrows == golden["nrows"] and A.nnz == golden["nnz"]
    h = golden["sha256"]
    assert sha(A.row_offsets) == h["row_offsets"]
    assert sha(A.packed_cols) == h["cols"]
    assert sha(A.packed_coefs) == h["vals"]
    assert sha(b) == h["b"]


def test_256_assembly_before_dirichlet_hashes(golden, system):
    n, _ = M.box_dims(*DIMS)
    A = M.CSRMatrix.empty_box(*DIMS)
    b = torch.empty(n, dtype=torch.float64, device="cuda")
    M.assemble_FE_data(*DIMS, A, b, impose_bc=False)
    assert sha(A.packed_coefs) == golden["sha256"]["vals_prebc"]
    assert sha(b) == golden["sha256"]["b_prebc"]
    del A, b
    torch.cuda.empty_cache()


def check_solution(golden, host, x, res):
    ro, cols, vals, bh = host
    xh = x.cpu().numpy()
    r = bh - O.matvec(ro, cols, vals, xh)
    rel = np.linalg.norm(r) / np.linalg.norm(bh)
    assert rel <= 1e-8, rel
    it_ref = golden["num_iters"]
    assert abs(res.num_iters - it_ref) <= ITER_BAND * it_ref, (res.num_iters, it_ref)
    xs = golden["x_samples"]
    dx = np.abs(xh[::golden["x_stride"]] - xs).max() / np.abs(xs).max()
    assert dx <= X_TOL, dx
    rc, err = M.verify_solution(*DIMS, x)
    assert rc == golden["verify"] == 0, err
    return rel, dx


def test_256_cg_csr_values(golden, system):
    A, b, host = system
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=2000, tol=1e-8, tol_mode="relative", f64_operator="csr")
    assert res.status == 0 and res.inner_operator == "none"
    rel, dx = check_solution(golden, host, x, res)
    print("256^3 CSR CG: %d iterations (reference %d), true rel residual %.3e, "
          "sampled x diff %.2e" % (res.num_iters, golden["num_iters"], rel, dx))


def test_256_cg_stencil64(golden, system):
    A, b, host = system
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=2000, tol=1e-8, tol_mode="relative")
    assert res.status == 0 and res.inner_operator == "stencil64"
    assert res.final_resid <= 1e-8 * res.normr0
    rel, dx = check_solution(golden, host, x, res)
    print("256^3 FP64 stencil CG: %d iterations (reference %d), true rel residual %.3e, "
          "sampled x diff %.2e, %.3f s" % (res.num_iters, golden["num_iters"], rel, dx,
                                           res.total_time))


def test_256_mixed(golden, system):
    A, b, host = system
    x = torch.zeros_like(b)
    res = M.cg_solve(A, b, x, max_iter=5000, tol=1e-8, tol_mode="relative", precision="mixed")
    assert res.status == 0 and res.inner_operator == "stencil"
    ro, cols, vals, bh = host
    xh = x.cpu().numpy()
    rel = np.linalg.norm(bh - O.matvec(ro, cols, vals, xh)) / np.linalg.norm(bh)
    assert rel <= 1e-8, rel
    xs = golden["x_samples"]
    dx = np.abs(xh[::golden["x_stride"]] - xs).max() / np.abs(xs).max()
    assert dx <= X_TOL, dx
    rc, err = M.verify_solution(*DIMS, x)
    assert rc == 0, err
    print("256^3 mixed: %d inner iterations, %d reliable updates, true rel residual %.3e, "
          "sampled x diff %.2e" % (res.num_iters, res.refinements, rel, dx))


def test_256_pcg_ell_generic(golden, system):
    """The solvers beside the hot path at 256^3, each checked by its true
    residual (the oracle's matvec) and against the reference's sampled
    solution: the Jacobi PCG (verified stencil operator: it stops on the
    true residual), the ELL CG iterating on its sliced copy, and the CG of a
    CSR that is not a box matrix (one interior row's columns rotated, the
    same operator; both of these stop on the recursive residual, as the
    reference, so the true one may drift past the tolerance a little)."""
    A, b, host = system
    ro, cols, vals, bh = host
    xs = golden["x_samples"]

    def check(x, slack):
        xh = x.cpu().numpy()
        rel = np.linalg.norm(bh - O.matvec(ro, cols, vals, xh)) / np.linalg.norm(bh)
        assert rel <= slack * 1e-8, rel
        dx = np.abs(xh[::golden["x_stride"]] - xs).max() / np.abs(xs).max()
        assert dx <= X_TOL, dx

    x = torch.zeros_like(b)
    r = M.cg_solve(A, b, x, max_iter=2000, tol=1e-8, tol_mode="relative", precond="jacobi")
    assert r.status == 0 and r.inner_operator == "stencil64"
    check(x, 1.001)

    E = M.ELLMatrix.from_csr(A)
    x = torch.zeros_like(b)
    r = M.cg_solve_ell(E, b, x, max_iter=2000, tol=1e-8, tol_mode="relative")
    assert r.status == 0
    check(x, 2.0)
    del E
    torch.cuda.empty_cache()

    Nx = DIMS[0] + 1
    row = Nx * Nx * (DIMS[2] // 2) + Nx * (DIMS[1] // 2) + DIMS[0] // 2
    a, e = int(ro[row]), int(ro[row + 1])
    gcols = A.packed_cols.clone()
    gvals = A.packed_coefs.clone()
    gcols[a:e] = torch.roll(gcols[a:e], 1)
    gvals[a:e] = torch.roll(gvals[a:e], 1)
    G = M.CSRMatrix(A.row_offsets, gcols, gvals)
    x = torch.zeros_like(b)
    r = M.cg_solve(G, b, x, max_iter=2000, tol=1e-8, tol_mode="relative")
    assert r.status == 0 and r.inner_operator == "none"
    check(x, 2.0)
    del G, gcols, gvals
    torch.cuda.empty_cache()
