"""Adjoint gradient dL/dkappa of the box solve (per-element conductivity).

Checked two ways, as the differentiation pattern requires:
  * against an FP64 reference gradient computed on the CPU with the oracle
    (assembly with kappa, FP64 CG forward and adjoint solves, element
    contraction) -- relative agreement 1e-8 of the largest component;
  * against central finite differences (h = 1e-6) of L = 0.5 ||u - u_target||^2
    on seeded random elements -- relative agreement 1e-4 of the largest
    component (FD truncation and the solves' rounding floor).
kappa = exp(g), g ~ N(0, 0.5^2) i.i.d. per element; u_target is the solve at
kappa * exp(N(0, 0.05^2)) (seeds S, S+1, elements drawn with S+2).
"""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():  # pragma: no cover
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import minife_gb300 as M  # noqa: E402
from minife_gb300 import adjoint  # noqa: E402

SEED = 1234


def setup_problem(dims, seed=SEED):
    E = dims[0] * dims[1] * dims[2]
    rng = np.random.default_rng(seed)
    g = rng.normal(0.0, 0.5, size=E)
    kappa = np.exp(g)
    rng1 = np.random.default_rng(seed + 1)
    kappa_t = kappa * np.exp(rng1.normal(0.0, 0.05, size=E))
    return kappa, kappa_t


def oracle_gradient(dims, kappa, u_target):
    ro, cols, vals, b = O.build_system(*dims, kappa=kappa)
    u, it, nr, st = O.cg_solve(ro, cols, vals, b, max_iter=20000, tol=1e-14, tol_mode=1)
    m0, m1 = O.bc_masks(*dims)
    rhs = u - u_target
    rhs[(m0 | m1).astype(bool)] = 0.0
    lam, it, nr, st = O.cg_solve(ro, cols, vals, rhs, max_iter=20000, tol=1e-14, tol_mode=1)
    return O.element_gradient(*dims, u, lam), u


def gpu_target(dims, kappa_t):
    with torch.no_grad():
        return adjoint.solve(torch.from_numpy(kappa_t).cuda(), dims, tol=1e-13)


@pytest.mark.parametrize("dims", [(8, 7, 6), (12, 10, 9)])
def test_adjoint_matches_fp64_reference_gradient(dims):
    kappa, kappa_t = setup_problem(dims)
    ut = gpu_target(dims, kappa_t)
    k = torch.from_numpy(kappa).cuda().requires_grad_(True)
    u = adjoint.solve(k, dims, tol=1e-13)
    loss = adjoint.loss_l2(u, ut)
    loss.backward()
    g_gpu = k.grad.detach().cpu().numpy()
    g_ref, u_ref = oracle_gradient(dims, kappa, ut.cpu().numpy())
    assert np.linalg.norm(u.detach().cpu().numpy() - u_ref) <= 1e-10 * np.linalg.norm(u_ref)
    scale = np.abs(g_ref).max()
    assert scale > 0
    assert np.abs(g_gpu - g_ref).max() <= 1e-8 * scale


def test_element_contraction_bitexact_with_oracle():
    dims = (6, 5, 4)
    rng = np.random.default_rng(3)
    n, _ = M.box_dims(*dims)
    u = rng.standard_normal(n)
    lam = rng.standard_normal(n)
    g = M.element_gradient(*dims, torch.from_numpy(u).cuda(), torch.from_numpy(lam).cuda())
    go = O.element_gradient(*dims, u, lam)
    assert np.array_equal(g.cpu().numpy().view(np.int64), go.view(np.int64))


@pytest.mark.parametrize("dims,nfd", [((16, 16, 16), 16), ((128, 128, 128), 16)])
def test_adjoint_matches_central_differences(dims, nfd):
    kappa, kappa_t = setup_problem(dims)
    ut = gpu_target(dims, kappa_t)
    k = torch.from_numpy(kappa).cuda().requires_grad_(True)
    u = adjoint.solve(k, dims, tol=1e-12)
    adjoint.loss_l2(u, ut).backward()
    g = k.grad.detach().cpu().numpy()
    E = kappa.size
    elems = np.random.default_rng(SEED + 2).choice(E, size=nfd, replace=False)
    fd = adjoint.finite_difference(torch.from_numpy(kappa).cuda(), dims, ut, elems,
                                   h=1e-6, tol=1e-10).numpy()
    scale = np.abs(g).max()
    err = np.abs(fd - g[elems]).max()
    assert err <= 1e-4 * scale, (err, scale, fd[:4], g[elems][:4])


@pytest.mark.parametrize("dims", [(8, 7, 6), (12, 10, 9)])
def test_native_adjoint_grad_matches_oracle_and_autograd(dims):
    """mfe_adjoint_grad (forward solve, adjoint solve and contraction in one C
    call) against the oracle's FP64 gradient and the autograd path."""
    kappa, kappa_t = setup_problem(dims)
    ut = gpu_target(dims, kappa_t)
    k = torch.from_numpy(kappa).cuda()
    loss, g, u = adjoint.grad_l2(k, dims, ut, tol=1e-13)
    g_ref, u_ref = oracle_gradient(dims, kappa, ut.cpu().numpy())
    assert np.linalg.norm(u.cpu().numpy() - u_ref) <= 1e-10 * np.linalg.norm(u_ref)
    assert abs(loss - 0.5 * float(np.sum((u_ref - ut.cpu().numpy()) ** 2))) <= 1e-9 * loss
    scale = np.abs(g_ref).max()
    assert np.abs(g.cpu().numpy() - g_ref).max() <= 1e-8 * scale
    ka = k.clone().requires_grad_(True)
    la = adjoint.loss_l2(adjoint.solve(ka, dims, tol=1e-13), ut)
    la.backward()
    assert np.abs(ka.grad.cpu().numpy() - g.cpu().numpy()).max() <= 1e-9 * scale
