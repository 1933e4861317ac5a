// Adjoint gradient in one call: L = 1/2 ||u - u_target||^2 (all nodes), u the
// solution of the miniFE box problem with per-element conductivity kappa
// (the extension of ref/fem/Hex8.hpp:273, k = 1.0 there), differentiated
// with respect to kappa:
//
//   A(kappa) u = b(kappa)                       forward assembly + CG
//   A lambda = (u - u_target), lambda_D = 0     adjoint CG (A is symmetric)
//   dL/dkappa_e = -lambda_e^T Khat_e u_e        element contraction
//
// (the Dirichlet lifting's kappa dependence enters through u_e's boundary
// values).  The same steps as minife_gb300.adjoint.BoxSolve, on the device
// and behind the C ABI.
#include <algorithm>
#include <cstring>

#include "mfe_internal.h"

namespace mfe {

mfe_status adjoint_grad(mfe_ctx* ctx, int nx, int ny, int nz, const double* kappa,
                        const double* u_target, const mfe_cg_opts* o, double* u_out,
                        double* grad, double* loss, mfe_cg_result* fwd, mfe_cg_result* adj)
{
  int64_t n = 0, nnz = 0;
  MFE_TRY(mfe_box_dims(nx, ny, nz, &n, &nnz));
  mfe_csr A;
  memset(&A, 0, sizeof(A));
  A.nrows = n;
  A.ncols = n;
  A.nnz = nnz;
  A.dtype = MFE_F64;
  A.max_row_len = 27;
  A.box_nx = nx;
  A.box_ny = ny;
  A.box_nz = nz;
  A.row_offsets = static_cast<int32_t*>(workspace(ctx, "adj.ro", sizeof(int32_t) * (size_t)(n + 1)));
  A.cols = static_cast<int32_t*>(workspace(ctx, "adj.cols", sizeof(int32_t) * (size_t)(nnz + 4)));
  A.vals = workspace(ctx, "adj.vals", sizeof(double) * (size_t)(nnz + 4));
  const size_t vb = sizeof(double) * (size_t)(n + 4);
  double* b = static_cast<double*>(workspace(ctx, "adj.b", vb));
  double* u = u_out ? u_out : static_cast<double*>(workspace(ctx, "adj.u", vb));
  double* rhs = static_cast<double*>(workspace(ctx, "adj.rhs", vb));
  double* lam = static_cast<double*>(workspace(ctx, "adj.lambda", vb));
  double* dscal = static_cast<double*>(workspace(ctx, "adj.scalar", sizeof(double) * 2));
  if (!A.row_offsets || !A.cols || !A.vals || !b || !u || !rhs || !lam || !dscal)
    return fail(ctx, MFE_OOM, "adjoint workspace allocation failed");
  MFE_TRY(launch_structure(ctx, nx, ny, nz, A.row_offsets, A.cols));
  MFE_TRY(launch_assemble(ctx, nx, ny, nz, kappa, A.row_offsets, static_cast<double*>(A.vals), b, 1));

  mfe_cg_result rf, ra;
  memset(&rf, 0, sizeof(rf));
  memset(&ra, 0, sizeof(ra));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(u, 0, sizeof(double) * (size_t)n, ctx->stream));
  mfe_status st = cg_solve_impl(ctx, &A, b, u, o, &rf);
  rf.status = st;
  if (fwd) *fwd = rf;
  if (st != MFE_OK) return fail(ctx, st, "forward CG did not converge");

  // dL/du = u - u_target; L = 1/2 of its squared norm (all nodes)
  MFE_TRY(launch_waxpby(ctx, n, 1.0, u, -1.0, u_target, rhs));
  MFE_TRY(launch_dot(ctx, n, rhs, rhs, dscal));
  double hl = 0.0;
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(&hl, dscal, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (loss) *loss = 0.5 * hl;

  // adjoint: lambda = 0 on the Dirichlet rows
  MFE_TRY(launch_zero_boundary(ctx, nx, ny, nz, rhs));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(lam, 0, sizeof(double) * (size_t)n, ctx->stream));
  MFE_TRY(launch_dot(ctx, n, rhs, rhs, dscal));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(&hl, dscal, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (hl > 0.0) {
    st = cg_solve_impl(ctx, &A, rhs, lam, o, &ra);
    ra.status = st;
    if (adj) *adj = ra;
    if (st != MFE_OK) return fail(ctx, st, "adjoint CG did not converge");
  } else if (adj) {
    *adj = ra;
  }
  return launch_element_gradient(ctx, nx, ny, nz, u, lam, grad);
}

}  // namespace mfe
