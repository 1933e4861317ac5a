// The reference's ELLMatrix (ref/src/ELLMatrix.hpp, MINIFE_ELL_MATRIX):
// num_cols_per_row entries per row, row-major (row r at r*num_cols_per_row),
// the row's columns ascending first and then padding entries with column 0
// and coefficient 0 (MatrixInitOp<ELLMatrix>, ref/src/MatrixInitOp.hpp:
// 160-220; the vectors are value-initialised).  Its matvec
// (ref/src/SparseMatrix_functions.hpp:579-611) sums every entry, padding
// included, which adds 0 * x[0].
//
// On the device an ELL matrix is a CSR whose row offsets are r *
// num_cols_per_row, so the CSR kernels (and the CG) run on it unchanged: this
// file converts a CSR into the reference's ELL layout and builds that view.
#include <algorithm>
#include <cstring>

#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

namespace {

template <typename T>
__global__ void k_csr_to_ell(int64_t n, int K, const int32_t* __restrict__ ro,
                             const int32_t* __restrict__ cols, const T* __restrict__ vals,
                             int32_t* __restrict__ ecols, T* __restrict__ evals, unsigned* too_long)
{
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int32_t a = ro[r], len = ro[r + 1] - a;
    if (len > K) {
      atomicOr(too_long, 1u);
      continue;
    }
    int32_t* c = ecols + r * K;
    T* v = evals + r * K;
    for (int k = 0; k < len; ++k) {
      c[k] = cols[a + k];
      v[k] = vals[a + k];
    }
    for (int k = len; k < K; ++k) {
      c[k] = 0;
      v[k] = T(0);
    }
  }
}

__global__ void k_ell_offsets(int64_t n, int K, int32_t* __restrict__ ro)
{
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r <= n;
       r += (int64_t)gridDim.x * blockDim.x)
    ro[r] = (int32_t)(r * K);
}

int grid_for(mfe_ctx* ctx, int64_t n)
{
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n + 1, 256), (int64_t)ctx->sm_count * 8));
}

}  // namespace

mfe_status launch_csr_to_ell(mfe_ctx* ctx, const mfe_csr* A, mfe_ell* E)
{
  unsigned* flag = static_cast<unsigned*>(workspace(ctx, "ell.flag", sizeof(unsigned)));
  if (!flag) return fail(ctx, MFE_OOM, "workspace allocation failed");
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(flag, 0, sizeof(unsigned), ctx->stream));
  const int g = grid_for(ctx, A->nrows);
  if (A->dtype == MFE_F64)
    k_csr_to_ell<double><<<g, 256, 0, ctx->stream>>>(
        A->nrows, E->ncols_per_row, A->row_offsets, A->cols, static_cast<const double*>(A->vals),
        E->cols, static_cast<double*>(E->vals), flag);
  else
    k_csr_to_ell<float><<<g, 256, 0, ctx->stream>>>(
        A->nrows, E->ncols_per_row, A->row_offsets, A->cols, static_cast<const float*>(A->vals),
        E->cols, static_cast<float*>(E->vals), flag);
  MFE_TRY(check_launch(ctx, "k_csr_to_ell"));
  unsigned h = 0;
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(&h, flag, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (h) return fail(ctx, MFE_BAD_ARG, "a row has more entries than ncols_per_row");
  E->nrows = A->nrows;
  E->dtype = A->dtype;
  return MFE_OK;
}

mfe_status ell_view(mfe_ctx* ctx, const mfe_ell* E, mfe_csr* V)
{
  int32_t* ro = static_cast<int32_t*>(workspace(ctx, "ell.ro", sizeof(int32_t) * (size_t)(E->nrows + 1)));
  if (!ro) return fail(ctx, MFE_OOM, "workspace allocation failed");
  // rebuilt on every call: cheap (4 bytes per row) and never stale
  k_ell_offsets<<<grid_for(ctx, E->nrows), 256, 0, ctx->stream>>>(E->nrows, E->ncols_per_row, ro);
  MFE_TRY(check_launch(ctx, "k_ell_offsets"));
  memset(V, 0, sizeof(*V));
  V->nrows = E->nrows;
  V->ncols = E->nrows;
  V->nnz = E->nrows * (int64_t)E->ncols_per_row;
  V->row_offsets = ro;
  V->cols = E->cols;
  V->vals = E->vals;
  V->dtype = E->dtype;
  V->max_row_len = E->ncols_per_row;
  return MFE_OK;
}

}  // namespace mfe
