// The reference's debug dump format (MINIFE_DEBUG): write_matrix
// (ref/src/SparseMatrix_functions.hpp:98-140) and write_vector
// (ref/src/Vector_functions.hpp:49-82), one rank.  The file is
// "<filename>.1.0"; a matrix file holds "nrows nnz" and then one "row col
// coef" line per stored entry in CSR order, a vector file "n" and then one
// "index coef" line per entry; numbers use the default std::ostream format
// (6 significant digits), as the reference writes them.
#include <fstream>
#include <string>
#include <vector>

#include "mfe_internal.h"

using namespace mfe;

namespace {

std::string dump_name(const char* filename) { return std::string(filename) + ".1.0"; }

}  // namespace

extern "C" {

mfe_status mfe_write_matrix(mfe_ctx* ctx, const mfe_csr* A, const char* filename)
{
  if (!ctx) return MFE_BAD_ARG;
  if (!A || !filename || A->nrows < 0 || A->nnz < 0) return fail(ctx, MFE_BAD_ARG, "bad arguments");
  const int64_t n = A->nrows, nnz = A->nnz;
  std::vector<int32_t> ro(n + 1), cols(nnz);
  std::vector<double> vals(nnz);
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(ro.data(), A->row_offsets, sizeof(int32_t) * (n + 1),
                                    cudaMemcpyDeviceToHost, ctx->stream));
  if (nnz > 0) {
    MFE_CUDA_TRY(ctx, cudaMemcpyAsync(cols.data(), A->cols, sizeof(int32_t) * nnz,
                                      cudaMemcpyDeviceToHost, ctx->stream));
    if (A->dtype == MFE_F64) {
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(vals.data(), A->vals, sizeof(double) * nnz,
                                        cudaMemcpyDeviceToHost, ctx->stream));
    } else {
      std::vector<float> v32(nnz);
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(v32.data(), A->vals, sizeof(float) * nnz,
                                        cudaMemcpyDeviceToHost, ctx->stream));
      MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      for (int64_t k = 0; k < nnz; ++k) vals[k] = v32[k];
    }
  }
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  std::ofstream ofs(dump_name(filename).c_str());
  if (!ofs) return fail(ctx, MFE_BAD_ARG, "cannot open the dump file");
  ofs << (size_t)n << " " << (size_t)nnz << std::endl;
  for (int64_t i = 0; i < n; ++i)
    for (int32_t k = ro[i]; k < ro[i + 1]; ++k) ofs << (int)i << " " << cols[k] << " " << vals[k] << std::endl;
  return ofs ? MFE_OK : fail(ctx, MFE_BAD_ARG, "writing the dump file failed");
}

mfe_status mfe_write_vector(mfe_ctx* ctx, int64_t n, const double* x, int64_t start_index,
                            const char* filename)
{
  if (!ctx) return MFE_BAD_ARG;
  if (!filename || n < 0 || (n > 0 && !x)) return fail(ctx, MFE_BAD_ARG, "bad arguments");
  std::vector<double> h(n);
  if (n > 0) {
    MFE_CUDA_TRY(ctx, cudaMemcpyAsync(h.data(), x, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                      ctx->stream));
    MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  std::ofstream ofs(dump_name(filename).c_str());
  if (!ofs) return fail(ctx, MFE_BAD_ARG, "cannot open the dump file");
  ofs << (size_t)n << std::endl;
  for (int64_t i = 0; i < n; ++i) ofs << (int)(start_index + i) << " " << h[i] << std::endl;
  return ofs ? MFE_OK : fail(ctx, MFE_BAD_ARG, "writing the dump file failed");
}

}  // extern "C"
