// The reference's ELLMatrix (ref/src/ELLMatrix.hpp, MINIFE_ELL_MATRIX):
// num_cols_per_row entries per row, row-major (row r at r*num_cols_per_row),
// the row's columns ascending first and then padding entries with column 0
// and coefficient 0 (MatrixInitOp<ELLMatrix>, ref/src/MatrixInitOp.hpp:
// 160-220; the vectors are value-initialised).  Its matvec
// (ref/src/SparseMatrix_functions.hpp:579-611) sums every entry, padding
// included, which adds 0 * x[0].
//
// On the device an ELL matrix is a CSR whose row offsets are r *
// num_cols_per_row, so the CSR kernels run on it unchanged: this file
// converts a CSR into the reference's ELL layout and builds that view.
//
// Row-major ELL suits a CPU walking one row at a time; on the GPU a warp of
// consecutive rows then reads its entries 8 * num_cols_per_row bytes apart.
// The ELL CG therefore runs on a sliced copy (mfe_sell): rows in slices of
// 32, column-major inside a slice, so entry k of 32 consecutive rows is one
// 256-byte line of values and one 128-byte line of columns, and a lane per
// row sums its row with no staging and no reduction -- one FP64 FMA per
// stored entry, as the ELL matvec.  The copy is made once per solve by a
// shared-memory transpose of each slice (k_ell_to_sell); the FP64 CG makes
// the same copy of any CSR that is not a box matrix (k_csr_to_sell, rows
// padded to the longest).
#include <algorithm>
#include <cstring>

#include "mfe_cgstate.cuh"
#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

namespace {

// CSR -> row-major ELL, a warp per group of 32 rows: the group's output is
// one contiguous range of 32 K entries (and its input one contiguous CSR
// range), so lane l writes entries l, l + 32, ... of the range -- coalesced,
// where a thread per row writes 27 entries 216 bytes apart -- reading each
// row's bounds from shared memory.  Rows longer than K set *too_long (the
// call then fails; their first K entries are written).
constexpr int kCeW = 8;  // warps per block
template <typename T>
__global__ void __launch_bounds__(kCeW * 32)
    k_csr_to_ell(int64_t n, int K, const int32_t* __restrict__ ro, const int32_t* __restrict__ cols,
                 const T* __restrict__ vals, int32_t* __restrict__ ecols, T* __restrict__ evals,
                 unsigned* too_long)
{
  __shared__ int32_t s_a[kCeW][32], s_len[kCeW][32];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int64_t ngroups = (n + 31) / 32;
  for (int64_t g = (int64_t)blockIdx.x * kCeW + w; g < ngroups; g += (int64_t)gridDim.x * kCeW) {
    const int64_t r0 = g * 32;
    const int rows = (int)min((int64_t)32, n - r0);
    int32_t a = 0, len = 0;
    if (lane < rows) {
      a = __ldg(&ro[r0 + lane]);
      len = __ldg(&ro[r0 + lane + 1]) - a;
    }
    if (__any_sync(0xffffffffu, len > K) && lane == 0) atomicOr(too_long, 1u);
    s_a[w][lane] = a;
    s_len[w][lane] = min(len, K);
    __syncwarp();
    const int total = rows * K;
    int32_t* c = ecols + r0 * K;
    T* v = evals + r0 * K;
    for (int e = lane; e < total; e += 32) {
      const int row = e / K, k = e - row * K;
      const bool in = k < s_len[w][row];
      const int64_t src = (int64_t)s_a[w][row] + k;
      c[e] = in ? __ldg(&cols[src]) : 0;
      v[e] = in ? __ldg(&vals[src]) : T(0);
    }
    __syncwarp();  // s_a / s_len are rewritten for the next group
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

constexpr int kSellRows = 32;   // rows per slice
constexpr int kSellKC = 64;     // columns of a slice transposed at a time
constexpr int kSellT = 256;     // threads per block

// one block per slice at a time: the slice's rows [r0, r0 + 32) are one
// contiguous row-major range of the ELL arrays; kSellKC of its columns at a
// time go through shared memory, read coalesced along the rows and written
// coalesced along the slice's column-major order.  Shared rows are kSellLD =
// kSellKC + 1 long: the write-out reads one column of 32 rows, which at an
// even stride would put all 32 lanes on one bank
constexpr int kSellLD = kSellKC + 1;
__global__ void __launch_bounds__(kSellT)
    k_ell_to_sell(int64_t n, int K, const int32_t* __restrict__ ec, const double* __restrict__ ev,
                  int32_t* __restrict__ sc, double* __restrict__ sv)
{
  __shared__ double tv[kSellRows * kSellLD];
  __shared__ int32_t tc[kSellRows * kSellLD];
  const int64_t nslices = (n + kSellRows - 1) / kSellRows;
  for (int64_t sl = blockIdx.x; sl < nslices; sl += gridDim.x) {
    const int64_t r0 = sl * kSellRows;
    const int rows = (int)min((int64_t)kSellRows, n - r0);
    for (int k0 = 0; k0 < K; k0 += kSellKC) {
      const int kc = min(kSellKC, K - k0);
      for (int i = threadIdx.x; i < kSellRows * kc; i += kSellT) {
        const int lr = i / kc, k = i - lr * kc;
        const bool in = lr < rows;
        const int64_t e = (r0 + lr) * K + k0 + k;
        tv[lr * kSellLD + k] = in ? ev[e] : 0.0;
        tc[lr * kSellLD + k] = in ? ec[e] : 0;
      }
      __syncthreads();
      for (int i = threadIdx.x; i < kSellRows * kc; i += kSellT) {
        const int k = i / kSellRows, lr = i - k * kSellRows;
        const int64_t o = (sl * K + k0 + k) * kSellRows + lr;
        sv[o] = tv[lr * kSellLD + k];
        sc[o] = tc[lr * kSellLD + k];
      }
      __syncthreads();
    }
  }
}

// y = A x over a sliced ELL matrix, a warp per slice and a lane per row; DOT:
// x.y into the CG state (p.Ap and the breakdown pre-test) or into dot_out.
// Eight blocks per SM (32 registers): the gathers of x are latency-bound and
// want every resident warp.  The dot's epilogue needs registers the unrolled
// loop would otherwise hold, so the DOT form unrolls two entry pairs (not four) and
// spills nothing (at 256^3 in the FP64 CG: 1.15 ms per iteration, against
// 1.40 ms at 40 registers and six blocks per SM)
template <bool DOT>
__global__ void __launch_bounds__(kSellT, 8)
    k_spmv_sell(int64_t n, int K, const int32_t* __restrict__ sc, const double* __restrict__ sv,
                const double* __restrict__ x, double* __restrict__ y, double* partials,
                unsigned* ticket, CgState* cg, double* dot_out)
{
  __shared__ double red[32];
  const int lane = threadIdx.x & 31;
  const int64_t nslices = (n + kSellRows - 1) / kSellRows;
  const int64_t wstride = (int64_t)gridDim.x * (kSellT / 32);
  double dacc = 0.0;
  for (int64_t sl = (int64_t)blockIdx.x * (kSellT / 32) + (threadIdx.x >> 5); sl < nslices;
       sl += wstride) {
    const int64_t base = sl * K * kSellRows + lane;
    const double* v = sv + base;
    const int32_t* c = sc + base;
    double s0 = 0.0, s1 = 0.0;
    int k = 0;
    constexpr int kUnroll = DOT ? 2 : 4;
#pragma unroll kUnroll
    for (; k + 1 < K; k += 2) {
      s0 = fma(__ldg(v + (int64_t)k * kSellRows), __ldg(x + __ldg(c + (int64_t)k * kSellRows)), s0);
      s1 = fma(__ldg(v + (int64_t)(k + 1) * kSellRows),
               __ldg(x + __ldg(c + (int64_t)(k + 1) * kSellRows)), s1);
    }
    if (k < K) s0 = fma(__ldg(v + (int64_t)k * kSellRows), __ldg(x + __ldg(c + (int64_t)k * kSellRows)), s0);
    const double sum = s0 + s1;
    const int64_t r = sl * kSellRows + lane;
    if (r < n) {
      y[r] = sum;
      if (DOT) dacc = fma(sum, __ldg(x + r), dacc);
    }
  }
  if (!DOT) return;
  const double bt = block_sum(dacc, red);
  double total;
  if (grid_reduce_last(bt, partials, ticket, red, &total) && threadIdx.x == 0) {
    if (cg != nullptr) {
      cg->pAp = total;
      if (total < cg->brkdown_tol) cg->check_pending = 1;
    } else {
      *dot_out = total;
    }
  }
}

// a CSR with rows of at most K entries into the sliced layout, one thread
// per output entry (writes coalesced; each row's entries padded with column
// 0, value 0)
__global__ void __launch_bounds__(kSellT)
    k_csr_to_sell(int64_t n, int K, const int32_t* __restrict__ ro, const int32_t* __restrict__ cols,
                  const double* __restrict__ vals, int32_t* __restrict__ sc, double* __restrict__ sv,
                  int64_t total)
{
  for (int64_t o = (int64_t)blockIdx.x * kSellT + threadIdx.x; o < total;
       o += (int64_t)gridDim.x * kSellT) {
    const int64_t sk = o / kSellRows;  // slice * K + k
    const int lane = (int)(o - sk * kSellRows);
    const int64_t sl = sk / K;
    const int k = (int)(sk - sl * K);
    const int64_t r = sl * kSellRows + lane;
    int32_t c = 0;
    double v = 0.0;
    if (r < n) {
      const int32_t a = __ldg(ro + r), e = __ldg(ro + r + 1);
      if (k < e - a) {
        c = __ldg(cols + a + k);
        v = __ldg(vals + a + k);
      }
    }
    sc[o] = c;
    sv[o] = v;
  }
}

}  // namespace

int64_t sell_entries(int64_t nrows, int K) { return ceil_div(nrows, (int64_t)kSellRows) * kSellRows * K; }

mfe_status launch_csr_to_sell(mfe_ctx* ctx, const mfe_csr* A, int K, mfe_sell* S)
{
  const int64_t total = sell_entries(A->nrows, K);
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(total, (int64_t)kSellT),
                                                            (int64_t)ctx->sm_count * 16));
  k_csr_to_sell<<<g, kSellT, 0, ctx->stream>>>(A->nrows, K, A->row_offsets, A->cols,
                                               static_cast<const double*>(A->vals), S->cols, S->vals,
                                               total);
  MFE_TRY(check_launch(ctx, "k_csr_to_sell"));
  S->nrows = A->nrows;
  S->ncols_per_row = K;
  return MFE_OK;
}

mfe_status launch_ell_to_sell(mfe_ctx* ctx, const mfe_ell* E, mfe_sell* S)
{
  const int64_t nslices = ceil_div(E->nrows, (int64_t)kSellRows);
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(nslices, (int64_t)ctx->sm_count * 8));
  k_ell_to_sell<<<g, kSellT, 0, ctx->stream>>>(E->nrows, E->ncols_per_row, E->cols,
                                               static_cast<const double*>(E->vals), S->cols, S->vals);
  MFE_TRY(check_launch(ctx, "k_ell_to_sell"));
  S->nrows = E->nrows;
  S->ncols_per_row = E->ncols_per_row;
  return MFE_OK;
}

mfe_status launch_spmv_sell(mfe_ctx* ctx, const mfe_sell* S, const double* x, double* y,
                            const DotSink* sink, void* cg_state)
{
  const int64_t nslices = ceil_div(S->nrows, (int64_t)kSellRows);
  CgState* cg = static_cast<CgState*>(cg_state);
  const bool dot = cg != nullptr || (sink != nullptr && sink->out != nullptr);
  const void* k = dot ? (const void*)k_spmv_sell<true> : (const void*)k_spmv_sell<false>;
  const int g = (int)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(nslices, (int64_t)(kSellT / 32)),
                           (int64_t)resident_blocks(ctx, k, kSellT, 0)));
  if (dot) {
    if (!sink || !sink->partials || !sink->ticket)
      return fail(ctx, MFE_BAD_ARG, "sliced ELL SpMV: a dot needs reduction buffers");
    k_spmv_sell<true><<<g, kSellT, 0, ctx->stream>>>(S->nrows, S->ncols_per_row, S->cols, S->vals, x, y,
                                                     sink->partials, sink->ticket, cg,
                                                     cg ? nullptr : sink->out);
  } else {
    k_spmv_sell<false><<<g, kSellT, 0, ctx->stream>>>(S->nrows, S->ncols_per_row, S->cols, S->vals, x, y,
                                                      nullptr, nullptr, nullptr, nullptr);
  }
  return check_launch(ctx, "k_spmv_sell");
}

mfe_status launch_csr_to_ell(mfe_ctx* ctx, const mfe_csr* A, mfe_ell* E)
{
  unsigned* flag = static_cast<unsigned*>(workspace(ctx, "ell.flag", sizeof(unsigned)));
  if (!flag) return fail(ctx, MFE_OOM, "workspace allocation failed");
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(flag, 0, sizeof(unsigned), ctx->stream));
  const int g = (int)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(ceil_div(A->nrows, (int64_t)32), (int64_t)kCeW),
                           (int64_t)ctx->sm_count * 8));
  if (A->dtype == MFE_F64)
    k_csr_to_ell<double><<<g, kCeW * 32, 0, ctx->stream>>>(
        A->nrows, E->ncols_per_row, A->row_offsets, A->cols, static_cast<const double*>(A->vals),
        E->cols, static_cast<double*>(E->vals), flag);
  else
    k_csr_to_ell<float><<<g, kCeW * 32, 0, ctx->stream>>>(
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
