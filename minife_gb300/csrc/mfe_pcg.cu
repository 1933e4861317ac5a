// Jacobi-preconditioned CG (FP64): the preconditioned form of the
// reference's cg_solve (ref/src/cg_solve.hpp:69-229) with M = diag(A):
//
//   r = b - A x, z = M^-1 r, p = z, rz = r.z
//   loop: Ap = A p, alpha = rz / p.Ap, x += alpha p, r -= alpha Ap,
//         z = M^-1 r, rz' = r.z, beta = rz' / rz, p = z + beta p
//
// stopping on ||r|| (absolute, or relative to ||r0||) after the update, at
// most max_iter iterations.  Kernels: the SpMV of the unpreconditioned solver
// (box-structured or generic, with p.Ap fused -- or, for a verified miniFE box
// operator and a tolerance of at least 2^-36 of the initial residual, the
// FP64 stencil operator, the solve then stopping only once ||b - A x|| with
// the CSR values meets the tolerance, restarting from that residual
// otherwise, as the unpreconditioned solver), one update kernel that also
// applies M^-1 and reduces r.z and r.r, one p update; the loop is a CUDA graph
// with a conditional while node, as for the other solvers.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

namespace {

constexpr int kPT = 256;
constexpr int kPMaxBlocks = 2048;
constexpr int kPMaxSpmvPartials = 8192;

struct PcgState {
  double rz, rr, pAp, beta, normr, normr0, tol_abs;
  int k, max_iter, cont, status;
  unsigned err;
};

// dinv[r] = 1 / A[r, r] (1 when the row has no nonzero diagonal)
__global__ void k_diag_inv(int64_t n, const int32_t* __restrict__ ro, const int32_t* __restrict__ cols,
                           const double* __restrict__ vals, double* __restrict__ dinv)
{
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n;
       r += (int64_t)gridDim.x * blockDim.x) {
    double d = 0.0;
    for (int32_t k = ro[r]; k < ro[r + 1]; ++k)
      if (cols[k] == r) d = vals[k];
    dinv[r] = d != 0.0 ? 1.0 / d : 1.0;
  }
}

// Two dots at once: the block sums of (a, b) go to partials[2*block], the last
// block sums them in block order.  Returns true in thread 0 of the last block.
__device__ bool two_dot_last(double a, double b, double* partials, unsigned* ticket, double* red,
                             double* ta, double* tb)
{
  __shared__ bool last;
  const double sa = block_sum(a, red);
  const double sb = block_sum(b, red + 32);
  if (threadIdx.x == 0) {
    partials[2 * blockIdx.x] = sa;
    partials[2 * blockIdx.x + 1] = sb;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  double ua = 0.0, ub = 0.0;
  for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
    ua += __ldcg(&partials[2 * i]);
    ub += __ldcg(&partials[2 * i + 1]);
  }
  ua = block_sum(ua, red);
  ub = block_sum(ub, red + 32);
  if (threadIdx.x == 0) {
    *ta = ua;
    *tb = ub;
    *ticket = 0u;
  }
  return threadIdx.x == 0;
}

// z = M^-1 r, p = z, rz = r.z, rr = r.r (after the initial residual, or
// after a true residual to restart from: restart keeps k and normr0)
__global__ void __launch_bounds__(kPT)
    k_pcg_init(int64_t n, const double* __restrict__ r, const double* __restrict__ dinv,
               double* __restrict__ z, double* __restrict__ p, PcgState* st, double* partials,
               unsigned* ticket, int restart)
{
  __shared__ double red[64];
  double a = 0.0, c = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kPT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kPT) {
    const double zi = dinv[i] * r[i];
    z[i] = zi;
    p[i] = zi;
    a = fma(r[i], zi, a);
    c = fma(r[i], r[i], c);
  }
  double rz, rr;
  if (two_dot_last(a, c, partials, ticket, red, &rz, &rr)) {
    st->rz = rz;
    st->rr = rr;
    st->normr = sqrt(rr);
    if (!restart) {
      st->normr0 = st->normr;
      st->k = 0;
    }
    st->cont = st->k < st->max_iter && st->normr > st->tol_abs;
  }
}

// x += alpha p, r -= alpha Ap, z = M^-1 r, then rz', rr; the last block
// decides whether the loop goes on and forms beta
__global__ void __launch_bounds__(kPT)
    k_pcg_update(int64_t n, double* __restrict__ x, double* __restrict__ r, double* __restrict__ z,
                 const double* __restrict__ p, const double* __restrict__ Ap,
                 const double* __restrict__ dinv, PcgState* st, double* partials, unsigned* ticket,
                 cudaGraphConditionalHandle h, int in_graph)
{
  __shared__ double red[64];
  const double pAp = st->pAp;
  const double alpha = pAp > 0.0 ? st->rz / pAp : 0.0;
  double a = 0.0, c = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kPT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kPT) {
    x[i] = fma(alpha, p[i], x[i]);
    const double ri = fma(-alpha, Ap[i], r[i]);
    r[i] = ri;
    const double zi = dinv[i] * ri;
    z[i] = zi;
    a = fma(ri, zi, a);
    c = fma(ri, ri, c);
  }
  double rz, rr;
  if (two_dot_last(a, c, partials, ticket, red, &rz, &rr)) {
    st->k += 1;
    st->rr = rr;
    st->normr = sqrt(rr);
    if (!(pAp > 0.0)) st->status = MFE_BREAKDOWN;
    st->beta = st->rz > 0.0 ? rz / st->rz : 0.0;
    st->rz = rz;
    st->cont = st->status == 0 && st->k < st->max_iter && st->normr > st->tol_abs;
    if (in_graph) cudaGraphSetConditional(h, st->cont ? 1u : 0u);
  }
}

__global__ void __launch_bounds__(kPT)
    k_pcg_p(int64_t n, const double* __restrict__ z, double* __restrict__ p, const PcgState* st)
{
  const double beta = st->beta;
  for (int64_t i = (int64_t)blockIdx.x * kPT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kPT)
    p[i] = fma(beta, p[i], z[i]);
}

__global__ void k_pcg_begin(const PcgState* st, cudaGraphConditionalHandle h)
{
  cudaGraphSetConditional(h, st->cont ? 1u : 0u);
}

}  // namespace

mfe_status cg_jacobi(mfe_ctx* ctx, const mfe_csr* A, const double* b, double* x,
                     const mfe_cg_opts* o, mfe_cg_result* res)
{
  if (o->precision != MFE_PREC_F64)
    return fail(ctx, MFE_NOT_SUPPORTED, "the Jacobi-preconditioned solver runs in FP64");
  const int64_t n = A->nrows;
  const size_t vb = sizeof(double) * (size_t)(n + 8);
  double* r = static_cast<double*>(workspace(ctx, "pcg.r", vb));
  double* z = static_cast<double*>(workspace(ctx, "pcg.z", vb));
  double* p = static_cast<double*>(workspace(ctx, "pcg.p", vb));
  double* Ap = static_cast<double*>(workspace(ctx, "pcg.Ap", vb));
  double* dinv = static_cast<double*>(workspace(ctx, "pcg.dinv", vb));
  PcgState* st = static_cast<PcgState*>(workspace(ctx, "pcg.state", sizeof(PcgState)));
  double* partials = static_cast<double*>(workspace(ctx, "pcg.partials", sizeof(double) * 2 * kPMaxBlocks));
  double* spart = static_cast<double*>(workspace(ctx, "pcg.spmv_partials", sizeof(double) * kPMaxSpmvPartials));
  const bool fresh = ctx->ws.find("pcg.tickets") == ctx->ws.end();
  unsigned* tickets = static_cast<unsigned*>(workspace(ctx, "pcg.tickets", sizeof(unsigned) * 4));
  if (!r || !z || !p || !Ap || !dinv || !st || !partials || !spart || !tickets)
    return fail(ctx, MFE_OOM, "PCG workspace allocation failed");
  if (spmv_grid(ctx, A) > kPMaxSpmvPartials) return fail(ctx, MFE_NOT_SUPPORTED, "matrix too large");
  bool st64 = false;
  double w8[8] = {}, dd = 0.0;
  if (fresh) MFE_CUDA_TRY(ctx, cudaMemsetAsync(tickets, 0, sizeof(unsigned) * 4, ctx->stream));

  // pinned scratch sized once for the stencil check's class table too, so
  // it is not reallocated under hs
  PcgState* hs = static_cast<PcgState*>(host_scratch(ctx, 32768));
  if (!hs) return fail(ctx, MFE_OOM, "pinned scratch allocation failed");
  memset(hs, 0, sizeof(PcgState));
  hs->max_iter = o->max_iter;
  hs->tol_abs = o->tol;
  const int vg = (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(n, kPT),
                                                              std::min(ctx->sm_count * 8, kPMaxBlocks)));
  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(st, hs, sizeof(PcgState), cudaMemcpyHostToDevice, ctx->stream));
  k_diag_inv<<<vg, kPT, 0, ctx->stream>>>(n, A->row_offsets, A->cols,
                                         static_cast<const double*>(A->vals), dinv);
  MFE_TRY(check_launch(ctx, "k_diag_inv"));
  // r = b - A x0
  DotSink rs{spart, tickets + 2, &st->rr};
  MFE_TRY(launch_spmv(ctx, A, x, r, &rs, b, nullptr));
  int csr_products = 1;
  double tol_abs = o->tol;
  const bool try_st64 = o->f64_operator == 0 && csr_is_box(A) && A->dtype == MFE_F64;
  if (o->tol_mode == MFE_TOL_RELATIVE || try_st64) {
    MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    double rr0 = 0.0;
    MFE_CUDA_TRY(ctx, cudaMemcpy(&rr0, &st->rr, sizeof(double), cudaMemcpyDeviceToHost));
    if (o->tol_mode == MFE_TOL_RELATIVE) {
      // tol_abs = tol * ||r0|| (the initial kernel reads rr written just above)
      tol_abs = o->tol * sqrt(rr0);
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(&st->tol_abs, &tol_abs, sizeof(double), cudaMemcpyHostToDevice,
                                        ctx->stream));
      MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    // the verified FP64 stencil operator: tolerances below 2^-36 of the
    // initial residual would meet its rounding-level difference from A
    bool ok = false;
    if (try_st64 && tol_abs >= std::ldexp(sqrt(rr0), -36))
      MFE_TRY(stencil64_prepare(ctx, A, w8, &dd, &ok));  // overwrites hs
    st64 = ok;
  }
  k_pcg_init<<<vg, kPT, 0, ctx->stream>>>(n, r, dinv, z, p, st, partials, tickets, 0);
  MFE_TRY(check_launch(ctx, "k_pcg_init"));
  DotSink ps{spart, tickets + 2, &st->pAp};

  auto body = [&](cudaGraphConditionalHandle h, int in_graph) -> mfe_status {
    if (st64)
      MFE_TRY(launch_spmv_st64(ctx, A, w8, dd, p, Ap, &ps, nullptr));
    else
      MFE_TRY(launch_spmv(ctx, A, p, Ap, &ps, nullptr, nullptr));
    k_pcg_update<<<vg, kPT, 0, ctx->stream>>>(n, x, r, z, p, Ap, dinv, st, partials, tickets, h,
                                             in_graph);
    MFE_TRY(check_launch(ctx, "k_pcg_update"));
    k_pcg_p<<<vg, kPT, 0, ctx->stream>>>(n, z, p, st);
    return check_launch(ctx, "k_pcg_p");
  };
  const bool eager = getenv("MFE_CG_EAGER") != nullptr;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ex = nullptr;
  auto release = [&]() {
    if (ex) cudaGraphExecDestroy(ex);
    if (g) cudaGraphDestroy(g);
    ex = nullptr;
    g = nullptr;
  };
  if (!eager) {
    cudaStream_t run_stream = ctx->stream, s = ctx->own_stream;
    cudaGraphConditionalHandle h = 0;
    mfe_status bst = MFE_OK;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    if (e == cudaSuccess) {
      ctx->stream = s;
      e = cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
      if (e == cudaSuccess) {
        k_pcg_begin<<<1, 1, 0, s>>>(st, h);
        e = cudaStreamEndCapture(s, &g);
      }
      cudaGraphNode_t nodes[4];
      size_t nn = 4;
      if (e == cudaSuccess) e = cudaGraphGetNodes(g, nodes, &nn);
      alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)];
      memset(cp_buf, 0, sizeof(cp_buf));
      cudaGraphNodeParams* cp = reinterpret_cast<cudaGraphNodeParams*>(cp_buf);
      cp->type = cudaGraphNodeTypeConditional;
      cp->conditional.handle = h;
      cp->conditional.type = cudaGraphCondTypeWhile;
      cp->conditional.size = 1;
      cudaGraphNode_t cnode;
      if (e == cudaSuccess) e = cudaGraphAddNode(&cnode, g, &nodes[0], nullptr, 1, cp);
      if (e == cudaSuccess) {
        cudaGraph_t bg = cp->conditional.phGraph_out[0];
        e = cudaStreamBeginCaptureToGraph(s, bg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        if (e == cudaSuccess) {
          bst = body(h, 1);
          cudaGraph_t tmp;
          const cudaError_t e2 = cudaStreamEndCapture(s, &tmp);
          if (e == cudaSuccess) e = e2;
        }
      }
      ctx->stream = run_stream;
      if (e == cudaSuccess && bst == MFE_OK) e = cudaGraphInstantiate(&ex, g, 0);
    }
    if (bst != MFE_OK) {
      release();
      return bst;
    }
    if (e != cudaSuccess) {
      release();
      return cuda_fail(ctx, e, "PCG graph");
    }
  }
  // the loop; a stencil solve that met its test is checked with the CSR
  // values and, should the operator's rounding-level difference from A ever
  // matter, restarted from the true residual (at most three times)
  double true_resid = -1.0;
  bool maxed = false;
  for (int restarts = 0;; ++restarts) {
    if (eager) {
      for (;;) {
        MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, st, sizeof(PcgState), cudaMemcpyDeviceToHost, ctx->stream));
        MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
        if (!hs->cont) break;
        MFE_TRY(body((cudaGraphConditionalHandle)0, 0));
      }
    } else {
      const cudaError_t e = cudaGraphLaunch(ex, ctx->stream);
      if (e != cudaSuccess) {
        release();
        return cuda_fail(ctx, e, "PCG graph launch");
      }
    }
    MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, st, sizeof(PcgState), cudaMemcpyDeviceToHost, ctx->stream));
    MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (!st64 || hs->status != 0 || !(hs->normr <= hs->tol_abs)) break;
    DotSink ts{spart, tickets + 2, &st->rr};
    MFE_TRY(launch_spmv(ctx, A, x, r, &ts, b, nullptr));
    ++csr_products;
    double rr = 0.0;
    MFE_CUDA_TRY(ctx, cudaMemcpyAsync(&hs->rr, &st->rr, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    rr = hs->rr;
    true_resid = sqrt(std::max(rr, 0.0));
    if (true_resid <= hs->tol_abs) break;
    if (restarts >= 3 || hs->k >= hs->max_iter) {
      maxed = true;
      break;
    }
    k_pcg_init<<<vg, kPT, 0, ctx->stream>>>(n, r, dinv, z, p, st, partials, tickets, 1);
    MFE_TRY(check_launch(ctx, "k_pcg_init"));
  }
  release();
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, st, sizeof(PcgState), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  // the PCG's products report their bounded waits in the context's SpMV word
  MFE_TRY(take_spmv_error(ctx));
  MFE_CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  memset(res, 0, sizeof(*res));
  res->num_iters = hs->k;
  res->normr = hs->normr;
  res->normr0 = hs->normr0;
  res->final_resid = true_resid >= 0.0 ? true_resid : hs->normr;
  res->times[4] = ms * 1e-3;
  res->fp64_spmvs = st64 ? csr_products : hs->k + 1;
  res->inner_operator = st64 ? MFE_INNER_STENCIL64 : MFE_INNER_NONE;
  ctx->history.clear();
  if (hs->status) return MFE_BREAKDOWN;
  if (maxed) return fail(ctx, MFE_MAXITER, "Jacobi PCG: the CSR residual stayed above the tolerance");
  return res->final_resid <= hs->tol_abs ? MFE_OK : MFE_MAXITER;
}

}  // namespace mfe
