// BLAS-1 kernels and the CG solver (ref/src/cg_solve.hpp, Vector_functions.hpp).
//
// The reference's loop per iteration is: p update (waxpby), matvec, dot(Ap,p),
// breakdown test, alpha, two waxpbys, dot(r,r) at the top of the next
// iteration.  Here one iteration is three kernels with the reductions fused
// into the producers of their operands:
//   k_cg_p       p = r + beta p                  (p = r at k = 1)
//   k_spmv_tiled Ap = A p, p.Ap                  (mfe_spmv.cu, SPMV_DOT)
//   k_cg_update  x += alpha p, r -= alpha Ap, r.r, scalar bookkeeping
// i.e. 11 vector passes per iteration plus one read of the matrix.  The loop
// itself is a CUDA graph with a conditional while node: the last block of
// k_cg_update decides whether another iteration runs (the reference's loop
// test, cg_solve.hpp:152) and sets the graph condition, so a whole solve is
// one graph launch with no host round trip.  The breakdown test
// (cg_solve.hpp:186-198) needs two extra norms; when its pre-test fires the
// graph exits and the host finishes that iteration with separate kernels.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "mfe_cgstate.cuh"
#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

constexpr int kVecThreads = 256;
constexpr int kMaxPartials = 8192;

// ---------------------------------------------------------------------------
// BLAS-1
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kVecThreads)
    k_dot(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
          double* partials, unsigned* ticket, double* out)
{
  __shared__ double red[32];
  double acc = 0.0;
  for (int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kVecThreads)
    acc = fma(x[i], y[i], acc);
  const double bt = block_sum(acc, red);
  double total;
  if (grid_reduce_last(bt, partials, ticket, red, &total) && threadIdx.x == 0) *out = total;
}

// x.y of FP32 vectors with the mixed solvers' reduction: products and sums
// in double-float (DFAcc: TwoProduct + TwoSum on the FP32 pipe, about 48
// significant bits), block and grid sums in double-float too, one FP64
// addition at the end
__global__ void __launch_bounds__(kVecThreads)
    k_dot_df(int64_t n, const float* __restrict__ x, const float* __restrict__ y,
             double* partials, unsigned* ticket, double* out)
{
  __shared__ float2 red[32];
  DFAcc acc;
  for (int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kVecThreads)
    acc.add_product(x[i], y[i]);
  double total;
  if (grid_reduce_last_df(acc, partials, ticket, red, &total) && threadIdx.x == 0) *out = total;
}

__global__ void __launch_bounds__(kVecThreads)
    k_waxpby(int64_t n, double alpha, const double* __restrict__ x, double beta,
             const double* __restrict__ y, double* __restrict__ w)
{
  for (int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kVecThreads)
    w[i] = fma(alpha, x[i], beta * y[i]);
}

// out[i] = x[idx[i]] (the send buffer of a halo exchange,
// exchange_externals.hpp: send_buffer[i] = x[elements_to_send[i]])
__global__ void __launch_bounds__(kVecThreads)
    k_gather_idx(int64_t n, const int32_t* __restrict__ idx, const double* __restrict__ x,
                 double* __restrict__ out)
{
  for (int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kVecThreads)
    out[i] = x[idx[i]];
}

// fused_waxpby (Vector_functions.hpp:154-185): both updates in one pass
__global__ void __launch_bounds__(kVecThreads)
    k_fused_waxpby(int64_t n, double alpha, const double* __restrict__ x, double beta,
                   const double* __restrict__ y, double* w, double alpha2,
                   const double* __restrict__ x2, double beta2, const double* __restrict__ y2,
                   double* w2)
{
  for (int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kVecThreads) {
    const double a = fma(alpha, x[i], beta * y[i]);
    const double c = fma(alpha2, x2[i], beta2 * y2[i]);
    w[i] = a;
    w2[i] = c;
  }
}

// ---------------------------------------------------------------------------
// CG iteration kernels
// ---------------------------------------------------------------------------
// r = b and r.r for a zero initial guess: the reference's r = b - A x0
// (cg_solve.hpp:124-138) is b exactly when x0 = 0, so a solve can start
// before the matrix values are on the device.  x0 is checked on the bit
// patterns (either zero passes); a nonzero entry sets st->x0_nonzero and the
// caller falls back to the CSR residual.
__global__ void __launch_bounds__(kVecThreads)
    k_cg_init_b(int64_t n, const double* __restrict__ b, const double* __restrict__ x,
                double* __restrict__ r, double* partials, unsigned* ticket, CgState* st)
{
  __shared__ double red[32];
  double acc = 0.0;
  bool nz = false;
  for (int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kVecThreads) {
    const double bv = b[i];
    r[i] = bv;
    acc = fma(bv, bv, acc);
    nz = nz || ((unsigned long long)__double_as_longlong(x[i]) << 1) != 0ull;
  }
  if (__syncthreads_or(nz) && threadIdx.x == 0) atomicOr(&st->x0_nonzero, 1u);
  const double bt = block_sum(acc, red);
  double total;
  if (grid_reduce_last(bt, partials, ticket, red, &total) && threadIdx.x == 0) cg_resid_init(st, total);
}

__global__ void k_cg_begin(const CgState* st, cudaGraphConditionalHandle h)
{
  cudaGraphSetConditional(h, st->cont ? 1u : 0u);
}

// p = r (k == 1, cg_solve.hpp:153-155, or a restart) or p = r + beta p
// (:156-161).  Vectorised as double2 when every array is 16-byte aligned (VEC).
template <bool VEC>
__global__ void __launch_bounds__(kVecThreads)
    k_cg_p(int64_t n, const double* __restrict__ r, double* __restrict__ p, const CgState* st)
{
  const bool first = (st->k == 1) || st->p_reset;
  const double beta = st->beta;
  const int64_t stride = (int64_t)gridDim.x * kVecThreads;
  int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x;
  if (VEC) {
    const int64_t n2 = n >> 1;
    const double2* r2 = reinterpret_cast<const double2*>(r);
    double2* p2 = reinterpret_cast<double2*>(p);
    for (int64_t j = i; j < n2; j += stride) {
      const double2 rv = r2[j];
      double2 pv;
      if (first) pv = rv;
      else {
        pv = p2[j];
        pv.x = fma(beta, pv.x, rv.x);
        pv.y = fma(beta, pv.y, rv.y);
      }
      p2[j] = pv;
    }
    if (i == 0 && (n & 1)) p[n - 1] = first ? r[n - 1] : fma(beta, p[n - 1], r[n - 1]);
  } else {
    for (; i < n; i += stride) p[i] = first ? r[i] : fma(beta, p[i], r[i]);
  }
}

// Scalar bookkeeping after r.r of iteration k is known (last block, thread 0):
// records the iteration, evaluates the loop test for k + 1 with the normr of
// the top of iteration k (cg_solve.hpp:152,163), and prepares beta, rtrans and
// normr for iteration k + 1 (cg_solve.hpp:157-163).
__device__ __forceinline__ void cg_after_update(CgState* st, double rr_new)
{
  const int k = st->k;
  st->rr_new = rr_new;
  st->num_iters = k;
  st->p_reset = 0;
  const int cont = (k + 1 <= st->max_iter) && (st->normr > st->tol_abs);
  st->cont = cont;
  if (cont) {
    st->beta = rr_new / st->rtrans;
    st->oldrtrans = st->rtrans;
    st->rtrans = rr_new;
    st->normr = sqrt(rr_new);
    st->k = k + 1;
    if (st->record) st->history[k + 1] = st->normr;
  }
}

// x += alpha p, r -= alpha Ap, r.r (cg_solve.hpp:201-213 + :158).
template <bool VEC>
__global__ void __launch_bounds__(kVecThreads)
    k_cg_update(int64_t n, double* __restrict__ x, double* __restrict__ r,
                const double* __restrict__ p, const double* __restrict__ Ap, CgState* st,
                double* partials, unsigned* ticket, cudaGraphConditionalHandle h, int in_graph)
{
  __shared__ double red[32];
  __shared__ double s_alpha;
  if (st->check_pending) {
    // the breakdown pre-test fired in the SpMV epilogue: stop the graph loop
    // and let the host finish this iteration
    if (in_graph && blockIdx.x == 0 && threadIdx.x == 0) cudaGraphSetConditional(h, 0u);
    return;
  }
  if (threadIdx.x == 0) s_alpha = st->rtrans / st->pAp;
  __syncthreads();
  const double alpha = s_alpha;
  double acc = 0.0;
  const int64_t stride = (int64_t)gridDim.x * kVecThreads;
  int64_t i = (int64_t)blockIdx.x * kVecThreads + threadIdx.x;
  if (VEC) {
    const int64_t n2 = n >> 1;
    double2* x2 = reinterpret_cast<double2*>(x);
    double2* r2 = reinterpret_cast<double2*>(r);
    const double2* p2 = reinterpret_cast<const double2*>(p);
    const double2* a2 = reinterpret_cast<const double2*>(Ap);
    for (int64_t j = i; j < n2; j += stride) {
      double2 xv = x2[j], rv = r2[j];
      const double2 pv = p2[j], av = a2[j];
      xv.x = fma(alpha, pv.x, xv.x);
      xv.y = fma(alpha, pv.y, xv.y);
      rv.x = fma(-alpha, av.x, rv.x);
      rv.y = fma(-alpha, av.y, rv.y);
      x2[j] = xv;
      r2[j] = rv;
      acc = fma(rv.x, rv.x, acc);
      acc = fma(rv.y, rv.y, acc);
    }
    if (i == 0 && (n & 1)) {
      const int64_t t = n - 1;
      x[t] = fma(alpha, p[t], x[t]);
      const double rv = fma(-alpha, Ap[t], r[t]);
      r[t] = rv;
      acc = fma(rv, rv, acc);
    }
  } else {
    for (; i < n; i += stride) {
      x[i] = fma(alpha, p[i], x[i]);
      const double rv = fma(-alpha, Ap[i], r[i]);
      r[i] = rv;
      acc = fma(rv, rv, acc);
    }
  }
  const double bt = block_sum(acc, red);
  double total;
  if (grid_reduce_last(bt, partials, ticket, red, &total) && threadIdx.x == 0) {
    cg_after_update(st, total);
    if (in_graph) cudaGraphSetConditional(h, st->cont ? 1u : 0u);
  }
}

// ---------------------------------------------------------------------------
// host: launch helpers
// ---------------------------------------------------------------------------
static int vec_grid(mfe_ctx* ctx, int64_t n)
{
  return (int)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(std::max<int64_t>(n, 1), kVecThreads),
                           std::min<int64_t>((int64_t)ctx->sm_count * 8, kMaxPartials)));
}

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

struct RedBufs {
  double* partials;
  unsigned* tickets;  // 4 tickets
  double* scalars;    // 8 device scalars
};

static mfe_status red_bufs(mfe_ctx* ctx, RedBufs* rb)
{
  const bool fresh = ctx->ws.find("red.partials") == ctx->ws.end();
  rb->partials = static_cast<double*>(workspace(ctx, "red.partials", sizeof(double) * kMaxPartials * 4));
  rb->tickets = static_cast<unsigned*>(workspace(ctx, "red.tickets", sizeof(unsigned) * 8));
  rb->scalars = static_cast<double*>(workspace(ctx, "red.scalars", sizeof(double) * 8));
  if (!rb->partials || !rb->tickets || !rb->scalars)
    return fail(ctx, MFE_OOM, "reduction workspace allocation failed");
  if (fresh) MFE_CUDA_TRY(ctx, cudaMemsetAsync(rb->tickets, 0, sizeof(unsigned) * 8, ctx->stream));
  return MFE_OK;
}

mfe_status launch_dot(mfe_ctx* ctx, int64_t n, const double* x, const double* y, double* dev_out)
{
  RedBufs rb;
  MFE_TRY(red_bufs(ctx, &rb));
  k_dot<<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, x, y, rb.partials, rb.tickets,
                                                           dev_out);
  return check_launch(ctx, "k_dot");
}

mfe_status launch_dot_f32(mfe_ctx* ctx, int64_t n, const float* x, const float* y, double* dev_out)
{
  RedBufs rb;
  MFE_TRY(red_bufs(ctx, &rb));
  k_dot_df<<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, x, y, rb.partials, rb.tickets,
                                                              dev_out);
  return check_launch(ctx, "k_dot_df");
}

mfe_status launch_fused_waxpby(mfe_ctx* ctx, int64_t n, double alpha, const double* x, double beta,
                               const double* y, double* w, double alpha2, const double* x2,
                               double beta2, const double* y2, double* w2)
{
  if (n <= 0) return MFE_OK;
  k_fused_waxpby<<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, alpha, x, beta, y, w, alpha2,
                                                                    x2, beta2, y2, w2);
  return check_launch(ctx, "k_fused_waxpby");
}

mfe_status launch_gather(mfe_ctx* ctx, int64_t n, const int32_t* idx, const double* x, double* out)
{
  if (n <= 0) return MFE_OK;
  k_gather_idx<<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, idx, x, out);
  return check_launch(ctx, "k_gather_idx");
}

mfe_status launch_waxpby(mfe_ctx* ctx, int64_t n, double alpha, const double* x, double beta,
                         const double* y, double* w)
{
  if (n <= 0) return MFE_OK;
  k_waxpby<<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, alpha, x, beta, y, w);
  return check_launch(ctx, "k_waxpby");
}

// ---------------------------------------------------------------------------
// CG graph
// ---------------------------------------------------------------------------
struct CgBufs {
  double* r;
  double* p;
  double* Ap;
  CgState* st;
  double* history;
  // the verified FP64 stencil operator (mfe_stencil64.cu) instead of the CSR
  // values: its eight mirror-class weights and the Dirichlet diagonal
  bool st64 = false;
  double w8[8] = {};
  double dd = 0.0;
  // the sliced ELL copy of an ELL matrix (mfe_ell.cu) for the iterations'
  // products
  const mfe_sell* sell = nullptr;
};

}  // namespace mfe

struct mfe_cg_graph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  cudaGraphConditionalHandle handle = 0;
  // what the graph was built for: operands, and the stencil operator's
  // weights (kernel parameters baked into the graph) when it runs
  const void* key[12] = {};
  double op[10] = {};
  int64_t n = 0;
  cudaStream_t stream = nullptr;
};

namespace mfe {

void cg_graph_destroy(mfe_cg_graph* g)
{
  if (!g) return;
  if (g->exec) cudaGraphExecDestroy(g->exec);
  if (g->graph) cudaGraphDestroy(g->graph);
  delete g;
}

static mfe_status launch_cg_p(mfe_ctx* ctx, int64_t n, const CgBufs& B)
{
  const bool vec = aligned16(B.r) && aligned16(B.p);
  if (vec)
    k_cg_p<true><<<vec_grid(ctx, n / 2), kVecThreads, 0, ctx->stream>>>(n, B.r, B.p, B.st);
  else
    k_cg_p<false><<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, B.r, B.p, B.st);
  return check_launch(ctx, "k_cg_p");
}

static mfe_status launch_cg_update(mfe_ctx* ctx, int64_t n, double* x, const CgBufs& B,
                                   const RedBufs& rb, cudaGraphConditionalHandle h, int in_graph)
{
  const bool vec = aligned16(x) && aligned16(B.r) && aligned16(B.p) && aligned16(B.Ap);
  double* partials = rb.partials + kMaxPartials;  // separate from the SpMV partials
  unsigned* ticket = rb.tickets + 1;
  if (vec)
    k_cg_update<true><<<vec_grid(ctx, n / 2), kVecThreads, 0, ctx->stream>>>(
        n, x, B.r, B.p, B.Ap, B.st, partials, ticket, h, in_graph);
  else
    k_cg_update<false><<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(
        n, x, B.r, B.p, B.Ap, B.st, partials, ticket, h, in_graph);
  return check_launch(ctx, "k_cg_update");
}

static mfe_status launch_cg_spmv(mfe_ctx* ctx, const mfe_csr* A, const CgBufs& B,
                                 const RedBufs& rb)
{
  DotSink sink;
  sink.partials = rb.partials;
  sink.ticket = rb.tickets;
  sink.out = rb.scalars;
  if (B.st64) return launch_spmv_st64(ctx, A, B.w8, B.dd, B.p, B.Ap, &sink, B.st);
  if (B.sell) return launch_spmv_sell(ctx, B.sell, B.p, B.Ap, &sink, B.st);
  return launch_spmv(ctx, A, B.p, B.Ap, &sink, nullptr, B.st);
}

static mfe_status build_graph(mfe_ctx* ctx, const mfe_csr* A, double* x, const CgBufs& B,
                              const RedBufs& rb, mfe_cg_graph** out)
{
  mfe_cg_graph* g = new mfe_cg_graph();
  const int64_t n = A->nrows;
  // capture on the context's own stream (the legacy default stream cannot be
  // captured); the executable graph is launched on ctx->stream afterwards
  cudaStream_t run_stream = ctx->stream;
  cudaStream_t s = ctx->own_stream;
  ctx->stream = s;
  auto bail = [&](cudaError_t e, const char* where) {
    cudaStreamCaptureStatus cs;
    if (cudaStreamIsCapturing(s, &cs) == cudaSuccess && cs != cudaStreamCaptureStatusNone) {
      cudaGraph_t tmp;
      cudaStreamEndCapture(s, &tmp);
    }
    ctx->stream = run_stream;
    cg_graph_destroy(g);
    cudaGetLastError();
    return cuda_fail(ctx, e, where);
  };
  cudaError_t e = cudaGraphCreate(&g->graph, 0);
  if (e != cudaSuccess) return bail(e, "cudaGraphCreate");
  e = cudaGraphConditionalHandleCreate(&g->handle, g->graph, 0, cudaGraphCondAssignDefault);
  if (e != cudaSuccess) return bail(e, "cudaGraphConditionalHandleCreate");

  // begin node: set the loop condition from the state
  e = cudaStreamBeginCaptureToGraph(s, g->graph, nullptr, nullptr, 0,
                                    cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return bail(e, "cudaStreamBeginCaptureToGraph");
  k_cg_begin<<<1, 1, 0, s>>>(B.st, g->handle);
  e = cudaStreamEndCapture(s, &g->graph);
  if (e != cudaSuccess) return bail(e, "cudaStreamEndCapture(begin)");
  cudaGraphNode_t nodes[4];
  size_t nn = 4;
  e = cudaGraphGetNodes(g->graph, nodes, &nn);
  if (e != cudaSuccess || nn != 1) return bail(e, "cudaGraphGetNodes");

  // cudaGraphNodeParams has no default constructor (it holds a union)
  alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)];
  memset(cp_buf, 0, sizeof(cp_buf));
  cudaGraphNodeParams* cp = reinterpret_cast<cudaGraphNodeParams*>(cp_buf);
  cp->type = cudaGraphNodeTypeConditional;
  cp->conditional.handle = g->handle;
  cp->conditional.type = cudaGraphCondTypeWhile;
  cp->conditional.size = 1;
  cudaGraphNode_t cnode;
  e = cudaGraphAddNode(&cnode, g->graph, &nodes[0], nullptr, 1, cp);
  if (e != cudaSuccess) return bail(e, "cudaGraphAddNode(while)");
  cudaGraph_t body = cp->conditional.phGraph_out[0];

  e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
  if (e != cudaSuccess) return bail(e, "cudaStreamBeginCaptureToGraph(body)");
  mfe_status st = launch_cg_p(ctx, n, B);
  if (st == MFE_OK) st = launch_cg_spmv(ctx, A, B, rb);
  if (st == MFE_OK) st = launch_cg_update(ctx, n, x, B, rb, g->handle, 1);
  e = cudaStreamEndCapture(s, &body);
  if (st != MFE_OK) {
    ctx->stream = run_stream;
    cg_graph_destroy(g);
    return st;
  }
  if (e != cudaSuccess) return bail(e, "cudaStreamEndCapture(body)");
  e = cudaGraphInstantiate(&g->exec, g->graph, 0);
  if (e != cudaSuccess) return bail(e, "cudaGraphInstantiate");
  ctx->stream = run_stream;
  *out = g;
  return MFE_OK;
}

// ---------------------------------------------------------------------------
// FP64 CG
// ---------------------------------------------------------------------------
static mfe_status cg_f64(mfe_ctx* ctx, const mfe_csr* A_in, const double* b, double* x,
                         const mfe_cg_opts* o, mfe_cg_result* res, const CgSpec* spec,
                         const mfe_sell* sell = nullptr, const mfe_ell* ell = nullptr)
{
  const int64_t n = A_in->nrows;
  mfe_csr A = *A_in;
  int max_len = 0;
  MFE_TRY(ensure_max_row_len(ctx, &A, &max_len));
  A.max_row_len = max_len;
  if (!csr_is_box(&A) && !sell) {
    // a CSR without box dimensions may still be a miniFE box matrix (e.g. one
    // handed over through the host drop-in call): recognise it once per solve
    int bx, by, bz;
    MFE_TRY(detect_box(ctx, &A, &bx, &by, &bz));
    A.box_nx = bx;
    A.box_ny = by;
    A.box_nz = bz;
  }

  CgBufs B;
  B.sell = sell;
  B.r = static_cast<double*>(workspace(ctx, "cg.r", sizeof(double) * std::max<int64_t>(n, 1)));
  B.p = static_cast<double*>(workspace(ctx, "cg.p", sizeof(double) * std::max<int64_t>(n, 1)));
  B.Ap = static_cast<double*>(workspace(ctx, "cg.Ap", sizeof(double) * std::max<int64_t>(n, 1)));
  B.st = static_cast<CgState*>(workspace(ctx, "cg.state", sizeof(CgState)));
  const int max_iter = std::max(0, o->max_iter);
  B.history = static_cast<double*>(
      workspace(ctx, "cg.history", sizeof(double) * ((size_t)max_iter + 2)));
  if (!B.r || !B.p || !B.Ap || !B.st || !B.history)
    return fail(ctx, MFE_OOM, "CG workspace allocation failed");
  RedBufs rb;
  MFE_TRY(red_bufs(ctx, &rb));
  if (!workspace(ctx, "spmv.err", sizeof(unsigned))) return fail(ctx, MFE_OOM, "workspace");

  // initial state (host -> device through pinned scratch; sized once for the
  // stencil check's class table too, so the buffer is not reallocated below)
  static_assert(sizeof(CgState) <= 2048, "state must fit the first half of the scratch");
  char* hbuf = static_cast<char*>(host_scratch(ctx, 32768));
  if (!hbuf) return fail(ctx, MFE_OOM, "pinned scratch allocation failed");
  CgState* hs = reinterpret_cast<CgState*>(hbuf);
  double* hn = reinterpret_cast<double*>(hbuf + 2048);
  memset(hs, 0, sizeof(CgState));
  hs->max_iter = max_iter;
  hs->tol_abs = o->tol;  // scaled by normr0 in the residual epilogue when relative
  hs->tol_mode = o->tol_mode == MFE_TOL_RELATIVE ? 1 : 0;
  hs->brkdown_tol = 2.220446049250313e-16;  // std::numeric_limits<double>::epsilon()
  hs->record = o->record_history ? 1 : 0;
  hs->history = B.history;
  hs->k = 1;

  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(B.st, hs, sizeof(CgState), cudaMemcpyHostToDevice, ctx->stream));
  int csr_products = 0;  // products with the CSR values
  if (spec) {
    // r = b (x0 = 0, checked by the kernel), nothing read from A yet
    k_cg_init_b<<<vec_grid(ctx, n), kVecThreads, 0, ctx->stream>>>(n, b, x, B.r, rb.partials,
                                                                    rb.tickets, B.st);
    MFE_TRY(check_launch(ctx, "k_cg_init_b"));
  } else {
    // r = b - A x0 with r.r (cg_solve.hpp:124-138; the reference first
    // copies x into p and forms A p)
    DotSink sink;
    sink.partials = rb.partials;
    sink.ticket = rb.tickets;
    sink.out = rb.scalars;
    if (ell) MFE_TRY(launch_spmv_ell(ctx, ell, x, B.r, &sink, b, B.st));
    else MFE_TRY(launch_spmv(ctx, &A, x, B.r, &sink, b, B.st));
    csr_products = 1;
  }
  // A CSR that is not a box matrix: the iterations' products run on a
  // sliced copy (32-row slices, column-major inside a slice, rows padded to
  // the longest) when its rows are short and even enough for the padding to
  // stay within a quarter of the nonzeros and the solve may run long enough
  // to repay the copy; the residuals keep the CSR
  mfe_sell gen_sell;
  if (!sell && !csr_is_box(&A) && A.dtype == MFE_F64 && max_iter >= 4 && max_len >= 1 &&
      max_len <= 64) {
    const int64_t ne = sell_entries(n, max_len);
    if (ne < ((int64_t)1 << 31) && (double)ne <= 1.25 * (double)A.nnz + 32.0 * max_len) {
      memset(&gen_sell, 0, sizeof(gen_sell));
      gen_sell.cols = static_cast<int32_t*>(workspace(ctx, "cg.sell.cols", sizeof(int32_t) * (size_t)ne));
      gen_sell.vals = static_cast<double*>(workspace(ctx, "cg.sell.vals", sizeof(double) * (size_t)ne));
      if (!gen_sell.cols || !gen_sell.vals) return fail(ctx, MFE_OOM, "sliced copy allocation failed");
      MFE_TRY(launch_csr_to_sell(ctx, &A, max_len, &gen_sell));
      sell = &gen_sell;
      B.sell = sell;
    }
  }
  // The verified FP64 stencil operator (checked on every call) when the
  // tolerance is at least 2^-36 of the initial residual: the operator lies
  // within 2^-39 of every entry of A, so tighter stops (the reference's
  // absolute DBL_EPSILON) would meet its rounding-level difference from A
  // and use the CSR values.
  if (spec) {
    MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, B.st, sizeof(CgState), cudaMemcpyDeviceToHost, ctx->stream));
    MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (hs->err || hs->x0_nonzero || !(hs->tol_abs >= std::ldexp(hs->normr0, -36))) return kSpecFailed;
    for (int c = 0; c < 8; ++c) B.w8[c] = spec->w8[c];
    B.dd = spec->dd;
    B.st64 = true;
  } else if (o->f64_operator == 0 && csr_is_box(&A)) {
    MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, B.st, sizeof(CgState), cudaMemcpyDeviceToHost, ctx->stream));
    MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (!hs->err && hs->tol_abs >= std::ldexp(hs->normr0, -36))
      MFE_TRY(stencil64_prepare(ctx, &A, B.w8, &B.dd, &B.st64));  // overwrites hs
  }

  // (re)build the graph when the operands changed
  const void* key[12] = {A.row_offsets, A.cols, A.vals, x, b, B.r, B.p, B.Ap, B.st,
                         (const void*)(uintptr_t)(((int64_t)A.box_nx << 42) ^
                                                  ((int64_t)A.box_ny << 21) ^ A.box_nz),
                         sell ? (const void*)sell->vals : nullptr,
                         sell ? (const void*)sell->cols : nullptr};
  double op[10] = {B.st64 ? 1.0 : 0.0, B.dd};
  for (int c = 0; c < 8; ++c) op[2 + c] = B.w8[c];
  mfe_cg_graph* g = ctx->cg_graph;
  if (!g || g->n != n || g->stream != ctx->stream || memcmp(g->key, key, sizeof(key)) != 0 ||
      memcmp(g->op, op, sizeof(op)) != 0) {
    cg_graph_destroy(g);
    ctx->cg_graph = nullptr;
    MFE_TRY(build_graph(ctx, &A, x, B, rb, &g));
    memcpy(g->key, key, sizeof(key));
    memcpy(g->op, op, sizeof(op));
    g->n = n;
    g->stream = ctx->stream;
    ctx->cg_graph = g;
  }

  int status = MFE_OK;
  bool confirmed = spec == nullptr;
  double true_resid = -1.0;    // ||b - A x|| with the CSR values (stencil solves)
  // MFE_CG_EAGER=1 issues the same three kernels per iteration as ordinary
  // launches from the host (one small state read per iteration) instead of
  // the graph's device-side loop: identical work, visible to per-kernel
  // profilers that do not descend into conditional graph nodes
  const bool eager = getenv("MFE_CG_EAGER") != nullptr;
  for (int restarts = 0;; ++restarts) {
    for (int round = 0;; ++round) {
      if (eager) {
        for (;;) {
          MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, B.st, sizeof(CgState), cudaMemcpyDeviceToHost, ctx->stream));
          MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
          if (!hs->cont || hs->check_pending || hs->err) break;
          MFE_TRY(launch_cg_p(ctx, n, B));
          MFE_TRY(launch_cg_spmv(ctx, &A, B, rb));
          MFE_TRY(launch_cg_update(ctx, n, x, B, rb, 0, 0));
        }
      } else {
        MFE_CUDA_TRY(ctx, cudaGraphLaunch(g->exec, ctx->stream));
      }
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, B.st, sizeof(CgState), cudaMemcpyDeviceToHost, ctx->stream));
      MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      if (hs->err) return fail(ctx, MFE_TIMEOUT, "a bounded device wait gave up during CG");
      if (!hs->check_pending) break;
      // breakdown() (cg_solve.hpp:49-67): |p.Ap| <= 100 ||Ap|| ||p|| eps
      double* d = rb.scalars + 2;
      MFE_TRY(launch_dot(ctx, n, B.Ap, B.Ap, d));
      MFE_TRY(launch_dot(ctx, n, B.p, B.p, d + 1));
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hn, d, 2 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
      MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      const double norms[2] = {hn[0], hn[1]};
      const double pAp = hs->pAp;
      const bool brk = pAp < 0 ||
                       std::fabs(pAp) <= 100 * std::sqrt(norms[0]) * std::sqrt(norms[1]) *
                                             2.220446049250313e-16;
      if (brk) {
        status = MFE_BREAKDOWN;
        break;
      }
      hs->brkdown_tol = 0.1 * pAp;
      hs->check_pending = 0;
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(B.st, hs, sizeof(CgState), cudaMemcpyHostToDevice, ctx->stream));
      MFE_TRY(launch_cg_update(ctx, n, x, B, rb, 0, 0));
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, B.st, sizeof(CgState), cudaMemcpyDeviceToHost, ctx->stream));
      MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      if (!hs->cont) break;
    }
    // a speculative start: the values are on the device and passed their
    // checks before any result counts
    if (!confirmed) {
      confirmed = true;
      if (!spec->confirm(spec->arg)) return kSpecFailed;
    }
    // A stencil solve that met the loop's test is checked with the CSR
    // values: r = b - A x (written to r, the restart residual if it is
    // needed) and ||r|| against the same tolerance.  Should the operator's
    // rounding-level difference from A ever matter, CG restarts from x with
    // the true residual (at most kMaxRestarts times, within max_iter).
    if (!B.st64 || status != MFE_OK || !(hs->normr <= hs->tol_abs)) break;
    {
      DotSink sink;
      sink.partials = rb.partials;
      sink.ticket = rb.tickets;
      sink.out = rb.scalars + 4;
      MFE_TRY(launch_spmv(ctx, &A, x, B.r, &sink, b, nullptr));
      ++csr_products;
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hn, rb.scalars + 4, sizeof(double), cudaMemcpyDeviceToHost,
                                        ctx->stream));
      MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      // this product reports its bounded waits in the context's SpMV word
      MFE_TRY(take_spmv_error(ctx));
    }
    const double rr = hn[0];
    true_resid = std::sqrt(std::max(rr, 0.0));
    constexpr int kMaxRestarts = 3;
    if (true_resid <= hs->tol_abs) break;
    if (restarts >= kMaxRestarts || hs->num_iters + 1 > max_iter) {
      status = MFE_MAXITER;
      fail(ctx, MFE_MAXITER, "FP64 stencil CG: the CSR residual stayed above the tolerance");
      break;
    }
    hs->rtrans = rr;
    hs->rr_new = rr;
    hs->normr = true_resid;
    hs->k = hs->num_iters + 1;
    hs->p_reset = 1;
    hs->check_pending = 0;
    hs->cont = hs->normr > hs->tol_abs ? 1 : 0;
    MFE_CUDA_TRY(ctx, cudaMemcpyAsync(B.st, hs, sizeof(CgState), cudaMemcpyHostToDevice, ctx->stream));
  }
  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);

  res->num_iters = hs->num_iters;
  res->status = status;
  res->normr = hs->normr;
  res->normr0 = hs->normr0;
  res->final_resid = true_resid >= 0.0 ? true_resid : std::sqrt(std::max(hs->rr_new, 0.0));
  for (double& t : res->times) t = 0.0;
  res->times[4] = ms * 1e-3;
  res->refinements = 0;
  res->fp64_spmvs = B.st64 ? csr_products : hs->num_iters + 1;
  res->inner_operator = B.st64 ? MFE_INNER_STENCIL64 : MFE_INNER_NONE;
  if (o->record_history) {
    const int cnt = hs->num_iters + 1;
    ctx->history.resize(cnt);
    MFE_CUDA_TRY(ctx, cudaMemcpy(ctx->history.data(), B.history, sizeof(double) * cnt,
                                 cudaMemcpyDeviceToHost));
  } else {
    ctx->history.clear();
  }
  return (mfe_status)status;
}

mfe_status cg_solve_impl(mfe_ctx* ctx, const mfe_csr* A, const double* b, double* x,
                         const mfe_cg_opts* opts, mfe_cg_result* res)
{
  if (opts->precond == 1) return cg_jacobi(ctx, A, b, x, opts, res);
  if (opts->precision == MFE_PREC_F64) return cg_f64(ctx, A, b, x, opts, res, nullptr);
  return cg_mixed(ctx, A, b, x, opts, res);
}

mfe_status cg_solve_sell(mfe_ctx* ctx, const mfe_csr* V, const mfe_sell* S, const double* b,
                         double* x, const mfe_cg_opts* opts, mfe_cg_result* res, const mfe_ell* E)
{
  if (opts->precond != 0 || opts->precision != MFE_PREC_F64)
    return fail(ctx, MFE_BAD_ARG, "the sliced ELL CG is FP64 without preconditioner");
  return cg_f64(ctx, V, b, x, opts, res, nullptr, S, E);
}

mfe_status cg_solve_spec(mfe_ctx* ctx, const mfe_csr* A, const double* b, double* x,
                         const mfe_cg_opts* opts, mfe_cg_result* res, const CgSpec* spec)
{
  if (opts->precond != 0 || opts->precision != MFE_PREC_F64 || opts->f64_operator != 0 ||
      !csr_is_box(A))
    return kSpecFailed;
  return cg_f64(ctx, A, b, x, opts, res, spec);
}

}  // namespace mfe
