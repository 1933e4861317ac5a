// Mixed-precision CG: FP32 matrix, vectors and FMAs, FP64 dots, scalars and
// solution, with reliable updates against the FP64 matrix.
//
// The reference solves in FP64 only (ref/src/cg_solve.hpp).  Here the inner
// recurrence runs the reference's CG steps (p update, A p, p.Ap, alpha, x and
// r updates, r.r, beta) on an FP32 copy of the matrix with FP32 vectors --
// half the bytes of every pass -- while every reduction is carried to FP64
// accuracy (double-float sums on the FP32 pipe, or FP64 sums of values
// widened with integer operations, mfe_common.cuh) and alpha / beta stay
// FP64.  The FP32 iterate is a correction x32 to the FP64 solution x.  A
// reliable update -- x += x32, x32 = 0, r = b - A x in FP64 (the box SpMV
// writing the residual straight into the FP32 r) -- replaces the drifting
// recursive residual with the true one; the search direction p is kept, so
// the recurrence continues instead of restarting and the iteration count stays
// close to the FP64 solver's.  Updates happen every refine_k iterations, when
// the recursive residual has dropped by inner_tol (default a hundredfold)
// since the last update, and whenever the recursive residual claims
// convergence; the solve stops only when the true FP64 residual meets the
// tolerance (or after max_refine updates, when that cap is set).
//
// One iteration is three kernels (k_mx_p, the FP32 operator with p.Ap -- the
// verified stencil of mfe_stencil.cu or the box SpMV over an FP32 copy of
// the values -- and k_mx_update) plus two that only work when an update is
// due (the graph cannot branch cheaply per iteration, so k_mx_xupdate and the
// FP64 residual SpMV check a device-side gate and return at once when it is
// closed) and a one-thread bookkeeping kernel that sets the loop condition.
// The whole solve is one CUDA graph launch with a conditional while node.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

struct MixState {
  double rr;            // r.r of the current recursive residual (FP64 accumulated)
  double rr_new;        // r.r after this iteration's update
  double pAp;           // written by the FP32 SpMV's epilogue
  double beta;
  double rr_true;       // ||b - A x||^2 from the gated FP64 residual SpMV
  double rr_at_update;  // rr right after the last reliable update
  double normr0, tol_abs, normr_true;
  double delta2;        // update when rr_new < delta2 * rr_at_update
  double alpha_prev;    // alpha of the last update, whose x32 += alpha p is still pending
  int k;                // inner iterations done
  int max_iter;
  int since;            // iterations since the last reliable update
  int refine_k;         // update at least every refine_k iterations
  int max_refine;       // stop after this many updates (0: no cap)
  int gate;             // 1: a reliable update runs in this iteration
  int cont;             // loop condition
  int first;            // next p update is p = r
  int updates;          // reliable updates done
  int status;           // 0 ok, MFE_BREAKDOWN
  int record;
  unsigned err;
  int x_pending;        // 1: x32 += alpha_prev p is due (done by the next p update or
                        // the gated x update, whichever comes first)
  double* history;      // recursive normr per iteration (record)
};

constexpr int kT = 256;
constexpr int kMaxPart = 8192;

// p = r (first) or p = r + beta p, FP32 (cg_solve.hpp:153-161).  The previous
// iteration's x32 += alpha p (cg_solve.hpp:201-205) is done here, where the
// old p is read anyway, unless the reliable update already folded it in:
// the update kernel then reads only r and Ap.
__global__ void __launch_bounds__(kT)
    k_mx_p(int64_t n, const float* __restrict__ r, float* __restrict__ p, float* __restrict__ x32,
           const MixState* st)
{
  const bool first = st->first != 0;
  const bool addx = !first && st->x_pending != 0;
  const float beta = (float)st->beta;
  const float alpha = (float)st->alpha_prev;
  const int64_t stride = (int64_t)gridDim.x * kT;
  const int64_t n4 = n >> 2;
  const float4* r4 = reinterpret_cast<const float4*>(r);
  float4* p4 = reinterpret_cast<float4*>(p);
  float4* x4 = reinterpret_cast<float4*>(x32);
  for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n4; i += stride) {
    const float4 rv = r4[i];
    float4 pv;
    if (first) pv = rv;
    else {
      pv = p4[i];
      if (addx) {
        float4 xv = x4[i];
        xv.x = fmaf(alpha, pv.x, xv.x);
        xv.y = fmaf(alpha, pv.y, xv.y);
        xv.z = fmaf(alpha, pv.z, xv.z);
        xv.w = fmaf(alpha, pv.w, xv.w);
        x4[i] = xv;
      }
      pv.x = fmaf(beta, pv.x, rv.x);
      pv.y = fmaf(beta, pv.y, rv.y);
      pv.z = fmaf(beta, pv.z, rv.z);
      pv.w = fmaf(beta, pv.w, rv.w);
    }
    p4[i] = pv;
  }
  const int64_t t = (n4 << 2) + (int64_t)blockIdx.x * kT + threadIdx.x;
  if (blockIdx.x == 0 && t < n) {
    if (addx) x32[t] = fmaf(alpha, p[t], x32[t]);
    p[t] = first ? r[t] : fmaf(beta, p[t], r[t]);
  }
}

// r -= alpha Ap, r.r (cg_solve.hpp:206-213, :158) accumulated in double-float
// per thread (FP32 operations: one FP64 FMA per row would make the kernel
// FP64-bound on GB300) and summed in FP64 across threads and blocks; x32 +=
// alpha p is left pending (k_mx_p / k_mx_xupdate).  The last block decides
// whether a reliable update is due; inside the graph it also does the
// bookkeeping of an iteration without one (k_mx_after's, which then runs only
// in the conditional node of the update) and sets both graph conditions.
__global__ void __launch_bounds__(kT)
    k_mx_update(int64_t n, float* __restrict__ r, const float* __restrict__ Ap, MixState* st,
                double* partials, unsigned* ticket, cudaGraphConditionalHandle h_loop,
                cudaGraphConditionalHandle h_upd, int in_graph)
{
  __shared__ float2 red[32];
  __shared__ float s_alpha;
  if (threadIdx.x == 0) s_alpha = st->pAp > 0.0 ? (float)(st->rr / st->pAp) : 0.0f;
  __syncthreads();
  const float alpha = s_alpha;
  DFAcc acc;
  const int64_t stride = (int64_t)gridDim.x * kT;
  const int64_t n4 = n >> 2;
  float4* r4 = reinterpret_cast<float4*>(r);
  const float4* a4 = reinterpret_cast<const float4*>(Ap);
  for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n4; i += stride) {
    float4 rv = r4[i];
    const float4 av = a4[i];
    rv.x = fmaf(-alpha, av.x, rv.x);
    rv.y = fmaf(-alpha, av.y, rv.y);
    rv.z = fmaf(-alpha, av.z, rv.z);
    rv.w = fmaf(-alpha, av.w, rv.w);
    r4[i] = rv;
    acc.add_product(rv.x, rv.x);
    acc.add_product(rv.y, rv.y);
    acc.add_product(rv.z, rv.z);
    acc.add_product(rv.w, rv.w);
  }
  const int64_t t = (n4 << 2) + (int64_t)blockIdx.x * kT + threadIdx.x;
  if (blockIdx.x == 0 && t < n) {
    const float rv = fmaf(-alpha, Ap[t], r[t]);
    r[t] = rv;
    acc.add_product(rv, rv);
  }
  double total;
  if (grid_reduce_last_df(acc, partials, ticket, red, &total) && threadIdx.x == 0) {
    st->rr_new = total;
    st->alpha_prev = alpha;
    st->x_pending = 1;
    st->k += 1;
    st->since += 1;
    st->first = 0;
    if (st->record) st->history[st->k] = sqrt(total);
    if (!(st->pAp > 0.0)) st->status = MFE_BREAKDOWN;  // cg_solve.hpp:187
    st->gate = st->status == 0 &&
               (st->since >= st->refine_k || total < st->delta2 * st->rr_at_update ||
                total <= st->tol_abs * st->tol_abs || st->k >= st->max_iter);
    if (in_graph) {
      if (!st->gate) {
        if (st->status != 0) {
          st->cont = 0;
        } else {
          st->beta = total / st->rr;
          st->rr = total;
          st->cont = st->k < st->max_iter;
        }
        cudaGraphSetConditional(h_loop, st->cont ? 1u : 0u);
      }
      cudaGraphSetConditional(h_upd, st->gate ? 1u : 0u);
    }
  }
}

// reliable update, part 1 (gated): x += x32, x32 = 0
// x32 may be x-padded (rows of Nx + pad entries; row i at i + (i / Nx) * pad)
__global__ void __launch_bounds__(kT)
    k_mx_xupdate(int64_t n, double* __restrict__ x, float* __restrict__ x32,
                 const float* __restrict__ p, MixState* st, int Nx, int pad)
{
  if (st->gate == 0) return;
  // the pending x32 += alpha p folded in (the same FP32 FMA k_mx_p would do)
  const float alpha = (float)st->alpha_prev;
  for (int64_t i = (int64_t)blockIdx.x * kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
    const int64_t j = pad ? i + (i / Nx) * pad : i;
    x[i] += f2d_exact(fmaf(alpha, p[j], x32[j]));
    x32[j] = 0.0f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) st->x_pending = 0;  // read next by k_mx_p only
}

// bookkeeping (one thread): finish a reliable update, set the loop condition
__global__ void k_mx_after(MixState* st, cudaGraphConditionalHandle h, int in_graph)
{
  if (st->status != 0) {
    st->cont = 0;
  } else if (st->gate) {
    st->updates += 1;
    st->since = 0;
    st->normr_true = sqrt(st->rr_true);
    if (st->normr_true <= st->tol_abs || st->k >= st->max_iter ||
        (st->max_refine > 0 && st->updates >= st->max_refine)) {
      st->cont = 0;
    } else {
      // continue the recurrence from the true residual, keeping p
      st->beta = st->rr_true / st->rr;
      st->rr = st->rr_true;
      st->rr_at_update = st->rr_true;
      st->cont = 1;
    }
  } else {
    st->beta = st->rr_new / st->rr;
    st->rr = st->rr_new;
    st->cont = st->k < st->max_iter;
  }
  st->gate = 0;
  if (in_graph) cudaGraphSetConditional(h, st->cont ? 1u : 0u);
}

__global__ void k_mx_init(MixState* st)
{
  // after the first FP64 residual: r32 = b - A x0, rr_true = ||r||^2
  const double nr = sqrt(st->rr_true);
  st->normr0 = nr;
  st->normr_true = nr;
  if (st->gate) st->tol_abs *= nr;  // relative tolerance (gate carries tol_mode here)
  st->gate = 0;
  st->rr = st->rr_true;
  st->rr_at_update = st->rr_true;
  st->cont = (st->max_iter > 0) && (nr > st->tol_abs);
  if (st->record) st->history[0] = nr;
}

__global__ void k_mx_begin(const MixState* st, cudaGraphConditionalHandle h)
{
  cudaGraphSetConditional(h, st->cont ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------
namespace {

struct MixBufs {
  float *r, *p, *Ap, *x32;
  MixState* st;
  double* history;
  double* partials;  // 2 * kMaxPart
  unsigned* tickets; // 2
  bool stencil = false;  // FP32 stencil operator (x-padded vectors, p with ghost zones)
  float coef[28];        // its interior stencil and Dirichlet diagonal
  int stencil_grid = 0;
  int64_t nv = 0;        // length of the FP32 vectors
  int pad = 0;           // x padding of the FP32 vectors (0: natural layout)
  unsigned* err = nullptr;
};

// one wave of resident blocks of `kernel`
int grid_for(mfe_ctx* ctx, int64_t n, const void* kernel)
{
  return (int)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(std::max<int64_t>(n, 1), kT),
                           (int64_t)resident_blocks(ctx, kernel, kT, 0)));
}

// one iteration up to the update decision: p update, FP32 operator with
// p.Ap, r update (h_upd: the graph condition of the reliable update)
mfe_status launch_iter(mfe_ctx* ctx, const mfe_csr& A32, const mfe_csr& A64, const double* b,
                       double* x, const MixBufs& B, cudaGraphConditionalHandle h,
                       cudaGraphConditionalHandle h_upd, int in_graph)
{
  const int64_t nv = B.nv;
  k_mx_p<<<grid_for(ctx, nv / 4, (const void*)k_mx_p), kT, 0, ctx->stream>>>(nv, B.r, B.p, B.x32, B.st);
  MFE_TRY(check_launch(ctx, "k_mx_p"));
  DotSink s1;
  s1.partials = B.partials;
  s1.ticket = B.tickets;
  s1.out = &B.st->pAp;
  if (B.stencil)
    MFE_TRY(launch_spmv_stencil(ctx, &A32, B.coef, B.p, B.Ap, &s1, B.stencil_grid, B.err));
  else
    MFE_TRY(launch_spmv(ctx, &A32, B.p, B.Ap, &s1, nullptr, nullptr));
  k_mx_update<<<grid_for(ctx, nv / 4, (const void*)k_mx_update), kT, 0, ctx->stream>>>(
      nv, B.r, B.Ap, B.st, B.partials + kMaxPart, B.tickets + 1, h, h_upd, in_graph);
  return check_launch(ctx, "k_mx_update");
}

// the reliable update (gated: its kernels return at once unless it is due;
// inside the graph they run in a conditional node) and the bookkeeping
mfe_status launch_update(mfe_ctx* ctx, const mfe_csr& A64, const double* b, double* x,
                         const MixBufs& B, cudaGraphConditionalHandle h, int in_graph)
{
  const int64_t n = A64.nrows;
  k_mx_xupdate<<<grid_for(ctx, n, (const void*)k_mx_xupdate), kT, 0, ctx->stream>>>(
      n, x, B.x32, B.p, B.st, A64.box_nx + 1, B.pad);
  MFE_TRY(check_launch(ctx, "k_mx_xupdate"));
  DotSink s2;
  s2.partials = B.partials;
  s2.ticket = B.tickets;
  s2.out = &B.st->rr_true;
  MFE_TRY(launch_box_resid_f32out(ctx, &A64, x, b, B.r, &s2, &B.st->gate, B.pad));
  k_mx_after<<<1, 1, 0, ctx->stream>>>(B.st, h, in_graph);
  return check_launch(ctx, "k_mx_after");
}

}  // namespace

mfe_status cg_mixed(mfe_ctx* ctx, const mfe_csr* A64_in, const double* b, double* x,
                    const mfe_cg_opts* o, mfe_cg_result* res)
{
  if (!mixed_opts_valid(o)) return fail(ctx, MFE_BAD_ARG, "inner_tol must lie in [0, 1) and max_refine must be >= 0");
  const int64_t n = A64_in->nrows;
  mfe_csr A64 = *A64_in;
  if (!csr_is_box(&A64)) {
    int bx, by, bz;
    MFE_TRY(detect_box(ctx, &A64, &bx, &by, &bz));
    A64.box_nx = bx;
    A64.box_ny = by;
    A64.box_nz = bz;
  }
  if (!csr_is_box(&A64))
    return fail(ctx, MFE_NOT_SUPPORTED,
                "the mixed-precision solver needs a box-structured matrix (miniFE assembly)");
  if (((uintptr_t)A64.vals & 15u) || ((uintptr_t)x & 15u))
    return fail(ctx, MFE_BAD_ARG, "mixed solver: matrix values and x must be 16-byte aligned");
  A64.max_row_len = 27;

  // The inner FP32 operator: the verified stencil when the matrix is a
  // miniFE box operator (checked on every call), else an FP32 copy of the
  // values (made on every call: a cache keyed on the values pointer would go
  // stale when an allocator hands the same address to another matrix).
  MixBufs B;
  bool use_stencil = false;
  if (o->mixed_operator == 0 && o->A32 == nullptr)
    MFE_TRY(stencil_prepare(ctx, &A64, B.coef, &use_stencil));
  mfe_csr A32;
  if (o->A32 != nullptr) {
    A32 = *o->A32;
    if (A32.dtype != MFE_F32 || A32.nnz != A64.nnz || A32.nrows != n)
      return fail(ctx, MFE_BAD_ARG, "opts->A32 does not match A");
  } else {
    A32 = A64;
    A32.dtype = MFE_F32;
    A32.vals = nullptr;
    if (!use_stencil) {
      float* v32 = static_cast<float*>(workspace(ctx, "mixed.vals32", sizeof(float) * (size_t)(A64.nnz + 4)));
      if (!v32) return fail(ctx, MFE_OOM, "FP32 matrix copy allocation failed");
      MFE_TRY(launch_convert_f32(ctx, static_cast<const double*>(A64.vals), v32, A64.nnz));
      A32.vals = v32;
    }
  }
  A32.box_nx = A64.box_nx;
  A32.box_ny = A64.box_ny;
  A32.box_nz = A64.box_nz;
  A32.max_row_len = 27;

  // with the stencil the FP32 vectors are x-padded and p has ghost zones of
  // zero rows around it
  B.nv = use_stencil ? stencil_rows(&A64) : n;
  B.pad = use_stencil ? stencil_pitch(&A64) - (A64.box_nx + 1) : 0;
  const size_t vb = sizeof(float) * (size_t)std::max<int64_t>(B.nv + 4, 4);
  B.r = static_cast<float*>(workspace(ctx, "mixed.r", vb));
  const int64_t ghost = use_stencil ? stencil_ghost(&A64) : 0;
  const size_t pb = sizeof(float) * (size_t)(std::max<int64_t>(B.nv + 4, 4) + 2 * ghost);
  float* pbase = static_cast<float*>(workspace(ctx, use_stencil ? "mixed.pg" : "mixed.p", pb));
  B.p = pbase ? pbase + ghost : nullptr;
  if (use_stencil) {
    B.stencil = true;
    MFE_TRY(stencil_grid(ctx, B.coef, &B.stencil_grid));
  }
  B.Ap = static_cast<float*>(workspace(ctx, "mixed.Ap", vb));
  B.x32 = static_cast<float*>(workspace(ctx, "mixed.x32", vb));
  B.st = static_cast<MixState*>(workspace(ctx, "mixed.state", sizeof(MixState)));
  B.err = B.st ? &B.st->err : nullptr;  // the stencil SpMV's bounded waits report here
  const int max_iter = std::max(0, o->max_iter);
  B.history = static_cast<double*>(workspace(ctx, "mixed.history", sizeof(double) * ((size_t)max_iter + 2)));
  B.partials = static_cast<double*>(workspace(ctx, "mixed.partials", sizeof(double) * 2 * kMaxPart));
  const bool fresh = ctx->ws.find("mixed.tickets") == ctx->ws.end();
  B.tickets = static_cast<unsigned*>(workspace(ctx, "mixed.tickets", sizeof(unsigned) * 4));
  if (!B.r || !B.p || !B.Ap || !B.x32 || !B.st || !B.history || !B.partials || !B.tickets)
    return fail(ctx, MFE_OOM, "mixed solver workspace allocation failed");
  if (fresh) MFE_CUDA_TRY(ctx, cudaMemsetAsync(B.tickets, 0, sizeof(unsigned) * 4, ctx->stream));
  if (!workspace(ctx, "spmv.err", sizeof(unsigned))) return fail(ctx, MFE_OOM, "workspace");

  char* hbuf = static_cast<char*>(host_scratch(ctx, 4096));
  if (!hbuf) return fail(ctx, MFE_OOM, "pinned scratch allocation failed");
  MixState* hs = reinterpret_cast<MixState*>(hbuf);
  memset(hs, 0, sizeof(MixState));
  hs->max_iter = max_iter;
  hs->tol_abs = o->tol;
  hs->gate = o->tol_mode == MFE_TOL_RELATIVE ? 1 : 0;  // consumed by k_mx_init
  hs->refine_k = o->refine_k > 0 ? o->refine_k : 100;
  hs->delta2 = mixed_delta2(o);
  hs->max_refine = o->max_refine;
  hs->record = o->record_history ? 1 : 0;
  hs->history = B.history;
  hs->first = 1;

  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(B.st, hs, sizeof(MixState), cudaMemcpyHostToDevice, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(B.x32, 0, vb, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(pbase, 0, pb, ctx->stream));
  if (B.pad) MFE_CUDA_TRY(ctx, cudaMemsetAsync(B.r, 0, vb, ctx->stream));  // padding entries stay 0
  {
    DotSink s;
    s.partials = B.partials;
    s.ticket = B.tickets;
    s.out = &B.st->rr_true;
    MFE_TRY(launch_box_resid_f32out(ctx, &A64, x, b, B.r, &s, nullptr, B.pad));
  }
  k_mx_init<<<1, 1, 0, ctx->stream>>>(B.st);
  MFE_TRY(check_launch(ctx, "k_mx_init"));

  // occupancy queries before the loop is captured
  grid_for(ctx, 1, (const void*)k_mx_p);
  grid_for(ctx, 1, (const void*)k_mx_update);
  grid_for(ctx, 1, (const void*)k_mx_xupdate);
  if (getenv("MFE_CG_EAGER") != nullptr) {
    for (;;) {
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, B.st, sizeof(MixState), cudaMemcpyDeviceToHost, ctx->stream));
      MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      if (!hs->cont || hs->err) break;
      MFE_TRY(launch_iter(ctx, A32, A64, b, x, B, 0, 0, 0));
      MFE_TRY(launch_update(ctx, A64, b, x, B, 0, 0));
    }
  } else {
    // graph: begin kernel, then while(cont) { one iteration }
    cudaStream_t run_stream = ctx->stream;
    cudaStream_t s = ctx->own_stream;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ex = nullptr;
    cudaGraphConditionalHandle h = 0;
    cudaError_t e = cudaGraphCreate(&g, 0);
    if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
    mfe_status st = MFE_OK;
    if (e == cudaSuccess) {
      ctx->stream = s;
      e = cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
      if (e == cudaSuccess) {
        k_mx_begin<<<1, 1, 0, s>>>(B.st, h);
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
        // body: the iteration up to the update decision, then a conditional
        // node holding the reliable update, entered only when it is due
        cudaGraph_t body = cp->conditional.phGraph_out[0];
        cudaGraphConditionalHandle hu = 0;
        e = cudaGraphConditionalHandleCreate(&hu, body, 0, 0);
        if (e == cudaSuccess)
          e = cudaStreamBeginCaptureToGraph(s, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
        cudaGraphNode_t leaf[4];
        size_t nleaf = 0;
        if (e == cudaSuccess) {
          st = launch_iter(ctx, A32, A64, b, x, B, h, hu, 1);
          cudaStreamCaptureStatus cs;
          const cudaGraphNode_t* deps = nullptr;
          size_t nd = 0;
          cudaError_t e1 = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &deps, nullptr, &nd);
          if (e1 == cudaSuccess && nd >= 1 && nd <= 4) {
            for (size_t i = 0; i < nd; ++i) leaf[i] = deps[i];
            nleaf = nd;
          } else if (e1 == cudaSuccess) {
            e1 = cudaErrorUnknown;
          }
          cudaGraph_t tmp;
          cudaError_t e2 = cudaStreamEndCapture(s, &tmp);
          if (e == cudaSuccess) e = e1;
          if (e == cudaSuccess) e = e2;
        }
        alignas(cudaGraphNodeParams) unsigned char up_buf[sizeof(cudaGraphNodeParams)];
        memset(up_buf, 0, sizeof(up_buf));
        cudaGraphNodeParams* up = reinterpret_cast<cudaGraphNodeParams*>(up_buf);
        up->type = cudaGraphNodeTypeConditional;
        up->conditional.handle = hu;
        up->conditional.type = cudaGraphCondTypeIf;
        up->conditional.size = 1;
        cudaGraphNode_t unode;
        if (e == cudaSuccess && st == MFE_OK) e = cudaGraphAddNode(&unode, body, leaf, nullptr, nleaf, up);
        if (e == cudaSuccess && st == MFE_OK) {
          cudaGraph_t ubody = up->conditional.phGraph_out[0];
          e = cudaStreamBeginCaptureToGraph(s, ubody, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
          if (e == cudaSuccess) {
            st = launch_update(ctx, A64, b, x, B, h, 1);
            cudaGraph_t tmp;
            cudaError_t e2 = cudaStreamEndCapture(s, &tmp);
            if (e == cudaSuccess) e = e2;
          }
        }
      }
      ctx->stream = run_stream;
      if (e == cudaSuccess && st == MFE_OK) e = cudaGraphInstantiate(&ex, g, 0);
      if (e == cudaSuccess && st == MFE_OK) e = cudaGraphLaunch(ex, ctx->stream);
    }
    if (ex) cudaGraphExecDestroy(ex);
    if (g) cudaGraphDestroy(g);
    if (st != MFE_OK) return st;
    if (e != cudaSuccess) return cuda_fail(ctx, e, "mixed CG graph");
  }
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, B.st, sizeof(MixState), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  if (hs->err) return fail(ctx, MFE_TIMEOUT, "a bounded device wait gave up during mixed CG");
  // the FP64 residual products report their bounded waits in the context's word
  MFE_TRY(take_spmv_error(ctx));
  res->num_iters = hs->k;
  res->normr = hs->normr_true;
  res->normr0 = hs->normr0;
  res->final_resid = hs->normr_true;
  for (double& t : res->times) t = 0.0;
  res->times[4] = ms * 1e-3;
  res->refinements = hs->updates;
  res->fp64_spmvs = hs->updates + 1;
  res->inner_operator = B.stencil ? MFE_INNER_STENCIL : MFE_INNER_VALUES;
  mfe_status status = MFE_OK;
  if (hs->status != 0) status = MFE_BREAKDOWN;
  else if (hs->normr_true > hs->tol_abs) status = MFE_MAXITER;
  res->status = status;
  if (o->record_history) {
    const int cnt = hs->k + 1;
    ctx->history.resize(cnt);
    MFE_CUDA_TRY(ctx, cudaMemcpy(ctx->history.data(), B.history, sizeof(double) * cnt,
                                 cudaMemcpyDeviceToHost));
  } else {
    ctx->history.clear();
  }
  return status;
}

}  // namespace mfe
