// Internal declarations shared by the minife_gb300 translation units.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "minife_gb300.h"

struct mfe_cg_graph;  // cached CUDA graph of the CG loop (mfe_cg.cu)

struct mfe_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  // named device workspace, grown on demand and owned by the context
  struct Buf {
    void* ptr = nullptr;
    size_t bytes = 0;
  };
  std::map<std::string, Buf> ws;
  // pinned host scratch for small device->host reads
  void* host_scratch = nullptr;
  size_t host_scratch_bytes = 0;
  mfe_cg_graph* cg_graph = nullptr;
  std::vector<double> history;
  mfe_csr f32_copy{};
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  // mfe_inject_wait_timeout: the next SpMV with a staging ring (the box
  // kernel, the warp-staged CSR and ELL kernels) launched outside a graph
  // capture withholds its copies; its waits give up after this long
  uint64_t inject_wait_ns = 0;
  // launch shape of the multi-RHS stencil SpMM (mfe_multi_set_tuning): z
  // steps per work item, 0 = the default
  int multi_zchunk = 0;
  // the host drop-in call's second stream (the values copy and the operator
  // check beside a solve already running), its event and a pinned buffer
  cudaStream_t side_stream = nullptr;
  cudaEvent_t ev_side = nullptr;
  void* side_pinned = nullptr;
};

namespace mfe {

// Record a failure on ctx and return its status.
mfe_status fail(mfe_ctx* ctx, mfe_status st, const std::string& msg);
mfe_status cuda_fail(mfe_ctx* ctx, cudaError_t e, const char* where);
// Check the last launch; returns MFE_OK or MFE_CUDA_ERR.
mfe_status check_launch(mfe_ctx* ctx, const char* where);

// Read and clear the error word of the SpMV/SpMM launches that carry no
// solver state (ERR_WAIT_TIMEOUT / ERR_TILE_OVERFLOW): MFE_TIMEOUT if set.
mfe_status take_spmv_error(mfe_ctx* ctx);

// Named workspace buffer of at least `bytes` (contents undefined when grown).
void* workspace(mfe_ctx* ctx, const char* name, size_t bytes);
// Pinned host scratch of at least `bytes`.
void* host_scratch(mfe_ctx* ctx, size_t bytes);

// Blocks of `kernel` (threads per block, dynamic shared memory) resident at
// once on the context's device: occupancy x SM count, cached per kernel and
// device.  Grid-stride kernels sized to it run in one wave instead of a full
// wave plus a partial one.  Call it once before a graph capture.
int resident_blocks(mfe_ctx* ctx, const void* kernel, int threads, size_t smem);

// ---- assembly (mfe_assemble.cu) ----
mfe_status launch_structure(mfe_ctx* ctx, int nx, int ny, int nz, int32_t* ro, int32_t* cols);
mfe_status launch_assemble(mfe_ctx* ctx, int nx, int ny, int nz, const double* kappa,
                           const int32_t* ro, double* vals, double* b, int impose_bc);
mfe_status launch_impose_dirichlet(mfe_ctx* ctx, const mfe_csr* A, double* b, double value,
                                   const int32_t* bc_rows, int64_t n_bc);
mfe_status launch_convert_f32(mfe_ctx* ctx, const double* src, float* dst, int64_t n);
mfe_status launch_verify(mfe_ctx* ctx, int nx, int ny, int nz, const double* x, int whole,
                         double* max_err_host);
mfe_status launch_element_gradient(mfe_ctx* ctx, int nx, int ny, int nz, const double* u,
                                   const double* lambda, double* g);
mfe_status launch_zero_boundary(mfe_ctx* ctx, int nx, int ny, int nz, double* v);
int64_t box_nnz(int nx, int ny, int nz);

// ---- SpMV (mfe_spmv.cu) ----
struct DotSink {
  double* partials = nullptr;  // >= grid blocks
  unsigned* ticket = nullptr;
  double* out = nullptr;       // device scalar receiving the dot
};
int spmv_grid(mfe_ctx* ctx, const mfe_csr* A);
mfe_status ensure_max_row_len(mfe_ctx* ctx, const mfe_csr* A, int* max_len);
// y = A x, optionally with x.y (FP64-accumulated) into sink.out.  When
// resid_b != nullptr the kernel instead writes y = b - A x and the dot is y.y.
mfe_status launch_spmv(mfe_ctx* ctx, const mfe_csr* A, const void* x, void* y,
                       const DotSink* sink, const double* resid_b, void* cg_state);
mfe_status launch_spmm(mfe_ctx* ctx, const mfe_csr* A, int nrhs, const void* X, void* Y);
// the pending mfe_inject_wait_timeout for a launch that runs now (0: none);
// consumes it
mfe_status take_wait_injection(mfe_ctx* ctx, uint64_t* withhold_ns);
// y = E x or r = b - E x with r.r for the row-major ELL matrix (rows of up
// to 64 entries and 16-byte aligned arrays on the warp-staged kernel; other
// matrices, and products with x.y, through its CSR view)
mfe_status launch_spmv_ell(mfe_ctx* ctx, const mfe_ell* E, const void* x, void* y,
                           const DotSink* sink, const double* resid_b, void* cg_state);

// ---- box-structured SpMV (mfe_spmv_box.cu) ----
// True when A carries box dimensions consistent with its sizes (the caller
// vouches that its CSR layout is the 27-point box's).
bool csr_is_box(const mfe_csr* A);
// Infer box dimensions from row 0 and verify every row offset and column
// against the closed form; *nx = *ny = *nz = 0 when A is not a box matrix.
mfe_status detect_box(mfe_ctx* ctx, const mfe_csr* A, int* nx, int* ny, int* nz);
mfe_status launch_spmv_box(mfe_ctx* ctx, const mfe_csr* A, const void* x, void* y,
                           const DotSink* sink, const double* resid_b, void* cg_state);
// r32 = (float)(b - A64 x), ||b - A64 x||^2 (FP64) into sink->out; when gate
// is set the launch does nothing unless *gate != 0 (read on the device).
// r32_pad > 0: r32 has rows of Nx + r32_pad entries (x-padded layout).
mfe_status launch_box_resid_f32out(mfe_ctx* ctx, const mfe_csr* A64, const double* x,
                                   const double* b, float* r32, const DotSink* sink,
                                   const int* gate, int r32_pad = 0);

// ---- FP32 stencil operator of the mixed solver (mfe_stencil.cu) ----
// The stencil SpMV works on x-padded vectors: node (ix, iy, iz) at
// (iz * Ny + iy) * Nxp + ix with Nxp = Nx rounded up to a multiple of 4; the
// entries ix >= Nx are zero.  stencil_pitch is Nxp, stencil_rows the padded
// length, stencil_ghost the zero rows needed on both sides of the vector the
// SpMV reads.
int stencil_pitch(const mfe_csr* A);
int64_t stencil_rows(const mfe_csr* A);
int64_t stencil_ghost(const mfe_csr* A);
// checks that A64 is a miniFE box operator (Dirichlet rows dd * I, interior
// rows one 27-point stencil with Dirichlet neighbours zeroed) to FP32
// accuracy, row by row; on success coef[0..26] is the interior stencil in
// slot order (dz, dy, dx) and coef[27] = dd
mfe_status stencil_prepare(mfe_ctx* ctx, const mfe_csr* A64, float* coef, bool* ok);
// the same for one box of Nx x Ny x Nz nodes whose CSR values start at vals
mfe_status stencil_prepare_box(mfe_ctx* ctx, int Nx, int Ny, int Nz, const double* vals, float* coef,
                               bool* ok);
// the 8 mirror-class weights of a verified stencil (coef[0..26] slot order
// (dz, dy, dx)): weight 4|dz| + 2|dy| + |dx| is the entry at (|dz|, |dy|,
// |dx|); true when every entry lies within 2^-22 max|coef| of its class
// weight (the operator then stays within 2^-21 of every row of A)
bool stencil_mirror_classes(const float* coef, float* w8);
// resident CTAs (one wave) of the stencil SpMV variant coef selects
mfe_status stencil_grid(mfe_ctx* ctx, const float* coef, int* grid);
// y = S x and x.y into sink->out (the eight class weights when the stencil
// is mirror-symmetric, else the 27 coefficients), both x-padded (y's padding entries are
// written as zeros); x has stencil_ghost rows of zeros on both sides
mfe_status launch_spmv_stencil(mfe_ctx* ctx, const mfe_csr* A, const float* coef, const float* x,
                               float* y, const DotSink* sink, int grid, unsigned* err);

// ---- FP64 stencil operator of the FP64 CG (mfe_stencil64.cu; its check in
// mfe_stencil.cu) ----
// Tolerance of the FP64 operator: every entry of A within 2^-kSt64TolExp of
// its row's largest magnitude from its class row, every class-row entry
// within the same bound of its mirror-class weight, so the operator stays
// within 2^-(kSt64TolExp - 1) of every entry of A.
constexpr int kSt64TolExp = 40;
// checks that A64 is a miniFE box operator whose interior stencil is
// mirror-symmetric, to the FP64 bound above, row by row on the device; on
// success w8[c] is the weight of class c = 4|dz| + 2|dy| + |dx| and dd the
// Dirichlet diagonal
mfe_status stencil64_prepare(mfe_ctx* ctx, const mfe_csr* A64, double* w8, double* dd, bool* ok);
// The same check split for a matrix still on its way from host memory (the
// host drop-in call): stencil64_host_classes reads the 125 class rows of the
// HOST values of a CSR laid out as the box's (Nx x Ny x Nz nodes) into table
// (kSt64TableLen doubles), checks them against the model and the mirror
// classes and spot-checks rows spread over the box against them (a predictor
// only); stencil64_verify_on then checks every entry on the device against
// the table (already on the device), on stream s, setting *bad (device)
// nonzero on any mismatch.
constexpr int kSt64TableLen = 125 * 28;
bool stencil64_host_classes(int Nx, int Ny, int Nz, const double* vals, double* table, double* w8,
                            double* dd);
mfe_status stencil64_verify_on(mfe_ctx* ctx, cudaStream_t s, int Nx, int Ny, int Nz,
                               const double* vals, const double* table, unsigned* bad);
// y = S x in FP64 on natural-layout vectors (A's box dimensions), with x.y
// into the CG state (pAp and the breakdown pre-test) when cg_state is set,
// else into sink->out (when sink is set)
mfe_status launch_spmv_st64(mfe_ctx* ctx, const mfe_csr* A, const double* w8, double dd,
                            const double* x, double* y, const DotSink* sink, void* cg_state);

// ---- mixed-precision CG (mfe_mixed.cu) ----
// Reliable-update policy options of the mixed solvers: an update is due once
// the recursive residual has fallen by inner_tol since the last one (0: 0.01,
// a drop FP32 recursions follow closely; tenfold updates cost more FP64
// residual SpMVs for the same iteration count),
// and max_refine caps the number of updates (0: no cap; the solve then stops
// with MFE_MAXITER unless it converged).
inline bool mixed_opts_valid(const mfe_cg_opts* o)
{
  return o->inner_tol >= 0.0 && o->inner_tol < 1.0 && o->max_refine >= 0;
}
inline double mixed_delta2(const mfe_cg_opts* o)
{
  const double t = o->inner_tol > 0.0 ? o->inner_tol : 0.01;
  return t * t;
}

mfe_status cg_mixed(mfe_ctx* ctx, const mfe_csr* A64, const double* b, double* x,
                    const mfe_cg_opts* opts, mfe_cg_result* res);

// ---- adjoint gradient (mfe_adjoint.cu) ----
mfe_status adjoint_grad(mfe_ctx* ctx, int nx, int ny, int nz, const double* kappa,
                        const double* u_target, const mfe_cg_opts* opts, double* u_out,
                        double* grad, double* loss, mfe_cg_result* fwd, mfe_cg_result* adj);

// ---- the reference's ELL matrix (mfe_ell.cu) ----
mfe_status launch_csr_to_ell(mfe_ctx* ctx, const mfe_csr* A, mfe_ell* E);
// CSR view of an ELL matrix (row offsets r * ncols_per_row, cached in workspace)
mfe_status ell_view(mfe_ctx* ctx, const mfe_ell* E, mfe_csr* V);
// sliced ELL (mfe_sell): entries of a copy of nrows rows of K entries
int64_t sell_entries(int64_t nrows, int K);
// S->cols / S->vals allocated by the caller; E FP64
mfe_status launch_ell_to_sell(mfe_ctx* ctx, const mfe_ell* E, mfe_sell* S);
// the same from an FP64 CSR whose rows hold at most K entries
mfe_status launch_csr_to_sell(mfe_ctx* ctx, const mfe_csr* A, int K, mfe_sell* S);
// y = S x; x.y into the CG state (cg_state set) or sink->out (sink set)
mfe_status launch_spmv_sell(mfe_ctx* ctx, const mfe_sell* S, const double* x, double* y,
                            const DotSink* sink, void* cg_state);

// ---- Jacobi-preconditioned CG (mfe_pcg.cu) ----
mfe_status cg_jacobi(mfe_ctx* ctx, const mfe_csr* A, const double* b, double* x,
                     const mfe_cg_opts* opts, mfe_cg_result* res);

// ---- multi-RHS CG (mfe_multi.cu) ----
// True when Y = A X can take the box-structured SpMM (box matrix, nrhs
// dividing 32, 16-byte aligned values and vectors).
bool spmm_box_eligible(const mfe_csr* A, int nrhs, const void* X, const void* Y);
mfe_status launch_spmm_box(mfe_ctx* ctx, const mfe_csr* A, int nrhs, const void* X, void* Y);
mfe_status cg_multi(mfe_ctx* ctx, const mfe_csr* A64, int nrhs, const double* B, double* X,
                    const mfe_cg_opts* opts, mfe_cg_result* results);

// ---- batched uneven boxes (mfe_batch.cu) ----
mfe_status batch_create(mfe_ctx* ctx, int nbox, const int32_t* dims, mfe_batch** out);
void batch_destroy(mfe_batch* bt);
void batch_info(const mfe_batch* bt, int64_t* rows, int64_t* nnz, double* assembly_s,
                mfe_batch_tuning* tuning);
mfe_status batch_set_tuning(mfe_ctx* ctx, mfe_batch* bt, const mfe_batch_tuning* t);
mfe_status batch_solve(mfe_ctx* ctx, mfe_batch* bt, const mfe_cg_opts* opts, double* x_out,
                       mfe_cg_result* results);
mfe_status batch_solve_boxes(mfe_ctx* ctx, int nbox, const int32_t* dims, const mfe_cg_opts* opts,
                             double* x_out, mfe_cg_result* results);

// ---- BLAS-1 and CG (mfe_cg.cu) ----
mfe_status launch_dot(mfe_ctx* ctx, int64_t n, const double* x, const double* y,
                      double* dev_out);
mfe_status launch_waxpby(mfe_ctx* ctx, int64_t n, double alpha, const double* x, double beta,
                         const double* y, double* w);
mfe_status launch_fused_waxpby(mfe_ctx* ctx, int64_t n, double alpha, const double* x, double beta,
                               const double* y, double* w, double alpha2, const double* x2,
                               double beta2, const double* y2, double* w2);
// out[i] = x[idx[i]], i < n (halo exchange send buffers)
mfe_status launch_gather(mfe_ctx* ctx, int64_t n, const int32_t* idx, const double* x, double* out);
// x.y of FP32 vectors accumulated in double-float (the mixed solvers' dots)
mfe_status launch_dot_f32(mfe_ctx* ctx, int64_t n, const float* x, const float* y, double* dev_out);
mfe_status cg_solve_impl(mfe_ctx* ctx, const mfe_csr* A, const double* b, double* x,
                         const mfe_cg_opts* opts, mfe_cg_result* res);
// An FP64 stencil solve started before the matrix values are on the device
// (the host drop-in call): x0 must be zero (checked on the device), the
// operator's weights come from the host copy of the matrix, and confirm()
// runs once before anything reads the CSR values or the solve returns a
// result.  It must make ctx->stream wait for the values and return whether
// the layout and every entry passed their checks.  cg_solve_spec returns
// kSpecFailed when x0 is not zero, the tolerance is below the operator's
// gate or confirm() returns false; x on the device is then undefined.
struct CgSpec {
  double w8[8];
  double dd;
  bool (*confirm)(void* arg);
  void* arg;
};
constexpr mfe_status kSpecFailed = (mfe_status)1000;
mfe_status cg_solve_spec(mfe_ctx* ctx, const mfe_csr* A, const double* b, double* x,
                         const mfe_cg_opts* opts, mfe_cg_result* res, const CgSpec* spec);
// FP64 CG (no preconditioner) whose iterations' products run on the sliced
// ELL copy S of the matrix V (an ELL view); the initial residual uses the
// row-major ELL E itself when given, else V
mfe_status cg_solve_sell(mfe_ctx* ctx, const mfe_csr* V, const mfe_sell* S, const double* b,
                         double* x, const mfe_cg_opts* opts, mfe_cg_result* res,
                         const mfe_ell* E = nullptr);
void cg_graph_destroy(mfe_cg_graph* g);

}  // namespace mfe

#define MFE_CUDA_TRY(ctx, expr)                                      \
  do {                                                               \
    cudaError_t _e = (expr);                                         \
    if (_e != cudaSuccess) return ::mfe::cuda_fail((ctx), _e, #expr); \
  } while (0)

#define MFE_TRY(expr)                  \
  do {                                 \
    mfe_status _s = (expr);            \
    if (_s != MFE_OK) return _s;       \
  } while (0)
