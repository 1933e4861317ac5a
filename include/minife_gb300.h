/*
 * minife_gb300 -- C ABI of the GB300 (sm_103a) implementation of miniFE's
 * assemble-and-solve path.
 *
 * The reference (Mantevo miniFE, ref/ variant) binds this path at compile time
 * through C++ templates: cg_solve takes the matvec as a functor argument and
 * the CSRMatrix / Vector types by macro.  This header is the drop-in boundary
 * for that path as plain C: every entry point takes POD structs, raw pointers
 * and sizes, runs hand-written CUDA kernels on one GPU, and returns an
 * mfe_status.  Each declaration names the reference interface it replaces
 * (file:line in the reference repository).  There is no CPU fallback: a call
 * without a usable GPU returns MFE_CUDA_ERR.
 *
 * Conventions
 *  - "device" pointers are CUDA device addresses (cudaMalloc, or the data
 *    pointer of a CUDA tensor); "host" pointers are ordinary host memory
 *    (pinned memory gives the fastest copies).
 *  - One context = one CUDA stream on one device.  Calls on one context are
 *    ordered on its stream; a context is not thread-safe, distinct contexts
 *    are independent.  Entry points that return a value to the host
 *    (mfe_dot, mfe_cg_solve) synchronise the stream before returning.
 *  - Indices are 32-bit like the reference's LocalOrdinal/GlobalOrdinal = int
 *    (ref/src/Makefile:3-6); boxes whose nonzero count reaches 2^31 are
 *    rejected with MFE_BAD_ARG.
 */
#ifndef MINIFE_GB300_H
#define MINIFE_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MFE_ABI_VERSION 3

typedef enum mfe_status {
  MFE_OK = 0,
  MFE_BAD_ARG = 1,       /* invalid dimensions, null pointers, size overflow */
  MFE_OOM = 2,           /* device allocation failed */
  MFE_CUDA_ERR = 3,      /* CUDA runtime error (no device, launch failure) */
  MFE_BREAKDOWN = 4,     /* CG breakdown test fired (cg_solve.hpp:186-198) */
  MFE_MAXITER = 5,       /* returned by the refinement solver only: the target
                            residual was not reached within its limits */
  MFE_TIMEOUT = 6,       /* a bounded device-side wait gave up */
  MFE_NOT_SUPPORTED = 7  /* valid request the library does not implement */
} mfe_status;

typedef enum mfe_dtype { MFE_F64 = 0, MFE_F32 = 1 } mfe_dtype;

typedef struct mfe_ctx mfe_ctx;

/* CSR matrix in device memory, one rank: row i of the reference's
 * CSRMatrix (ref/src/CSRMatrix.hpp:43-129) with rows[i] == i,
 * row_offsets == CSRMatrix::row_offsets, cols == packed_cols,
 * vals == packed_coefs (double for MFE_F64, float for MFE_F32). */
typedef struct mfe_csr {
  int64_t nrows;
  int64_t ncols;
  int64_t nnz;
  int32_t* row_offsets; /* device, nrows + 1 */
  int32_t* cols;        /* device, nnz */
  void* vals;           /* device, nnz of dtype */
  int32_t dtype;        /* mfe_dtype */
  int32_t max_row_len;  /* 0 = unknown (computed on first use) */
  /* box the matrix was assembled on (0 if not an assembled box); lets the
   * solver use the 27-point stencil layout of those rows */
  int32_t box_nx, box_ny, box_nz;
  int32_t owned;        /* 1 if allocated by mfe_csr_alloc */
} mfe_csr;

/* ------------------------------------------------------------------ */
/* context, memory, errors                                             */
/* ------------------------------------------------------------------ */
int mfe_abi_version(void);
mfe_status mfe_ctx_create(int device, mfe_ctx** out);
mfe_status mfe_ctx_destroy(mfe_ctx* ctx);
/* Run this context's work on an existing CUDA stream (cudaStream_t).  NULL
 * selects the CUDA default stream, as it does for CUDA runtime calls. */
mfe_status mfe_set_stream(mfe_ctx* ctx, void* stream);
/* Return to the context's own (non-blocking) stream. */
mfe_status mfe_use_own_stream(mfe_ctx* ctx);
/* Wait for the context's stream.  Returns MFE_TIMEOUT (and clears the
 * condition) when a standalone SpMV/SpMM launched since the last call gave
 * up one of its bounded waits; solver calls report this themselves. */
mfe_status mfe_synchronize(mfe_ctx* ctx);
const char* mfe_last_error_string(const mfe_ctx* ctx);
const char* mfe_status_string(mfe_status s);
/* Number of SMs of the context's device (the grid-size unit). */
int mfe_device_sm_count(const mfe_ctx* ctx);

mfe_status mfe_device_alloc(mfe_ctx* ctx, size_t bytes, void** out);
mfe_status mfe_device_free(mfe_ctx* ctx, void* ptr);
mfe_status mfe_memcpy_h2d(mfe_ctx* ctx, void* dst, const void* src, size_t bytes);
mfe_status mfe_memcpy_d2h(mfe_ctx* ctx, void* dst, const void* src, size_t bytes);

/* Allocate device arrays for an nrows x nrows CSR with nnz nonzeros. */
mfe_status mfe_csr_alloc(mfe_ctx* ctx, int64_t nrows, int64_t nnz, mfe_dtype dtype,
                         mfe_csr* out);
mfe_status mfe_csr_free(mfe_ctx* ctx, mfe_csr* A);

/* ------------------------------------------------------------------ */
/* mesh, structure, assembly, boundary conditions                      */
/* ------------------------------------------------------------------ */

/* Rows and nonzeros of the nx x ny x nz element box (nodes = elements + 1
 * per dimension, 27-point rows): the sizes generate_matrix_structure
 * reserves (ref/src/generate_matrix_structure.hpp:63-130). */
mfe_status mfe_box_dims(int nx, int ny, int nz, int64_t* nrows, int64_t* nnz);

/* generate_matrix_structure + MatrixInitOp<CSR>
 * (ref/src/generate_matrix_structure.hpp:47-149, MatrixInitOp.hpp:127-156):
 * fills A->row_offsets and A->cols (ascending 27-point columns) and zeroes
 * A->vals.  A must be allocated for mfe_box_dims rows/nonzeros. */
mfe_status mfe_generate_structure(mfe_ctx* ctx, int nx, int ny, int nz, mfe_csr* A);

/* assemble_FE_data -> perform_element_loop -> sum_into_global_linear_system
 * (ref/src/assemble_FE_data.hpp:38-73, perform_element_loop.hpp:40-104,
 * SparseMatrix_functions.hpp:183-255): structure, Hex8 element matrices and
 * source vectors (ref/fem/Hex8.hpp:260-410), summed per coefficient in
 * ascending element order, so values match the reference bit for bit.
 * kappa (device, nullable): one conductivity per element in element-id order
 * replacing the constant k = 1.0 of Hex8.hpp:273; NULL = the reference.
 * impose_bc != 0 also applies both impose_dirichlet passes of
 * driver.hpp:214-218 (value 0 on faces x=0,y=0,z=0,y=1,z=1, then value 1 on
 * face x=1), fused into the same kernel.  b (device, nrows doubles) is
 * overwritten.  A->dtype must be MFE_F64. */
mfe_status mfe_assemble(mfe_ctx* ctx, int nx, int ny, int nz, const double* kappa,
                        mfe_csr* A, double* b, int impose_bc);

/* impose_dirichlet (ref/src/SparseMatrix_functions.hpp:434-480) for an
 * arbitrary CSR: bc_rows (device, sorted ascending, n_bc entries) replaces
 * the std::set.  Rows in the set become identity rows with b = value; every
 * other row moves value * (its coefficients in bc columns) to b and zeroes
 * those coefficients, keeping them as explicit zeros. */
mfe_status mfe_impose_dirichlet(mfe_ctx* ctx, mfe_csr* A, double* b, double value,
                                const int32_t* bc_rows, int64_t n_bc);

/* The boundary row sets of simple_mesh_description
 * (ref/src/simple_mesh_description.hpp:62-224) as ascending device arrays:
 * set 0 (faces x=0,y=0,z=0,y=1,z=1) or set 1 (face x=1).  count_out
 * receives the size; rows may be NULL to query the size only. */
mfe_status mfe_box_bc_rows(mfe_ctx* ctx, int nx, int ny, int nz, int which,
                           int32_t* rows, int64_t* count_out);

/* Convert the values of an FP64 CSR into an FP32 copy sharing its structure
 * (dst->row_offsets/cols may alias src's). */
mfe_status mfe_csr_convert_f32(mfe_ctx* ctx, const mfe_csr* src, mfe_csr* dst);

/* ------------------------------------------------------------------ */
/* kernels: matvec, dot, waxpby                                        */
/* ------------------------------------------------------------------ */

/* matvec_std<CSR>::operator() (ref/src/SparseMatrix_functions.hpp:545-578):
 * y = A x.  x and y have A->dtype. */
mfe_status mfe_spmv(mfe_ctx* ctx, const mfe_csr* A, const void* x, void* y);

/* The verified FP64 stencil operator of a miniFE box matrix (no counterpart
 * in the reference; it stands in for matvec_std, SparseMatrix_functions.hpp:
 * 545-578, on the matrices assemble_FE_data builds): eight mirror-class
 * weights w[4|dz| + 2|dy| + |dx|] of the interior 27-point stencil and the
 * Dirichlet diagonal dd, valid for the box's natural-layout vectors. */
typedef struct mfe_stencil64 {
  int32_t box_nx, box_ny, box_nz;  /* elements per dimension */
  int32_t reserved;
  double w[8];
  double dd;
} mfe_stencil64;

/* Check A (FP64, box dimensions set or detectable) on the device, every
 * entry within 2^-40 of its row's largest magnitude from its class value
 * (see mfe_cg_opts.f64_operator), and fill *S.  MFE_NOT_SUPPORTED when A is
 * not such an operator (per-element conductivity, fewer than 4 elements
 * along a dimension, not a box matrix). */
mfe_status mfe_stencil64_from_csr(mfe_ctx* ctx, const mfe_csr* A, mfe_stencil64* S);

/* y = S x (device vectors of the box's rows): 12.5 FP64 operations per row
 * on average instead of the CSR kernel's 27 FMAs; within 2^-39 sum_j
 * |a_ij x_j| (plus rounding) of A x for the A that S was made from. */
mfe_status mfe_spmv_stencil64(mfe_ctx* ctx, const mfe_stencil64* S, const double* x, double* y);

/* matvec_and_dot (ref/src/SparseMatrix_functions.hpp:491-536): y = A x and
 * *result = x . y (double, host), accumulated in FP64.  Blocks for the
 * scalar; returns MFE_TIMEOUT if the product gave up a bounded wait. */
mfe_status mfe_matvec_and_dot(mfe_ctx* ctx, const mfe_csr* A, const void* x, void* y,
                              double* result);

/* dot (ref/src/Vector_functions.hpp:194-226): *result (host) = x . y. */
mfe_status mfe_dot(mfe_ctx* ctx, int64_t n, const double* x, const double* y,
                   double* result);

/* Allocation-free dot product, for callers that may not allocate device
 * memory: applications whose GPU memory belongs to another allocator (a host
 * program or framework that reserves the device in its own pool and lets no
 * plugin allocate beside it) and latency-critical loops that cannot take the
 * implicit synchronisation of cudaMalloc/cudaFree.  No counterpart in the
 * reference.
 *
 * *result (DEVICE pointer, one double) = x . y, accumulated in FP64 in fixed
 * 8192-element chunks (deterministic for a given n), computed on the calling
 * thread's current device and on `stream` (cudaStream_t, NULL = default
 * stream); the call returns once the work is queued.  No context is needed
 * and nothing is allocated: the chunk partial sums live in a 512 KiB device
 * array inside the library (held by every GPU that loads the library until
 * the process exits).  The first call on each device resolves that array's
 * device address (cudaGetSymbolAddress) and should come before any stream
 * capture; calls outside a capture resolve it again, so the entry point
 * stays valid after a device reset, while calls during a capture use the
 * address resolved before it.  n > MFE_DOT_NOALLOC_MAX_N returns MFE_BAD_ARG
 * and launches nothing.  All calls share the array, so calls that overlap on
 * the GPU race: order them on one stream. */
#define MFE_DOT_NOALLOC_MAX_N ((int64_t)536870912) /* 2^29 elements */
mfe_status mfe_dot_noalloc(int64_t n, const double* x, const double* y, double* result,
                           void* stream);

/* waxpby (ref/src/Vector_functions.hpp:127-150): w = alpha x + beta y. */
mfe_status mfe_waxpby(mfe_ctx* ctx, int64_t n, double alpha, const double* x,
                      double beta, const double* y, double* w);

/* fused_waxpby (ref/src/Vector_functions.hpp:154-185): w = alpha x + beta y
 * and w2 = alpha2 x2 + beta2 y2 in one pass over the vectors. */
mfe_status mfe_fused_waxpby(mfe_ctx* ctx, int64_t n, double alpha, const double* x,
                            double beta, const double* y, double* w, double alpha2,
                            const double* x2, double beta2, const double* y2, double* w2);

/* Packing of a halo exchange (exchange_externals.hpp:122-124, send_buffer[i]
 * = x[elements_to_send[i]]): out[i] = x[idx[i]] for i < n, all device
 * arrays; idx entries must index x. */
mfe_status mfe_gather(mfe_ctx* ctx, int64_t n, const int32_t* idx, const double* x, double* out);

/* Dot product of FP32 vectors (device) as the mixed-precision solvers form
 * their alpha/beta and residual reductions: every product and sum in
 * double-float on the FP32 pipe (TwoProduct + TwoSum, about 48 significant
 * bits), *result (host) the FP64 sum of the final pair.  No counterpart in
 * the reference (its dot over Vector<float> returns float,
 * Vector_functions.hpp:194-226). */
mfe_status mfe_dot_f32(mfe_ctx* ctx, int64_t n, const float* x, const float* y,
                       double* result);

/* Fault injection for tests of the bounded-wait error path; no counterpart
 * in the reference.  The next SpMV with a shared-memory staging ring (the
 * box-structured kernel, or the warp-staged kernels of an FP64 CSR with rows
 * of at most 32 entries and of the ELL matrix) launched on ctx outside a
 * graph capture issues none of its copies, so its bounded waits run out
 * after wait_ns nanoseconds (1 ms .. 2 s) with no copy in flight; the call
 * that launched it returns MFE_TIMEOUT (a solve) or mfe_synchronize does
 * (mfe_spmv, mfe_spmv_ell).  The context stays usable. */
mfe_status mfe_inject_wait_timeout(mfe_ctx* ctx, int64_t wait_ns);

/* ------------------------------------------------------------------ */
/* CG                                                                  */
/* ------------------------------------------------------------------ */
typedef enum mfe_precision {
  MFE_PREC_F64 = 0,   /* the reference's FP64 CG */
  MFE_PREC_MIXED = 1  /* FP32 inner CG (FP32 matrix and vectors, FP64 dots)
                         inside FP64 iterative refinement */
} mfe_precision;

typedef enum mfe_tol_mode {
  MFE_TOL_ABSOLUTE = 0, /* the reference's test normr > tol (cg_solve.hpp:152) */
  MFE_TOL_RELATIVE = 1  /* normr > tol * ||b - A x0|| */
} mfe_tol_mode;

typedef struct mfe_cg_opts {
  int32_t max_iter;     /* reference: 200 (driver.hpp:241) */
  int32_t tol_mode;     /* mfe_tol_mode */
  double tol;           /* reference: DBL_EPSILON absolute (driver.hpp:245) */
  int32_t precision;    /* mfe_precision */
  int32_t refine_k;     /* mixed: max inner iterations per refinement sweep
                           (0 = library default: 100 for one box, 50 for
                           batched boxes and multiple right-hand sides) */
  double inner_tol;     /* mixed: a reliable update is due once the recursive
                           residual fell by this factor since the last one;
                           [0, 1), 0 = 0.01 */
  int32_t max_refine;   /* mixed: max reliable updates; the solve stops with
                           MFE_MAXITER after that many unless converged
                           (0 = no cap) */
  int32_t record_history; /* 1: keep normr of every iteration (see
                             mfe_cg_history) */
  const mfe_csr* A32;   /* mixed: optional prepared FP32 copy of A (NULL: the
                           library uses its stencil operator or converts a
                           copy on every call, see mixed_operator) */
  int32_t precond;      /* mfe_cg_solve: 0 none (the reference's CG), 1 Jacobi
                           (M = diag(A), FP64; stops on ||r|| after the update;
                           its products follow f64_operator as well, a
                           stencil solve stopping on ||b - A x|| with the CSR
                           values) */
  int32_t mixed_operator; /* mixed solves (mfe_cg_solve, mfe_batch_solve):
                           0 = the FP32 stencil operator (28 numbers: the
                           interior 27-point stencil and the Dirichlet
                           diagonal) when A is a miniFE box operator: every
                           row is dd * x_r (Dirichlet node) or the interior
                           stencil with the Dirichlet neighbours zeroed, every
                           entry within 2^-22 of its row's largest magnitude
                           (checked on the device on every call; once per
                           batch handle), else the FP32 copy of the values
                           (padded values for batches); 1 = always the FP32
                           values.  mfe_cg_result.inner_operator reports
                           which ran. */
  int32_t f64_operator; /* FP64 solves (mfe_cg_solve, with or without Jacobi):
                           0 = the verified FP64 stencil operator when A is a
                           miniFE box operator whose interior stencil is
                           mirror-symmetric (every box miniFE assembles with
                           k = 1) and the tolerance is at least 2^-36 of the
                           initial residual: every row is dd * x_r (Dirichlet node) or
                           the interior stencil with the Dirichlet neighbours
                           zeroed, every entry within 2^-40 of its row's
                           largest magnitude from its class value (checked on
                           the device on every call), so the operator is
                           within 2^-39 of every entry of A; the solve then
                           stops only once ||b - A x|| computed with the CSR
                           values meets the tolerance (restarting CG from x
                           with that residual otherwise).  Else, and with
                           1, the CSR values (matvec_std).
                           mfe_cg_result.inner_operator reports which ran. */
} mfe_cg_opts;

/* Fill opts with the reference's defaults (max_iter 200, absolute tol
 * DBL_EPSILON, FP64). */
void mfe_cg_opts_default(mfe_cg_opts* opts);

typedef struct mfe_cg_result {
  int32_t num_iters;    /* cg_solve's num_iters (total inner iterations for
                           the mixed solver) */
  int32_t status;       /* mfe_status of the solve */
  double normr;         /* cg_solve's normr: residual norm at the top of the
                           last iteration (FP64 true residual for mixed) */
  double normr0;        /* initial residual norm */
  double final_resid;   /* ||b - A x|| of the returned x, FP64 */
  double times[5];      /* seconds: WAXPY, DOT, MATVEC, MATVECDOT, TOTAL
                           (mytimer.hpp:37-43 order); fused kernels are
                           accounted to MATVECDOT and WAXPY */
  int32_t refinements;  /* mixed: outer refinement sweeps */
  int32_t fp64_spmvs;   /* number of matvecs with the FP64 CSR values */
  int32_t inner_operator; /* the operator of the CG iteration, one of
                             mfe_inner_operator: for mixed solves the FP32
                             one; for FP64 solves MFE_INNER_STENCIL64 or 0
                             (the CSR values) */
} mfe_cg_result;

/* mfe_cg_result.inner_operator */
typedef enum mfe_inner_operator {
  MFE_INNER_NONE = 0,
  MFE_INNER_STENCIL = 1,  /* verified 27-coefficient stencil (x and y only) */
  MFE_INNER_VALUES = 2,   /* FP32 copy of the CSR values */
  MFE_INNER_PADDED = 3,   /* FP32 values padded to fixed-length rows */
  MFE_INNER_STENCIL64 = 4 /* FP64 solves: the verified FP64 stencil operator
                             (eight mirror-class weights and the Dirichlet
                             diagonal; see mfe_cg_opts.f64_operator) */
} mfe_inner_operator;

/* cg_solve (ref/src/cg_solve.hpp:69-229): solves A x = b from the initial
 * guess in x (device).  FP64 precision follows the reference's loop exactly
 * (x0 copied to p, r = b - A p, then per iteration p update, A p, p.Ap,
 * breakdown test, x and r updates), with matvec_std on the CSR values or,
 * for verified miniFE box operators, the FP64 stencil operator
 * (opts->f64_operator); the loop runs on the device inside one CUDA graph (a
 * conditional while node), with no host round trip per iteration. */
mfe_status mfe_cg_solve(mfe_ctx* ctx, const mfe_csr* A, const double* b, double* x,
                        const mfe_cg_opts* opts, mfe_cg_result* result);

/* Drop-in for the reference's host-side call: CSR and vectors in HOST
 * memory (CSRMatrix/Vector storage), copied to the device, solved with
 * mfe_cg_solve, and x copied back.  For an FP64 solve without preconditioner
 * the host threads check, while the values are being copied, whether the
 * row offsets and columns are the 27-point box layout of some nx x ny x nz
 * box; if they are, only the values and vectors are copied (the solver
 * reads a box's structure in closed form), otherwise the structure too.
 * With x0 = 0 and the default FP64 operator the solve does not wait for the
 * copy: the verified FP64 stencil's weights are read from the host arrays
 * and the CG starts at once, while a second stream of ctx copies the values
 * and checks every entry on the device and a host thread checks the layout;
 * the result counts only after all three have passed (else the ordinary
 * solve runs from x0).  Nothing of the call is in flight when it returns. */
mfe_status mfe_cg_solve_host(mfe_ctx* ctx, int64_t nrows, int64_t nnz,
                             const int32_t* row_offsets, const int32_t* cols,
                             const double* vals, const double* b, double* x,
                             const mfe_cg_opts* opts, mfe_cg_result* result);

/* History of normr recorded by the last mfe_cg_solve on ctx with
 * record_history = 1: up to cap values (host), index 0 = initial residual. */
mfe_status mfe_cg_history(mfe_ctx* ctx, double* out, int32_t cap, int32_t* count);

/* ------------------------------------------------------------------ */
/* verification, adjoint, batching                                     */
/* ------------------------------------------------------------------ */

/* verify_solution (ref/fem/verify_solution.hpp:55-174, analytic_soln.hpp):
 * max |x - analytic| over nodes within 0.05 of the centre (all nodes when
 * whole_domain), 300 x 300 series terms, evaluated on the device.
 * *passed = max_err <= tolerance. */
mfe_status mfe_verify_solution(mfe_ctx* ctx, int nx, int ny, int nz, const double* x,
                               double tolerance, int whole_domain, double* max_err,
                               int* passed);

/* Adjoint contraction for per-element conductivity (extension of
 * Hex8.hpp:273): g[e] = -lambda_e^T Khat_e u_e, Khat_e the k = 1 element
 * matrix of element e, u and lambda nodal (device), g per element (device). */
mfe_status mfe_element_gradient(mfe_ctx* ctx, int nx, int ny, int nz, const double* u,
                                const double* lambda, double* g);

/* The whole adjoint gradient in one call: L = 1/2 ||u - u_target||^2 over all
 * nodes, u solving the box problem assembled with per-element conductivity
 * kappa (device, nx*ny*nz; NULL: k = 1 everywhere); grad (device, nx*ny*nz)
 * receives dL/dkappa: forward CG, adjoint CG on (u - u_target) with its
 * Dirichlet rows zeroed, element contraction (mfe_element_gradient).  opts
 * (relative tolerance recommended) serve both solves; u_out (device, rows),
 * loss (host), fwd and adj (host results) may be NULL. */
mfe_status mfe_adjoint_grad(mfe_ctx* ctx, int nx, int ny, int nz, const double* kappa,
                            const double* u_target, const mfe_cg_opts* opts, double* u_out,
                            double* grad, double* loss, mfe_cg_result* fwd,
                            mfe_cg_result* adj);

/* v[r] = 0 on every Dirichlet row of the box (faces of both boundary sets of
 * simple_mesh_description.hpp:62-224).  Used to form the adjoint right-hand
 * side of a box solve, which must vanish on the prescribed rows. */
mfe_status mfe_box_zero_boundary(mfe_ctx* ctx, int nx, int ny, int nz, double* v);

/* Multi-RHS: Y = A X for nrhs column vectors stored row-major (X[i*nrhs + j]),
 * reading A once per product.  FP64 or FP32 by A->dtype (X, Y same type).
 * Box matrices with nrhs dividing 32 and 16-byte aligned arrays take the
 * staged box kernel (one warp per row, one lane per column); others a
 * thread-per-(row, column) CSR kernel. */
mfe_status mfe_spmm(mfe_ctx* ctx, const mfe_csr* A, int32_t nrhs, const void* X, void* Y);

/* Launch shape of the multi-RHS solver on ctx (the autotuner's knob; no
 * counterpart in the reference): z_chunk = z steps per work item of the
 * 32-column stencil SpMM, 4..1024 (0 = the default, 32). */
typedef struct mfe_multi_tuning {
  int32_t z_chunk;
} mfe_multi_tuning;
mfe_status mfe_multi_set_tuning(mfe_ctx* ctx, const mfe_multi_tuning* t);

/* Multi-RHS CG on one matrix: nrhs independent CG solves (each with its own
 * alpha/beta and stopping test) advanced together so every iteration reads A
 * once.  B, X row-major (i*nrhs + j), device, FP64; opts as for mfe_cg_solve
 * (FP64 or MIXED).  results: nrhs entries (host). */
mfe_status mfe_cg_solve_multi(mfe_ctx* ctx, const mfe_csr* A, int32_t nrhs, const double* B,
                              double* X, const mfe_cg_opts* opts, mfe_cg_result* results);

/* Batched uneven boxes: nbox (1..1024) independent miniFE problems
 * (dims[3*i..3*i+2] = nx, ny, nz), each assembled as the reference does
 * (k = 1, its Dirichlet faces) into one concatenated device store, then
 * solved with CG, all boxes advancing together: one CUDA graph whose while
 * loop runs the iterations, each launch walking only the boxes still
 * iterating.  opts as for mfe_cg_solve (FP64: the reference's CG per box;
 * MIXED: FP32 SpMV with FP64 reliable updates, each box stopping on its true
 * FP64 residual).  x_out (device) receives the concatenated solutions (box i
 * at the prefix sum of the rows of boxes < i); results: nbox entries (host),
 * times[0] = assembly of the batch, times[4] = the batched solve (s).
 * mfe_batch_solve_boxes = create + solve + destroy. */
mfe_status mfe_batch_solve_boxes(mfe_ctx* ctx, int32_t nbox, const int32_t* dims,
                                 const mfe_cg_opts* opts, double* x_out,
                                 mfe_cg_result* results);

/* The same in steps: create assembles the batch once (owning its device
 * memory), solve may run any number of times (other tolerances, precision
 * or launch shape), destroy frees it. */
typedef struct mfe_batch mfe_batch;
/* Launch shape of a batched solve (the autotuner's knobs). */
typedef struct mfe_batch_tuning {
  int32_t spmv_rows;    /* rows per FP32 SpMV tile: 128 or 256 (default 256) */
  int32_t spmv_stages;  /* its shared-memory pipeline stages: 2..4 (default 2) */
  int32_t chunk_rows;   /* rows per vector-kernel chunk: 1024..2^20, multiple of 4 (8192) */
} mfe_batch_tuning;
mfe_status mfe_batch_create(mfe_ctx* ctx, int32_t nbox, const int32_t* dims, mfe_batch** out);
mfe_status mfe_batch_set_tuning(mfe_ctx* ctx, mfe_batch* batch, const mfe_batch_tuning* t);
/* rows and nonzeros of all boxes, assembly seconds, current launch shape
 * (any pointer may be NULL). */
mfe_status mfe_batch_info(const mfe_batch* batch, int64_t* rows, int64_t* nnz,
                          double* assembly_seconds, mfe_batch_tuning* tuning);
mfe_status mfe_batch_solve(mfe_ctx* ctx, mfe_batch* batch, const mfe_cg_opts* opts,
                           double* x_out, mfe_cg_result* results);
void mfe_batch_destroy(mfe_batch* batch);

/* ------------------------------------------------------------------ */
/* the reference's ELL matrix                                           */
/* ------------------------------------------------------------------ */

/* ELLMatrix (ref/src/ELLMatrix.hpp, MINIFE_ELL_MATRIX) on the device:
 * ncols_per_row entries per row, row-major (row r at r*ncols_per_row), the
 * row's columns ascending first, then padding entries with column 0 and
 * value 0 (MatrixInitOp<ELLMatrix>, ref/src/MatrixInitOp.hpp:160-220). */
typedef struct mfe_ell {
  int64_t nrows;
  int32_t ncols_per_row;   /* 27 for miniFE's matrices */
  int32_t dtype;           /* mfe_dtype */
  int32_t* cols;           /* device, nrows*ncols_per_row */
  void* vals;              /* device, nrows*ncols_per_row */
} mfe_ell;

/* E->cols/vals (caller-allocated, nrows*ncols_per_row each) and
 * E->ncols_per_row set by the caller; fills them from A (MFE_BAD_ARG if a row
 * is longer than ncols_per_row) and sets E->nrows and E->dtype. */
mfe_status mfe_csr_to_ell(mfe_ctx* ctx, const mfe_csr* A, mfe_ell* E);
/* matvec_std<ELLMatrix> (ref/src/SparseMatrix_functions.hpp:579-611): y = A x,
 * every stored entry summed (padding adds 0 * x[0]). */
mfe_status mfe_spmv_ell(mfe_ctx* ctx, const mfe_ell* E, const void* x, void* y);
/* cg_solve with the ELL matvec (FP64; opts as for mfe_cg_solve).  Without
 * preconditioner the iterations' products run on a sliced copy of E
 * (mfe_sell, made once per call in context workspace); the initial residual
 * r = b - A x0 uses E itself, and the reported final residual is the
 * recursive one, as cg_solve's (ref/src/cg_solve.hpp:152-163). */
mfe_status mfe_cg_solve_ell(mfe_ctx* ctx, const mfe_ell* E, const double* b, double* x,
                            const mfe_cg_opts* opts, mfe_cg_result* result);

/* Sliced ELL: the ELLMatrix layout transposed for the GPU (no counterpart in
 * the reference).  Rows come in slices of 32 and a slice is column-major:
 * entry k of row r sits at ((r / 32) * ncols_per_row + k) * 32 + r % 32, so
 * entry k of 32 consecutive rows is one 256-byte line of values and one
 * 128-byte line of columns.  The arrays hold ceil(nrows / 32) * 32 *
 * ncols_per_row entries; rows past nrows hold column 0, value 0.  FP64. */
typedef struct mfe_sell {
  int64_t nrows;
  int32_t ncols_per_row;
  int32_t reserved;
  int32_t* cols;  /* device */
  double* vals;   /* device */
} mfe_sell;

/* S->cols / S->vals (caller-allocated, ceil(nrows / 32) * 32 * ncols_per_row
 * entries each) filled from the FP64 ELL matrix E; sets S->nrows and
 * S->ncols_per_row. */
mfe_status mfe_ell_to_sell(mfe_ctx* ctx, const mfe_ell* E, mfe_sell* S);
/* y = A x with the sliced copy (every stored entry summed, as the ELL
 * matvec: one FP64 FMA per entry, two partial sums per row). */
mfe_status mfe_spmv_sell(mfe_ctx* ctx, const mfe_sell* S, const double* x, double* y);

/* ------------------------------------------------------------------ */
/* the reference's debug dumps                                          */
/* ------------------------------------------------------------------ */

/* write_matrix / write_vector (ref/src/SparseMatrix_functions.hpp:98-140,
 * ref/src/Vector_functions.hpp:49-82) on one rank: the file is
 * "<filename>.1.0"; matrix: "nrows nnz" then one "row col coef" line per
 * stored entry; vector: "n" then one "index coef" line (index from
 * start_index); numbers in the default std::ostream format (6 significant
 * digits).  Arrays on the device; the call synchronises the stream. */
mfe_status mfe_write_matrix(mfe_ctx* ctx, const mfe_csr* A, const char* filename);
mfe_status mfe_write_vector(mfe_ctx* ctx, int64_t n, const double* x, int64_t start_index,
                            const char* filename);

#ifdef __cplusplus
}
#endif

#endif /* MINIFE_GB300_H */
