/*
 * CPU restatement of miniFE's assemble-and-solve path (oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * product path: only tests/, __graft_entry__.smoke() and bench.py's
 * cpu_baseline / reference legs load it.  Nothing in the product
 * (libminife_gb300.so, the miniFE.x driver, the Python package) links,
 * loads or falls back to it.
 *
 * Every function restates the reference's serial C++ code (Mantevo miniFE,
 * ref/ variant) with the same floating-point operation order, so that for
 * matching inputs the results are bit-identical to ref/src compiled with
 * g++ (no FMA contraction).  Each definition cites the reference file:line
 * it follows.  Parity of this restatement is pinned against the reference
 * itself (oracle/_ref harness built from the reference sources) by the
 * golden fixtures under tests/golden/.
 */
#ifndef MINIFE_ORACLE_H
#define MINIFE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Number of node rows / nonzeros of the nx*ny*nz element box (one rank). */
int64_t orc_num_rows(int nx, int ny, int nz);
int64_t orc_num_nonzeros(int nx, int ny, int nz);

/* generate_matrix_structure + MatrixInitOp<CSR>: row_offsets[N+1], cols[nnz]. */
int orc_structure(int nx, int ny, int nz, int32_t* row_offsets, int32_t* cols);

/* compute_gradient_values: 8 gauss points x 8 nodes x 3 = 192 values. */
void orc_gradient_values(double* grad_vals);

/* get_elem_nodes_and_coords for element (ex,ey,ez): 8 node rows, 24 coords. */
void orc_elem_nodes_and_coords(int nx, int ny, int nz, int ex, int ey, int ez,
                               int32_t* node_rows, double* coords);

/* Hex8::diffusionMatrix_symm with conductivity k (reference: k = 1.0). */
void orc_diffusion_matrix_symm(const double* coords, const double* grad_vals,
                               double k, double* elem_mat36);

/* Hex8::sourceVector (Q = 1). */
void orc_source_vector(const double* coords, const double* grad_vals,
                       double* elem_vec8);

/* perform_element_loop: assemble into a zeroed CSR (structure from
 * orc_structure) and a zeroed b.  kappa (nullable) holds one conductivity per
 * element in element-id order; NULL means the reference's k = 1. */
int orc_assemble(int nx, int ny, int nz, const double* kappa,
                 const int32_t* row_offsets, const int32_t* cols,
                 double* vals, double* b);

/* Boundary sets of simple_mesh_description: mask0 = bc_rows_0 (faces x=0,
 * y=0, z=0, y=1, z=1), mask1 = bc_rows_1 (face x=1).  One byte per row. */
void orc_bc_masks(int nx, int ny, int nz, uint8_t* mask0, uint8_t* mask1);

/* impose_dirichlet(value, A, b, ..., bc_rows) with bc_rows as a row mask. */
void orc_impose_dirichlet(double value, int64_t nrows,
                          const int32_t* row_offsets, const int32_t* cols,
                          double* vals, double* b, const uint8_t* bc_mask);

/* matvec_std (CSR), dot, waxpby, fused_waxpby. */
void orc_matvec(int64_t nrows, const int32_t* row_offsets, const int32_t* cols,
                const double* vals, const double* x, double* y);
double orc_dot(int64_t n, const double* x, const double* y);
void orc_waxpby(int64_t n, double alpha, const double* x, double beta,
                const double* y, double* w);

/* cg_solve.  tol_mode 0: the reference's absolute test normr > tol.
 * tol_mode 1: relative, normr > tol * normr0 (same loop structure).
 * x is the initial guess on entry and the solution on exit.
 * history (nullable, max_iter+1 entries) receives normr before each
 * iteration; history[0] is the initial residual.
 * Returns 0 on normal exit, 1 on numerical breakdown. */
int orc_cg_solve(int64_t nrows, const int32_t* row_offsets, const int32_t* cols,
                 const double* vals, const double* b, double* x,
                 int max_iter, double tol, int tol_mode,
                 int* num_iters, double* normr, double* history);

/* Analytic solution (Carslaw & Jaeger series) and verify_solution. */
double orc_analytic_soln(double x, double y, double z, int max_p, int max_q);
int orc_verify_solution(int nx, int ny, int nz, const double* x, double tolerance,
                        int whole_domain, double* max_err);

/* The full reference pipeline for one box: structure, assembly (k = kappa or
 * 1), both Dirichlet passes.  Arrays sized by orc_num_rows / orc_num_nonzeros. */
int orc_build_system(int nx, int ny, int nz, const double* kappa,
                     int32_t* row_offsets, int32_t* cols, double* vals, double* b);

/* Element-wise gradient contraction used by the adjoint oracle:
 * g[e] = -lambda_e^T Khat_e u_e, Khat_e the k = 1 element matrix. */
void orc_element_gradient(int nx, int ny, int nz, const double* u,
                          const double* lambda, double* g);

#ifdef __cplusplus
}
#endif

#endif
