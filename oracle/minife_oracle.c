/*
 * CPU restatement of miniFE's assemble-and-solve path (oracle).
 *
 * TEST INFRASTRUCTURE ONLY -- see minife_oracle.h.  Compiled with
 * -ffp-contract=off so that no multiply-add is fused on any host (aarch64
 * contracts by default); the reference's x86-64 g++ build performs every
 * multiply and add separately, and so does this file.
 *
 * Reference paths below are relative to the Mantevo miniFE repository.
 */
#include "minife_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* mesh helpers                                                        */
/* ------------------------------------------------------------------ */

/* Node box of a single-rank run: nodes = elements + 1 per dimension when the
 * element box is non-empty (generate_matrix_structure.hpp:69-74). */
static int nodes_of(int n) { return n > 0 ? n + 1 : 0; }

int64_t orc_num_rows(int nx, int ny, int nz)
{
  return (int64_t)nodes_of(nx) * nodes_of(ny) * nodes_of(nz);
}

/* Neighbours of coordinate i in [0, n) including itself. */
static int64_t nbr_count(int i, int n)
{
  int c = 1;
  if (i > 0) ++c;
  if (i + 1 < n) ++c;
  return c;
}

int64_t orc_num_nonzeros(int nx, int ny, int nz)
{
  int Nx = nodes_of(nx), Ny = nodes_of(ny), Nz = nodes_of(nz);
  int64_t sx = 0, sy = 0, sz = 0;
  for (int i = 0; i < Nx; ++i) sx += nbr_count(i, Nx);
  for (int i = 0; i < Ny; ++i) sy += nbr_count(i, Ny);
  for (int i = 0; i < Nz; ++i) sz += nbr_count(i, Nz);
  return sx * sy * sz;
}

/* get_id (ref/utils/box_utils.hpp:99-111): -1 outside the box. */
static int64_t get_id(int nx, int ny, int nz, int x, int y, int z)
{
  if (x < 0 || y < 0 || z < 0) return -1;
  if (x >= nx || y >= ny || z >= nz) return -1;
  return (int64_t)x + (int64_t)nx * y + (int64_t)nx * ny * z;
}

/* get_coords (ref/utils/box_utils.hpp:64-82). */
static void get_coords(int64_t id, int nx, int ny, int nz,
                       double* x, double* y, double* z)
{
  const int xdiv = nx > 1 ? nx - 1 : 1;
  const int ydiv = ny > 1 ? ny - 1 : 1;
  const int zdiv = nz > 1 ? nz - 1 : 1;
  int64_t nxy = (int64_t)nx * ny;
  *z = (1.0 * (double)(id / nxy)) / zdiv;
  *y = 1.0 * (double)((id % nxy) / nx) / ydiv;
  *x = 1.0 * (double)(id % nx) / xdiv;
}

/* ------------------------------------------------------------------ */
/* structure: generate_matrix_structure.hpp:47-149, MatrixInitOp.hpp:127-156 */
/* ------------------------------------------------------------------ */
int orc_structure(int nx, int ny, int nz, int32_t* row_offsets, int32_t* cols)
{
  int Nx = nodes_of(nx), Ny = nodes_of(ny), Nz = nodes_of(nz);
  int64_t global_nrows = (int64_t)Nx * Ny * Nz;
  int64_t nnz = 0, r = 0;
  for (int iz = 0; iz < Nz; ++iz)
    for (int iy = 0; iy < Ny; ++iy)
      for (int ix = 0; ix < Nx; ++ix) {
        row_offsets[r++] = (int32_t)nnz;
        /* columns are produced in ascending id order, so the reference's
         * sort_if_needed (MatrixInitOp.hpp:155) leaves them unchanged */
        for (int sz = -1; sz <= 1; ++sz)
          for (int sy = -1; sy <= 1; ++sy)
            for (int sx = -1; sx <= 1; ++sx) {
              int64_t col = get_id(Nx, Ny, Nz, ix + sx, iy + sy, iz + sz);
              if (col >= 0 && col < global_nrows) cols[nnz++] = (int32_t)col;
            }
      }
  row_offsets[r] = (int32_t)nnz;
  return 0;
}

/* ------------------------------------------------------------------ */
/* Hex8 element math: ref/fem/Hex8.hpp, gauss_pts.hpp, Hex8_ElemData.hpp */
/* ------------------------------------------------------------------ */

/* gauss_pts(2) (ref/fem/gauss_pts.hpp:41,50-53): the truncated constant. */
static const double GP = 0.577350269;

/* Hex8::shape_fns (Hex8.hpp:44-65). */
static void shape_fns(const double* x, double* v)
{
  const double u = 1.0 - x[0], vv = 1.0 - x[1], w = 1.0 - x[2];
  const double up1 = 1.0 + x[0], vp1 = 1.0 + x[1], wp1 = 1.0 + x[2];
  v[0] = 0.125 * u * vv * w;
  v[1] = 0.125 * up1 * vv * w;
  v[2] = 0.125 * up1 * vp1 * w;
  v[3] = 0.125 * u * vp1 * w;
  v[4] = 0.125 * u * vv * wp1;
  v[5] = 0.125 * up1 * vv * wp1;
  v[6] = 0.125 * up1 * vp1 * wp1;
  v[7] = 0.125 * u * vp1 * wp1;
}

/* Hex8::gradients (Hex8.hpp:68-113). */
static void gradients(const double* x, double* g)
{
  const double u = 1.0 - x[0], v = 1.0 - x[1], w = 1.0 - x[2];
  const double up1 = 1.0 + x[0], vp1 = 1.0 + x[1], wp1 = 1.0 + x[2];
  g[0] = -0.125 * v * w;     g[1] = -0.125 * u * w;     g[2] = -0.125 * u * v;
  g[3] = 0.125 * v * w;      g[4] = -0.125 * up1 * w;   g[5] = -0.125 * up1 * v;
  g[6] = 0.125 * vp1 * w;    g[7] = 0.125 * up1 * w;    g[8] = -0.125 * up1 * vp1;
  g[9] = -0.125 * vp1 * w;   g[10] = 0.125 * u * w;     g[11] = -0.125 * u * vp1;
  g[12] = -0.125 * v * wp1;  g[13] = -0.125 * u * wp1;  g[14] = 0.125 * u * v;
  g[15] = 0.125 * v * wp1;   g[16] = -0.125 * up1 * wp1; g[17] = 0.125 * up1 * v;
  g[18] = 0.125 * vp1 * wp1; g[19] = 0.125 * up1 * wp1; g[20] = 0.125 * up1 * vp1;
  g[21] = -0.125 * vp1 * wp1; g[22] = 0.125 * u * wp1;  g[23] = 0.125 * u * vp1;
}

/* compute_gradient_values (Hex8_ElemData.hpp:37-61): ig -> pt[0], jg ->
 * pt[1], kg -> pt[2], kg fastest. */
void orc_gradient_values(double* grad_vals)
{
  const double gpts[2] = {-GP, GP};
  double pt[3];
  double* p = grad_vals;
  for (int ig = 0; ig < 2; ++ig) {
    pt[0] = gpts[ig];
    for (int jg = 0; jg < 2; ++jg) {
      pt[1] = gpts[jg];
      for (int kg = 0; kg < 2; ++kg) {
        pt[2] = gpts[kg];
        gradients(pt, p);
        p += 24;
      }
    }
  }
}

/* Jacobian accumulation shared by gradients_and_detJ (Hex8.hpp:116-175) and
 * gradients_and_invJ_and_detJ (Hex8.hpp:178-242). */
static void jacobian(const double* c, const double* g, double J[9])
{
  double J00 = 0, J01 = 0, J02 = 0, J10 = 0, J11 = 0, J12 = 0, J20 = 0, J21 = 0, J22 = 0;
  for (int i = 0; i < 8; ++i) {
    const double* gi = g + 3 * i;
    const double* ci = c + 3 * i;
    J00 += gi[0] * ci[0]; J01 += gi[0] * ci[1]; J02 += gi[0] * ci[2];
    J10 += gi[1] * ci[0]; J11 += gi[1] * ci[1]; J12 += gi[1] * ci[2];
    J20 += gi[2] * ci[0]; J21 += gi[2] * ci[1]; J22 += gi[2] * ci[2];
  }
  J[0] = J00; J[1] = J01; J[2] = J02; J[3] = J10; J[4] = J11; J[5] = J12;
  J[6] = J20; J[7] = J21; J[8] = J22;
}

/* gradients_and_invJ_and_detJ (Hex8.hpp:178-257). */
static void invJ_and_detJ(const double* coords, const double* g, double* invJ,
                          double* detJ)
{
  double J[9];
  jacobian(coords, g, J);
  const double J00 = J[0], J01 = J[1], J02 = J[2], J10 = J[3], J11 = J[4],
               J12 = J[5], J20 = J[6], J21 = J[7], J22 = J[8];
  double term0 = J22 * J11 - J21 * J12;
  double term1 = J22 * J01 - J21 * J02;
  double term2 = J12 * J01 - J11 * J02;
  *detJ = J00 * term0 - J10 * term1 + J20 * term2;
  double inv_detJ = 1.0 / *detJ;
  invJ[0] = term0 * inv_detJ;
  invJ[1] = -term1 * inv_detJ;
  invJ[2] = term2 * inv_detJ;
  invJ[3] = -(J22 * J10 - J20 * J12) * inv_detJ;
  invJ[4] = (J22 * J00 - J20 * J02) * inv_detJ;
  invJ[5] = -(J12 * J00 - J10 * J02) * inv_detJ;
  invJ[6] = (J21 * J10 - J20 * J11) * inv_detJ;
  invJ[7] = -(J21 * J00 - J20 * J01) * inv_detJ;
  invJ[8] = (J11 * J00 - J10 * J01) * inv_detJ;
}

/* Hex8::diffusionMatrix_symm (Hex8.hpp:260-361); the reference hard-codes
 * k = 1.0 (:273), here k is a parameter so per-element conductivity reuses
 * the same operation order (k*detJ*w at :307). */
void orc_diffusion_matrix_symm(const double* coords, const double* grad_vals,
                               double k, double* elem_mat)
{
  const double gwts[2] = {1.0, 1.0};
  double dpsidx[8], dpsidy[8], dpsidz[8], invJ[9], detJ = 0.0;
  for (int i = 0; i < 36; ++i) elem_mat[i] = 0.0;
  size_t gv_offset = 0;
  for (int ig = 0; ig < 2; ++ig) {
    double wi = gwts[ig];
    for (int jg = 0; jg < 2; ++jg) {
      double wi_wj = wi * gwts[jg];
      for (int kg = 0; kg < 2; ++kg) {
        double wi_wj_wk = wi_wj * gwts[kg];
        const double* gv = &grad_vals[gv_offset];
        gv_offset += 24;
        invJ_and_detJ(coords, gv, invJ, &detJ);
        double k_detJ_w = k * detJ * wi_wj_wk;
        for (int i = 0; i < 8; ++i) {
          double g0 = gv[3 * i], g1 = gv[3 * i + 1], g2 = gv[3 * i + 2];
          dpsidx[i] = g0 * invJ[0] + g1 * invJ[1] + g2 * invJ[2];
          dpsidy[i] = g0 * invJ[3] + g1 * invJ[4] + g2 * invJ[5];
          dpsidz[i] = g0 * invJ[6] + g1 * invJ[7] + g2 * invJ[8];
        }
        int off = 0;
        for (int m = 0; m < 8; ++m) {
          const double xm = dpsidx[m], ym = dpsidy[m], zm = dpsidz[m];
          elem_mat[off++] += k_detJ_w * ((xm * xm) + (ym * ym) + (zm * zm));
          for (int n = m + 1; n < 8; ++n)
            elem_mat[off++] += k_detJ_w * ((xm * dpsidx[n]) + (ym * dpsidy[n]) +
                                           (zm * dpsidz[n]));
        }
      }
    }
  }
}

/* Hex8::sourceVector (Hex8.hpp:364-410), Q = 1. */
void orc_source_vector(const double* coords, const double* grad_vals, double* elem_vec)
{
  const double gpts[2] = {-GP, GP};
  const double gwts[2] = {1.0, 1.0};
  const double Q = 1.0;
  double psi[8], pt[3], J[9];
  for (int i = 0; i < 8; ++i) elem_vec[i] = 0.0;
  size_t gv_offset = 0;
  for (int ig = 0; ig < 2; ++ig) {
    pt[0] = gpts[ig];
    double wi = gwts[ig];
    for (int jg = 0; jg < 2; ++jg) {
      pt[1] = gpts[jg];
      double wj = gwts[jg];
      for (int kg = 0; kg < 2; ++kg) {
        pt[2] = gpts[kg];
        double wk = gwts[kg];
        shape_fns(pt, psi);
        const double* gv = &grad_vals[gv_offset];
        gv_offset += 24;
        jacobian(coords, gv, J);
        double term0 = J[8] * J[4] - J[7] * J[5];
        double term1 = J[8] * J[1] - J[7] * J[2];
        double term2 = J[5] * J[1] - J[4] * J[2];
        double detJ = J[0] * term0 - J[3] * term1 + J[6] * term2;
        double term = Q * detJ * wi * wj * wk;
        for (int i = 0; i < 8; ++i) elem_vec[i] += psi[i] * term;
      }
    }
  }
}

/* get_elem_nodes_and_coords (ref/src/Hex8_box_utils.hpp:101-159) with
 * get_hex8_node_ids (:41-57) and get_hex8_node_coords_3d (:59-99). */
void orc_elem_nodes_and_coords(int nx, int ny, int nz, int ex, int ey, int ez,
                               int32_t* ids, double* c)
{
  int Nx = nx + 1, Ny = ny + 1, Nz = nz + 1;
  int64_t n0 = get_id(Nx, Ny, Nz, ex, ey, ez);
  int64_t NxNy = (int64_t)Nx * Ny;
  ids[0] = (int32_t)n0;
  ids[1] = (int32_t)(n0 + 1);
  ids[2] = (int32_t)(n0 + Nx + 1);
  ids[3] = (int32_t)(n0 + Nx);
  ids[4] = (int32_t)(n0 + NxNy);
  ids[5] = (int32_t)(n0 + 1 + NxNy);
  ids[6] = (int32_t)(n0 + Nx + NxNy + 1);
  ids[7] = (int32_t)(n0 + Nx + NxNy);
  double x, y, z;
  get_coords(n0, Nx, Ny, Nz, &x, &y, &z);
  double hx = 1.0 / nx, hy = 1.0 / ny, hz = 1.0 / nz;
  c[0] = x;       c[1] = y;       c[2] = z;
  c[3] = x + hx;  c[4] = y;       c[5] = z;
  c[6] = x + hx;  c[7] = y + hy;  c[8] = z;
  c[9] = x;       c[10] = y + hy; c[11] = z;
  c[12] = x;      c[13] = y;      c[14] = z + hz;
  c[15] = x + hx; c[16] = y;      c[17] = z + hz;
  c[18] = x + hx; c[19] = y + hy; c[20] = z + hz;
  c[21] = x;      c[22] = y + hy; c[23] = z + hz;
}

/* ------------------------------------------------------------------ */
/* assembly: perform_element_loop.hpp:40-104,                          */
/* SparseMatrix_functions.hpp:142-227 (sum_into_row,                   */
/* sum_in_symm_elem_matrix), Vector_functions.hpp:84-103               */
/* ------------------------------------------------------------------ */

/* sum_into_row (SparseMatrix_functions.hpp:142-160): lower_bound per col. */
static void sum_into_row(int row_len, const int32_t* row_cols, double* row_coefs,
                         int num_inputs, const int32_t* in_cols, const double* in_coefs)
{
  for (int i = 0; i < num_inputs; ++i) {
    int lo = 0, hi = row_len;
    while (lo < hi) {
      int mid = (lo + hi) >> 1;
      if (row_cols[mid] < in_cols[i]) lo = mid + 1; else hi = mid;
    }
    if (lo < row_len && row_cols[lo] == in_cols[i]) row_coefs[lo] += in_coefs[i];
  }
}

/* sum_in_symm_elem_matrix (SparseMatrix_functions.hpp:183-227). */
static void sum_in_symm_elem_matrix(const int32_t* ids, const double* coefs,
                                    const int32_t* ro, const int32_t* cols, double* vals)
{
  int row_offset = 0;
  for (int i = 0; i < 8; ++i) {
    int32_t row = ids[i];
    const double* row_coefs = &coefs[row_offset];
    int row_len = 8 - i;
    row_offset += row_len;
    int mlen = ro[row + 1] - ro[row];
    const int32_t* mcols = cols + ro[row];
    double* mvals = vals + ro[row];
    if (mlen == 0) continue;
    sum_into_row(mlen, mcols, mvals, row_len, &ids[i], row_coefs);
    int offset = i;
    for (int j = 0; j < i; ++j) {
      double coef = coefs[offset];
      sum_into_row(mlen, mcols, mvals, 1, &ids[j], &coef);
      offset += 8 - (j + 1);
    }
  }
}

int orc_assemble(int nx, int ny, int nz, const double* kappa,
                 const int32_t* ro, const int32_t* cols, double* vals, double* b)
{
  double grad_vals[192], coords[24], elem_mat[36], elem_vec[8];
  int32_t ids[8];
  orc_gradient_values(grad_vals);
  int64_t e = 0;
  /* BoxIterator order (BoxIterator.hpp:79-96): x fastest, then y, then z */
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex, ++e) {
        orc_elem_nodes_and_coords(nx, ny, nz, ex, ey, ez, ids, coords);
        orc_diffusion_matrix_symm(coords, grad_vals, kappa ? kappa[e] : 1.0, elem_mat);
        orc_source_vector(coords, grad_vals, elem_vec);
        sum_in_symm_elem_matrix(ids, elem_mat, ro, cols, vals);
        for (int i = 0; i < 8; ++i) b[ids[i]] += elem_vec[i];
      }
  return 0;
}

/* ------------------------------------------------------------------ */
/* Dirichlet: simple_mesh_description.hpp:62-224 (sets),               */
/* SparseMatrix_functions.hpp:410-480 (impose_dirichlet)               */
/* ------------------------------------------------------------------ */
void orc_bc_masks(int nx, int ny, int nz, uint8_t* mask0, uint8_t* mask1)
{
  int Nx = nodes_of(nx), Ny = nodes_of(ny), Nz = nodes_of(nz);
  int64_t r = 0;
  for (int iz = 0; iz < Nz; ++iz)
    for (int iy = 0; iy < Ny; ++iy)
      for (int ix = 0; ix < Nx; ++ix, ++r) {
        mask0[r] = (ix == 0 || iy == 0 || iz == 0 || iy == Ny - 1 || iz == Nz - 1);
        mask1[r] = (ix == Nx - 1);
      }
}

void orc_impose_dirichlet(double value, int64_t nrows, const int32_t* ro,
                          const int32_t* cols, double* vals, double* b,
                          const uint8_t* bc)
{
  /* first loop: ascending bc rows (set order) -> identity rows, b = value */
  for (int64_t row = 0; row < nrows; ++row) {
    if (!bc[row]) continue;
    b[row] = value;
    for (int32_t j = ro[row]; j < ro[row + 1]; ++j)
      vals[j] = (cols[j] == row) ? 1.0 : 0.0;
  }
  /* second loop: every non-bc row lifts its bc columns */
  for (int64_t i = 0; i < nrows; ++i) {
    if (bc[i]) continue;
    double sum = 0;
    for (int32_t j = ro[i]; j < ro[i + 1]; ++j) {
      if (bc[cols[j]]) {
        sum += vals[j];
        vals[j] = 0;
      }
    }
    b[i] -= sum * value;
  }
}

int orc_build_system(int nx, int ny, int nz, const double* kappa,
                     int32_t* ro, int32_t* cols, double* vals, double* b)
{
  int64_t n = orc_num_rows(nx, ny, nz);
  int64_t nnz = orc_num_nonzeros(nx, ny, nz);
  orc_structure(nx, ny, nz, ro, cols);
  memset(vals, 0, sizeof(double) * (size_t)nnz);
  memset(b, 0, sizeof(double) * (size_t)n);
  orc_assemble(nx, ny, nz, kappa, ro, cols, vals, b);
  uint8_t* m0 = (uint8_t*)malloc((size_t)n);
  uint8_t* m1 = (uint8_t*)malloc((size_t)n);
  if (!m0 || !m1) { free(m0); free(m1); return 1; }
  orc_bc_masks(nx, ny, nz, m0, m1);
  /* driver.hpp:214-218: the 0-valued faces first, then the x=1 face */
  orc_impose_dirichlet(0.0, n, ro, cols, vals, b, m0);
  orc_impose_dirichlet(1.0, n, ro, cols, vals, b, m1);
  free(m0);
  free(m1);
  return 0;
}

/* ------------------------------------------------------------------ */
/* kernels: SparseMatrix_functions.hpp:545-578, Vector_functions.hpp    */
/* ------------------------------------------------------------------ */
void orc_matvec(int64_t nrows, const int32_t* ro, const int32_t* cols,
                const double* vals, const double* x, double* y)
{
  for (int64_t row = 0; row < nrows; ++row) {
    /* the reference starts from beta*y[row] with beta = 0 (:565-568);
     * that is +-0 for finite y and does not change the sum's value */
    double sum = 0.0;
    for (int32_t i = ro[row]; i < ro[row + 1]; ++i) sum += vals[i] * x[cols[i]];
    y[row] = sum;
  }
}

double orc_dot(int64_t n, const double* x, const double* y)
{
  double r = 0;
  for (int64_t i = 0; i < n; ++i) r += x[i] * y[i];
  return r;
}

void orc_waxpby(int64_t n, double alpha, const double* x, double beta,
                const double* y, double* w)
{
  for (int64_t i = 0; i < n; ++i) w[i] = alpha * x[i] + beta * y[i];
}

/* breakdown (cg_solve.hpp:49-67) */
static int breakdown(double inner, int64_t n, const double* v, const double* w)
{
  double vnorm = sqrt(orc_dot(n, v, v));
  double wnorm = sqrt(orc_dot(n, w, w));
  return fabs(inner) <= 100 * vnorm * wnorm * 2.220446049250313e-16;
}

/* cg_solve (cg_solve.hpp:69-229), non-fused variant. */
int orc_cg_solve(int64_t n, const int32_t* ro, const int32_t* cols,
                 const double* vals, const double* b, double* x,
                 int max_iter, double tol, int tol_mode,
                 int* num_iters, double* normr_out, double* history)
{
  double* r = (double*)calloc((size_t)n, sizeof(double));
  double* p = (double*)calloc((size_t)n, sizeof(double));
  double* Ap = (double*)calloc((size_t)n, sizeof(double));
  if (!r || !p || !Ap) { free(r); free(p); free(Ap); return 2; }
  double normr = 0, rtrans = 0, oldrtrans = 0;
  const double one = 1.0, zero = 0.0;
  int status = 0;
  *num_iters = 0;

  orc_waxpby(n, one, x, zero, x, p);
  orc_matvec(n, ro, cols, vals, p, Ap);
  orc_waxpby(n, one, b, -one, Ap, r);
  rtrans = orc_dot(n, r, r);
  normr = sqrt(rtrans);
  if (history) history[0] = normr;
  const double abs_tol = tol_mode == 1 ? tol * normr : tol;
  double brkdown_tol = 2.220446049250313e-16;

  for (int k = 1; k <= max_iter && normr > abs_tol; ++k) {
    if (k == 1) {
      orc_waxpby(n, one, r, zero, r, p);
    } else {
      oldrtrans = rtrans;
      rtrans = orc_dot(n, r, r);
      double beta = rtrans / oldrtrans;
      orc_waxpby(n, one, r, beta, p, p);
    }
    normr = sqrt(rtrans);
    if (history) history[k] = normr;
    orc_matvec(n, ro, cols, vals, p, Ap);
    double p_ap_dot = orc_dot(n, Ap, p);
    if (p_ap_dot < brkdown_tol) {
      if (p_ap_dot < 0 || breakdown(p_ap_dot, n, Ap, p)) {
        status = 1;
        break;
      }
      brkdown_tol = 0.1 * p_ap_dot;
    }
    double alpha = rtrans / p_ap_dot;
    orc_waxpby(n, one, x, alpha, p, x);
    orc_waxpby(n, one, r, -alpha, Ap, r);
    *num_iters = k;
  }
  *normr_out = normr;
  free(r);
  free(p);
  free(Ap);
  return status;
}

/* ------------------------------------------------------------------ */
/* verification: ref/fem/analytic_soln.hpp:66-112,                      */
/* ref/fem/verify_solution.hpp:55-174                                  */
/* ------------------------------------------------------------------ */
static const double PI = 3.141592653589793238462;

double orc_analytic_soln(double x, double y, double z, int max_p, int max_q)
{
  const double PI_SQR = PI * PI;
  const double term0 = 16.0 / (PI_SQR);
  double sum = 0;
  for (int p = 0; p <= max_p; ++p) {
    const double p21y = (2 * p + 1) * PI * y;
    const double sin_py = sin(p21y) / (2 * p + 1);
    for (int q = 0; q <= max_q; ++q) {
      const double q21z = (2 * q + 1) * PI * z;
      const double sin_qz = sin(q21z) / (2 * q + 1);
      const double l = sqrt((2 * p + 1) * (2 * p + 1) * PI_SQR + (2 * q + 1) * (2 * q + 1) * PI_SQR);
      const double sinh1 = sinh(l * x);
      const double sinh2 = sinh(l);
      const double tmp = (sinh1 * sin_py) * (sin_qz / sinh2);
      if (tmp == tmp) sum += tmp;
      else break;
    }
  }
  return term0 * sum;
}

int orc_verify_solution(int nx, int ny, int nz, const double* xv, double tolerance,
                        int whole, double* max_err_out)
{
  int Nx = nodes_of(nx), Ny = nodes_of(ny), Nz = nodes_of(nz);
  double max_err = 0.0;
  int64_t r = 0;
  for (int iz = 0; iz < Nz; ++iz)
    for (int iy = 0; iy < Ny; ++iy)
      for (int ix = 0; ix < Nx; ++ix, ++r) {
        double x, y, z;
        get_coords(get_id(Nx, Ny, Nz, ix, iy, iz), Nx, Ny, Nz, &x, &y, &z);
        int check = whole || (fabs(x - 0.5) < 0.05 && fabs(y - 0.5) < 0.05 &&
                              fabs(z - 0.5) < 0.05);
        if (!check) continue;
        double a;
        if (x == 1.0) a = 1;
        else if (x == 0.0 || y == 0.0 || z == 0.0) a = 0;
        else if (y == 1.0 || z == 1.0) a = 0;
        else a = orc_analytic_soln(x, y, z, 300, 300);
        double err = fabs(a - xv[r]);
        if (err > max_err) max_err = err;
      }
  if (max_err_out) *max_err_out = max_err;
  return max_err > tolerance ? 1 : 0;
}

/* ------------------------------------------------------------------ */
/* adjoint contraction (extension: per-element conductivity replaces   */
/* the constant k of Hex8.hpp:273)                                     */
/* ------------------------------------------------------------------ */
void orc_element_gradient(int nx, int ny, int nz, const double* u,
                          const double* lambda, double* g)
{
  double grad_vals[192], coords[24], em[36];
  int32_t ids[8];
  orc_gradient_values(grad_vals);
  int64_t e = 0;
  for (int ez = 0; ez < nz; ++ez)
    for (int ey = 0; ey < ny; ++ey)
      for (int ex = 0; ex < nx; ++ex, ++e) {
        orc_elem_nodes_and_coords(nx, ny, nz, ex, ey, ez, ids, coords);
        orc_diffusion_matrix_symm(coords, grad_vals, 1.0, em);
        double K[8][8];
        int off = 0;
        for (int m = 0; m < 8; ++m)
          for (int n = m; n < 8; ++n) { K[m][n] = em[off]; K[n][m] = em[off]; ++off; }
        double s = 0.0;
        for (int m = 0; m < 8; ++m) {
          double t = 0.0;
          for (int n = 0; n < 8; ++n) t += K[m][n] * u[ids[n]];
          s += lambda[ids[m]] * t;
        }
        g[e] = -s;
      }
}
