// Exercises include/minife_gb300.hpp the way the reference's driver
// (ref/src/driver.hpp:150-305) does: the mesh from the global box, then
// generate_matrix_structure, assemble_FE_data and the two impose_dirichlet
// calls on the reference's CSRMatrix / Vector types in host memory, then
// matvec, dot, waxpby, fused_waxpby and cg_solve with the reference's
// signatures; then the same sequence on the ELLMatrix type (the reference
// built with MINIFE_ELL_MATRIX), compared with the CSR run.  Prints "key
// value" lines for tests/test_gpu_host.py.
#include <cstdio>
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <set>
#include <string>
#include <vector>

#include "minife_gb300.hpp"

int main(int argc, char** argv)
{
  using namespace minife_gb300;
  const int nx = argc > 1 ? atoi(argv[1]) : 10, ny = argc > 2 ? atoi(argv[2]) : nx,
            nz = argc > 3 ? atoi(argv[3]) : ny;
  typedef CSRMatrix<double, int, int> Mat;
  typedef Vector<double, int, int> Vec;
  Box global_box = {{0, nx, 0, ny, 0, nz}};
  simple_mesh_description<int> mesh(global_box, global_box);
  Mat A;
  generate_matrix_structure(mesh, A);
  const int64_t n = (int64_t)A.rows.size();
  Vec b(0, (int)n), x(0, (int)n);
  struct {
  } params;
  assemble_FE_data(mesh, A, b, params);
  impose_dirichlet(0.0, A, b, nx, ny, nz, mesh.bc_rows_0);
  impose_dirichlet(1.0, A, b, nx, ny, nz, mesh.bc_rows_1);
  // a fourth argument "dump": the reference's MINIFE_DEBUG files of the system
  const bool dump = argc > 4 && std::string(argv[4]) == "dump";
  if (dump) {
    write_matrix("A.mtx", A);
    write_vector("b.vec", b);
  }
  std::printf("bc_rows_0 %zu\nbc_rows_1 %zu\n", mesh.bc_rows_0.size(), mesh.bc_rows_1.size());
  A.has_local_indices = true;
  A.num_cols = (int)n;
  double vsum = 0, bsum = 0;
  for (double v : A.packed_coefs) vsum += v;
  for (double v : b.coefs) bsum += v;
  std::printf("vals_sum %.17g\nb_sum %.17g\n", vsum, bsum);
  // one matvec, dot, waxpby
  Vec y(0, (int)n), w(0, (int)n);
  for (int64_t i = 0; i < n; ++i) x.coefs[i] = 1.0 / (1.0 + i);
  matvec(A, x, y);
  std::printf("matvec_dot %.17g\n", dot(x, y));
  waxpby(2.0, x, -0.5, y, w);
  std::printf("waxpby_sum %.17g\n", dot(w, w));
  Vec w1(0, (int)n), w2(0, (int)n);
  fused_waxpby(2.0, x, -0.5, y, w1, 1.5, y, 0.25, x, w2);
  double fd = 0;
  for (int64_t i = 0; i < n; ++i) fd = std::max(fd, std::fabs(w1.coefs[i] - w.coefs[i]));
  std::printf("fused_waxpby_diff %.17g\nfused_waxpby_sum2 %.17g\n", fd, dot(w2, w2));
  // the reference's solve: max 200 iterations, tol DBL_EPSILON
  for (int64_t i = 0; i < n; ++i) x.coefs[i] = 0.0;
  int num_iters = 0;
  double normr = 0, tol = 2.220446049250313e-16;
  timer_type times[NUM_TIMERS];
  cg_solve(A, b, x, matvec_std<Mat, Vec>(), 200, tol, num_iters, normr, times);
  double xs = 0;
  for (double v : x.coefs) xs += v;
  std::printf("num_iters %d\nnormr %.17g\nx_sum %.17g\ntotal_time %.6g\n", num_iters, normr, xs,
              times[TOTAL]);

  // the ELL build: structure, element loop, both Dirichlet passes, then the
  // rows (padding left out) against the CSR's, a matvec and the solve
  typedef ELLMatrix<double, int, int> Ell;
  Ell E;
  generate_matrix_structure(mesh, E);
  Vec be(0, (int)n), xe(0, (int)n);
  assemble_FE_data(mesh, E, be, params);
  impose_dirichlet(0.0, E, be, nx, ny, nz, mesh.bc_rows_0);
  impose_dirichlet(1.0, E, be, nx, ny, nz, mesh.bc_rows_1);
  if (dump) write_matrix("A_ell.mtx", E);
  int same = E.num_cols_per_row == 27 && E.num_nonzeros() == (size_t)n * 27;
  for (int64_t r = 0; r < n && same; ++r) {
    size_t len = 0, clen = 0;
    int *ec = nullptr, *cc = nullptr;
    double *ev = nullptr, *cv = nullptr;
    E.get_row_pointers((int)r, len, ec, ev);
    A.get_row_pointers((int)r, clen, cc, cv);
    same = len == clen;
    for (size_t k = 0; k < len && same; ++k) same = ec[k] == cc[k] && ev[k] == cv[k];
    for (size_t k = len; k < 27 && same; ++k) same = ec[k] == 0 && ev[k] == 0.0;
  }
  for (int64_t i = 0; i < n && same; ++i) same = be.coefs[i] == b.coefs[i];
  std::printf("ell_same_as_csr %d\n", same);
  for (int64_t i = 0; i < n; ++i) xe.coefs[i] = 1.0 / (1.0 + i);
  Vec ye(0, (int)n);
  matvec(E, xe, ye);
  matvec(A, xe, y);
  double md = 0;
  for (int64_t i = 0; i < n; ++i) md = std::max(md, std::fabs(ye.coefs[i] - y.coefs[i]));
  std::printf("ell_matvec_diff %.17g\n", md);
  for (int64_t i = 0; i < n; ++i) xe.coefs[i] = 0.0;
  int ell_iters = 0;
  double ell_normr = 0, tol2 = 2.220446049250313e-16;
  cg_solve(E, be, xe, matvec_std<Ell, Vec>(), 200, tol2, ell_iters, ell_normr, times);
  double xd = 0, xm = 0;
  for (int64_t i = 0; i < n; ++i) {
    xd = std::max(xd, std::fabs(xe.coefs[i] - x.coefs[i]));
    xm = std::max(xm, std::fabs(x.coefs[i]));
  }
  std::printf("ell_num_iters %d\nell_normr %.17g\nell_x_rel_diff %.17g\n", ell_iters, ell_normr,
              xd / xm);
  return 0;
}
