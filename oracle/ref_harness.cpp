// Harness around the UNMODIFIED reference (Mantevo miniFE, ref/ variant).
//
// TEST INFRASTRUCTURE ONLY.  `make -C oracle ref` compiles this file together
// with the reference's own headers and utility sources, where they lie in the
// read-only reference checkout, into oracle/_ref/ref_harness.  It calls the
// reference's own functions in driver.hpp's order and writes every array at
// full precision (raw little-endian binary), which the 6-significant-digit
// MINIFE_DEBUG dumps (SparseMatrix_functions.hpp:98-140) cannot give.
//
// usage: ref_harness nx ny nz max_iter tol_mode tol outdir
//   tol_mode 0: the reference's absolute tolerance (driver.hpp:241-245 uses
//               max_iter 200, tol = DBL_EPSILON)
//   tol_mode 1: tol relative to the initial residual ||b|| (x0 = 0)
// special: ref_harness element outdir  -> element matrix/vector of the unit
//          cube at the origin (the known-answer case of the legacy unit test)

#include <cstdio>
#include <iostream>
#include <sstream>
#include <fstream>
#include <set>
#include <map>
#include <cstdlib>
#include <cstring>
#include <cmath>
#include <limits>
#include <string>
#include <vector>

#include <Box.hpp>
#include <BoxPartition.hpp>
#include <box_utils.hpp>
#include <Parameters.hpp>
#include <utils.hpp>
#include <CSRMatrix.hpp>
#include <Vector.hpp>
#include <simple_mesh_description.hpp>
#include <SparseMatrix_functions.hpp>
#include <generate_matrix_structure.hpp>
#include <assemble_FE_data.hpp>
#include <make_local_matrix.hpp>
#include <cg_solve.hpp>
#include <verify_solution.hpp>
#include <Hex8_ElemData.hpp>

template <typename T>
static void dump(const std::string& path, const T* p, size_t n)
{
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::perror(path.c_str()); std::exit(2); }
  if (n) std::fwrite(p, sizeof(T), n, f);
  std::fclose(f);
}

typedef miniFE::CSRMatrix<double, int, int> Mat;
typedef miniFE::Vector<double, int, int> Vec;

static int element_case(const std::string& out)
{
  miniFE::ElemData<int, double> ed;
  miniFE::compute_gradient_values(ed.grad_vals);
  // unit cube at the origin, h = 1 (the legacy unit test's element)
  miniFE::get_hex8_node_coords_3d(0.0, 0.0, 0.0, 1.0, 1.0, 1.0, ed.elem_node_coords);
  miniFE::compute_element_matrix_and_vector(ed);
  dump(out + "/elem_mat.f64", ed.elem_diffusion_matrix, 36);
  dump(out + "/elem_vec.f64", ed.elem_source_vector, 8);
  dump(out + "/grad_vals.f64", ed.grad_vals, 192);
  return 0;
}

int main(int argc, char** argv)
{
  if (argc == 3 && std::string(argv[1]) == "element") return element_case(argv[2]);
  if (argc != 8 && argc != 9) {
    std::fprintf(stderr, "usage: %s nx ny nz max_iter tol_mode tol outdir [dump]\n", argv[0]);
    return 1;
  }
  // dump: also write the reference's own MINIFE_DEBUG files (write_matrix /
  // write_vector, driver.hpp:206-234,308-310) into the working directory
  const bool dump_files = argc == 9 && std::string(argv[8]) == "dump";
  int nx = std::atoi(argv[1]), ny = std::atoi(argv[2]), nz = std::atoi(argv[3]);
  int max_iter = std::atoi(argv[4]);
  int tol_mode = std::atoi(argv[5]);
  double tol = std::atof(argv[6]);
  std::string out = argv[7];

  miniFE::Parameters params;
  params.nx = nx; params.ny = ny; params.nz = nz;
  Box global_box = {0, nx, 0, ny, 0, nz};
  Box my_box;
  box_partition(0, 1, 2, global_box, &my_box);

  miniFE::simple_mesh_description<int> mesh(global_box, my_box);
  Mat A;
  if (miniFE::generate_matrix_structure(mesh, A) != 0) return 3;
  int nrows = (int)A.rows.size();
  Vec b(A.rows[0], nrows), x(A.rows[0], nrows);
  miniFE::assemble_FE_data(mesh, A, b, params);
  dump(out + "/row_offsets.i32", &A.row_offsets[0], A.row_offsets.size());
  dump(out + "/cols.i32", &A.packed_cols[0], A.packed_cols.size());
  dump(out + "/vals_prebc.f64", &A.packed_coefs[0], A.packed_coefs.size());
  dump(out + "/b_prebc.f64", &b.coefs[0], b.coefs.size());
  if (dump_files) {
    miniFE::write_matrix("A_prebc.mtx", A);
    miniFE::write_vector("b_prebc.vec", b);
  }

  miniFE::impose_dirichlet(0.0, A, b, nx + 1, ny + 1, nz + 1, mesh.bc_rows_0);
  miniFE::impose_dirichlet(1.0, A, b, nx + 1, ny + 1, nz + 1, mesh.bc_rows_1);
  dump(out + "/vals.f64", &A.packed_coefs[0], A.packed_coefs.size());
  dump(out + "/b.f64", &b.coefs[0], b.coefs.size());
  if (dump_files) {
    miniFE::write_matrix("A.mtx", A);
    miniFE::write_vector("b.vec", b);
  }

  miniFE::make_local_matrix(A);

  double abs_tol = tol;
  if (tol_mode == 1) abs_tol = tol * std::sqrt(miniFE::dot(b, b));
  int num_iters = 0;
  double normr = 0;
  miniFE::timer_type times[miniFE::NUM_TIMERS];
  miniFE::cg_solve(A, b, x, miniFE::matvec_std<Mat, Vec>(), max_iter, abs_tol,
                   num_iters, normr, times);
  dump(out + "/x.f64", &x.coefs[0], x.coefs.size());
  if (dump_files) miniFE::write_vector("x.vec", x);
  int verify = miniFE::verify_solution(mesh, x, 0.06, false);

  FILE* f = std::fopen((out + "/meta.txt").c_str(), "w");
  std::fprintf(f, "nrows %d\nnnz %d\nnum_iters %d\nnormr %.17g\nverify %d\nabs_tol %.17g\n",
               nrows, (int)A.packed_cols.size(), num_iters, normr, verify, abs_tol);
  std::fclose(f);
  return 0;
}
