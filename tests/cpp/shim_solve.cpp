// Exercises include/minife_gb300.hpp the way reference host code would: the
// reference's CSRMatrix / Vector types filled on the host, then the shim's
// impose_dirichlet, matvec, dot, waxpby and cg_solve with the reference's
// signatures.  Prints "key value" lines for tests/test_gpu_host.py.
//
// The matrix is assembled on the device (mfe_assemble without boundary
// conditions) and copied into the host containers, standing in for the
// reference's own host assembly.
#include <cstdio>
#include <set>
#include <vector>

#include "minife_gb300.hpp"

int main(int argc, char** argv)
{
  using namespace minife_gb300;
  const int nx = argc > 1 ? atoi(argv[1]) : 10, ny = argc > 2 ? atoi(argv[2]) : nx,
            nz = argc > 3 ? atoi(argv[3]) : ny;
  typedef CSRMatrix<double, int, int> Mat;
  typedef Vector<double, int, int> Vec;
  mfe_ctx* ctx = Context::get().h();
  int64_t n, nnz;
  mfe_box_dims(nx, ny, nz, &n, &nnz);
  mfe_csr dA;
  Context::get().check(mfe_csr_alloc(ctx, n, nnz, MFE_F64, &dA), "alloc");
  double* db = nullptr;
  Context::get().check(mfe_device_alloc(ctx, 8 * n, (void**)&db), "alloc b");
  Context::get().check(mfe_assemble(ctx, nx, ny, nz, nullptr, &dA, db, 0), "assemble");
  Mat A;
  A.reserve_space((unsigned)n, 27);
  for (int64_t i = 0; i < n; ++i) A.rows[i] = (int)i;
  A.packed_cols.resize(nnz);
  A.packed_coefs.resize(nnz);
  Vec b(0, (int)n), x(0, (int)n);
  mfe_memcpy_d2h(ctx, A.row_offsets.data(), dA.row_offsets, 4 * (n + 1));
  mfe_memcpy_d2h(ctx, A.packed_cols.data(), dA.cols, 4 * nnz);
  mfe_memcpy_d2h(ctx, A.packed_coefs.data(), dA.vals, 8 * nnz);
  mfe_memcpy_d2h(ctx, b.coefs.data(), db, 8 * n);
  // boundary sets of simple_mesh_description (one rank)
  std::set<int> bc0, bc1;
  const int Nx = nx + 1, Ny = ny + 1, Nz = nz + 1;
  for (int iz = 0; iz < Nz; ++iz)
    for (int iy = 0; iy < Ny; ++iy)
      for (int ix = 0; ix < Nx; ++ix) {
        const int r = ix + Nx * (iy + Ny * iz);
        if (ix == 0 || iy == 0 || iz == 0 || iy == Ny - 1 || iz == Nz - 1) bc0.insert(r);
        if (ix == Nx - 1) bc1.insert(r);
      }
  impose_dirichlet(0.0, A, b, Nx, Ny, Nz, bc0);
  impose_dirichlet(1.0, A, b, Nx, Ny, Nz, bc1);
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
  mfe_device_free(ctx, db);
  mfe_csr_free(ctx, &dA);
  return 0;
}
