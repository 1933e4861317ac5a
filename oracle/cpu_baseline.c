/*
 * OpenMP-threaded CPU baseline of miniFE's CG solve (test/bench
 * infrastructure only, never part of the product).
 *
 * Restates the threading of the reference's openmp/ variant:
 *   matvec_std: `#pragma omp parallel for` over rows
 *               (openmp/src/SparseMatrix_functions.hpp:556)
 *   dot / dot_r2: `parallel for reduction(+:result)`
 *               (openmp/src/Vector_functions.hpp:248,288)
 *   daxpby: parallel for (openmp/src/Vector_functions.hpp:157-219)
 *   cg_solve loop: openmp/src/cg_solve.hpp:124-210
 * bench.py times this on the host cores as the reference arm / cpu_baseline
 * when the reference's own build is not available on the machine.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <omp.h>

int cpub_num_threads(void) { return omp_get_max_threads(); }

static void matvec(int64_t n, const int32_t* ro, const int32_t* cols,
                   const double* vals, const double* x, double* y)
{
#pragma omp parallel for schedule(static)
  for (int64_t row = 0; row < n; ++row) {
    double sum = 0.0;
    for (int32_t i = ro[row]; i < ro[row + 1]; ++i) sum += vals[i] * x[cols[i]];
    y[row] = sum;
  }
}

static double dot(int64_t n, const double* x, const double* y)
{
  double result = 0.0;
#pragma omp parallel for reduction(+ : result) schedule(static)
  for (int64_t i = 0; i < n; ++i) result += x[i] * y[i];
  return result;
}

/* y = alpha*x + beta*y */
static void daxpby(int64_t n, double alpha, const double* x, double beta, double* y)
{
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) y[i] = alpha * x[i] + beta * y[i];
}

/* Unpreconditioned CG from x (in/out); tol_mode 1 = relative to ||r0||.
 * Stops after max_iter iterations.  Returns the iteration count. */
int cpub_cg_solve(int64_t n, const int32_t* ro, const int32_t* cols,
                  const double* vals, const double* b, double* x,
                  int max_iter, double tol, int tol_mode, double* normr_out)
{
  double* r = (double*)malloc(sizeof(double) * (size_t)n);
  double* p = (double*)malloc(sizeof(double) * (size_t)n);
  double* Ap = (double*)malloc(sizeof(double) * (size_t)n);
  if (!r || !p || !Ap) { free(r); free(p); free(Ap); return -1; }
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) { p[i] = x[i]; r[i] = 0.0; Ap[i] = 0.0; }
  matvec(n, ro, cols, vals, p, Ap);
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; ++i) r[i] = b[i] - Ap[i];
  double rtrans = dot(n, r, r), oldrtrans;
  double normr = sqrt(rtrans);
  const double abs_tol = tol_mode == 1 ? tol * normr : tol;
  int it = 0;
  for (int k = 1; k <= max_iter && normr > abs_tol; ++k) {
    if (k == 1) {
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < n; ++i) p[i] = r[i];
    } else {
      oldrtrans = rtrans;
      rtrans = dot(n, r, r);
      daxpby(n, 1.0, r, rtrans / oldrtrans, p);
    }
    normr = sqrt(rtrans);
    matvec(n, ro, cols, vals, p, Ap);
    double pAp = dot(n, Ap, p);
    double alpha = rtrans / pAp;
    daxpby(n, alpha, p, 1.0, x);
    daxpby(n, -alpha, Ap, 1.0, r);
    it = k;
  }
  if (normr_out) *normr_out = normr;
  free(r);
  free(p);
  free(Ap);
  return it;
}
