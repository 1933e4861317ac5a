// Device-resident CG state shared by the SpMV and vector kernels.  The CG
// loop runs inside a CUDA graph: scalars (rtrans, pAp, alpha, beta, normr,
// the iteration counter and the loop condition) live here and are updated by
// the last block of each reduction, so no host round trip is needed per
// iteration.
#pragma once

#include <cuda_runtime.h>

namespace mfe {

struct CgState {
  double rtrans;       // r.r at the top of the current iteration (cg_solve.hpp:158)
  double oldrtrans;
  double rr_new;       // r.r after the latest x/r update
  double pAp;          // p.Ap of the current iteration (cg_solve.hpp:179)
  double beta;         // beta for the next p update
  double normr;        // the reference's normr (cg_solve.hpp:163)
  double normr0;       // initial residual norm (cg_solve.hpp:138)
  double tol_abs;      // absolute tolerance the loop tests against
  double brkdown_tol;  // cg_solve.hpp:144,199
  int k;               // current iteration, 1-based
  int max_iter;
  int num_iters;       // completed iterations (cg_solve.hpp:215)
  int cont;            // loop condition for the next iteration
  int check_pending;   // pAp < brkdown_tol: the host evaluates breakdown()
  int record;          // write normr of each iteration to history
  unsigned err;        // kernel error flags (mfe_common.cuh)
  int tol_mode;        // 0 absolute, 1 relative to normr0 (tol kept in tol_abs until init)
  int p_reset;         // the next p update is p = r (a restart from the true residual)
  unsigned x0_nonzero; // the zero-guess start (k_cg_init_b) found a nonzero entry in x0
  double* history;     // device, max_iter + 1 entries (when record)
};

// The state after the initial residual r = b - A x0 with r.r = total
// (cg_solve.hpp:124-144): rtrans, normr, normr0, the absolute tolerance
// (relative tolerances are scaled by normr0 here) and the loop condition.
// Called by the last block of the kernel that forms r.r.
__device__ __forceinline__ void cg_resid_init(CgState* cg, double total)
{
  const double normr = sqrt(total);
  cg->rtrans = total;
  cg->rr_new = total;
  cg->normr = normr;
  cg->normr0 = normr;
  const double tol_abs = cg->tol_mode ? cg->tol_abs * normr : cg->tol_abs;
  cg->tol_abs = tol_abs;
  cg->k = 1;
  cg->num_iters = 0;
  cg->cont = (1 <= cg->max_iter) && (normr > tol_abs);
  if (cg->record) cg->history[0] = cg->history[1] = normr;
}

}  // namespace mfe
