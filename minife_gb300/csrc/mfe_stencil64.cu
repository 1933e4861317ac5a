// FP64 verified stencil operator of the FP64 CG.
//
// On GB300 the FP64 pipe (1.9 FMA per clock per SM, 1/64 of the FP32 rate)
// bounds the CSR SpMV of miniFE's matrix: one FP64 FMA per nonzero, 27 per
// row, needs 0.76 ms at 256^3 while its bytes need 0.58 ms.  Every matrix
// miniFE assembles on a box is, row by row, either a Dirichlet row dd * x_r
// or the interior 27-point stencil with the entries of Dirichlet neighbours
// zeroed (simple_mesh_description.hpp puts all six faces into the boundary
// sets, SparseMatrix_functions.hpp:434-480 zeroes their columns), and the
// interior stencil is mirror-symmetric: its entry at (dz, dy, dx) depends on
// (|dz|, |dy|, |dx|) only.  stencil64_prepare (mfe_stencil.cu) checks this
// on the matrix itself on every solve, every entry within 2^-40 of its row's
// largest magnitude (the assembled entries of one class differ by rounding
// only: up to a few hundred ulps, 1e-13 relative), and the CG then applies
// the operator from its eight class weights w[4|dz| + 2|dy| + |dx|] and dd.
//
// A row as separable sums (x~ = x with the Dirichlet nodes zeroed):
//   per plane z and position p: a = x~[p], sx = x~[p-1] + x~[p+1],
//   sy = x~[p-Nx] + x~[p+Nx], sxy = the four diagonal neighbours;
//   P1(z) = w4 a + w5 sx + w6 sy + w7 sxy                (the |dz| = 1 part)
//   Q(z)  = P1(z-1) + w0 a + w1 sx + w2 sy + w3 sxy      (FMA chain from P1(z-1))
//   y(z)  = Q(z) + P1(z+1)
// Marching along z, each plane's class sums and P1 are formed once: with four
// adjacent positions per thread a plane costs 14 additions for the class sums
// (6 sums of lines y - 1 and y + 1, then 4 sx and 4 sxy), 16 operations for
// P1 and 16 FMAs for Q, and a row 1 final addition and 1 FMA for p.Ap: 13.5
// FP64 operations per row instead of the CSR kernel's 28.
//
// k_spmv_st64 works on the CG's natural-layout vectors.  A CTA owns 1024
// consecutive positions of the xy plane (four per thread) and a run of z
// steps; the (plane tile, z) steps are split evenly over the grid.  Each
// thread reads its 3 x 6 window x[p-1 .. p+4] of lines y-1, y, y+1 of each
// plane with 8-byte loads (lines of odd length defeat wider ones), the
// neighbouring lines and planes coming from L1/L2: the kernel is bound by
// the FP64 pipe, not by memory.  Window entries that are not interior nodes
// are zeroed by per-thread masks fixed for the whole z run, Dirichlet planes
// take warp-uniform branches, only warps holding a Dirichlet row replace
// its value by dd * x, and warps holding nothing but Dirichlet rows (the
// lines y = 0 and Ny - 1) or positions past the plane form dd * x alone.
// The last step of a run skips the halo plane's unused Q.  p.Ap is summed in FP64 per thread, then per block and
// over the grid in block order (deterministic for a fixed grid).
#include <algorithm>
#include <cmath>
#include <type_traits>

#include "mfe_cgstate.cuh"
#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

namespace {

constexpr int kT64 = 256;  // threads per CTA

struct St64Params {
  int Nx, Ny, Nz, NxNy, ntile;
  double w[8];  // mirror-class weights, class 4|dz| + 2|dy| + |dx|
  double dd;    // Dirichlet diagonal
  const double* __restrict__ x;
  double* __restrict__ y;
  double* partials;
  unsigned* ticket;
  double* dot_out;
  CgState* cg;
};

// CTAs per SM of the grid (three fit at the 76 registers ptxas picks with no
// minimum in the launch bounds): two give z runs half as
// long again, i.e. fewer halo planes recomputed, and still enough warps to
// keep the FP64 pipe fed -- measured at 256^3: 0.4842 ms per product against
// 0.4893 with three and 0.4853 with one.  (Runs of 16-byte loads of the
// window, masked afterwards, measured 0.517-0.66 ms: the load path is not
// what bounds the kernel.)  The kernel's launch bounds state the same two
// blocks, which lets ptxas use the registers the grid leaves free (110
// instead of 76): 0.4796 against 0.4817 ms per product, 0.2859 against
// 0.2867 s for the 256^3 CG, on one box in two interleaved rounds.
constexpr int kSt64CtasPerSm = 2;

// KP adjacent positions per thread (2 or 4): the window of a line is
// x~[p0 - 1 .. p0 + KP], KP + 2 values; a plane's class sums cost KP + 2
// additions (lines y - 1 and y + 1) plus 2 KP (sx, sxy), i.e. 3 + 2 / KP per
// row.  DOT: accumulate p.Ap (the CG's SpMV) or not (a plain product).
template <int KP, bool DOT>
__global__ void __launch_bounds__(kT64, kSt64CtasPerSm) k_spmv_st64(const __grid_constant__ St64Params P)
{
  constexpr int W = KP + 2;  // window length per line
  __shared__ double red[32];
  const int64_t T = (int64_t)P.ntile * P.Nz;
  const int64_t q0 = T * blockIdx.x / gridDim.x, q1 = T * (blockIdx.x + 1) / gridDim.x;
  double dacc = 0.0;
  for (int64_t q = q0; q < q1;) {
    const int tile = (int)(q / P.Nz), za = (int)(q - (int64_t)tile * P.Nz);
    const int zb = (int)min((int64_t)P.Nz, za + (q1 - q));
    const int p0 = tile * (KP * kT64) + KP * threadIdx.x;
    // mask bit W j + t: window entry (line y + j - 1, position p0 - 1 + t) is
    // an interior node of the plane (then its address lies inside the plane)
    unsigned mask = 0;
#pragma unroll
    for (int t = 0; t < W; ++t) {
      const int pp = p0 - 1 + t;
      if (pp >= 0 && pp < P.NxNy) {
        const int iy = pp / P.Nx, ix = pp - iy * P.Nx;
        const bool inx = ix >= 1 && ix <= P.Nx - 2;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int jy = iy + j - 1;
          if (inx && jy >= 1 && jy <= P.Ny - 2) mask |= 1u << (W * j + t);
        }
      }
    }
    bool valid[KP], bnd[KP];
    bool any_bnd = false;
#pragma unroll
    for (int r = 0; r < KP; ++r) {
      valid[r] = p0 + r < P.NxNy;
      bnd[r] = !((mask >> (W + 1 + r)) & 1u);  // a Dirichlet row (or past the plane)
      any_bnd = any_bnd || (valid[r] && bnd[r]);
    }
    const bool wb = __any_sync(0xffffffffu, any_bnd);
    bool any_row = false;  // an interior row among the thread's positions
#pragma unroll
    for (int r = 0; r < KP; ++r) any_row = any_row || (valid[r] && !bnd[r]);
    if (!__any_sync(0xffffffffu, any_row)) {
      // every row of the warp is a Dirichlet row (lines y = 0 and Ny - 1)
      // or past the plane: dd * x, with no stencil work
      const double* cp = P.x + (int64_t)za * P.NxNy + p0;
      double* yq = P.y + (int64_t)za * P.NxNy + p0;
      for (int z = za; z < zb; ++z) {
#pragma unroll
        for (int r = 0; r < KP; ++r) {
          if (valid[r]) {
            const double c = __ldg(cp + r);
            const double yv = P.dd * c;
            yq[r] = yv;
            if (DOT) dacc = fma(yv, c, dacc);
          }
        }
        cp += P.NxNy;
        yq += P.NxNy;
      }
      q += zb - za;
      continue;
    }
    const double* xp = P.x + p0 - 1;  // window origin of plane 0
    auto ld = [](const double* a) { return __ldg(a); };

    // plane z: centres (unmasked, cen), P1 and, when WITHQ, Q (the FMA chain
    // from P1 of plane z - 1); nothing else is loaded for Dirichlet planes
    auto plane = [&](auto withq, int z, const double* P1in, double* P1, double* Qo, double* cen) {
      constexpr bool WQ = decltype(withq)::value;
      const double* b = xp + (int64_t)z * P.NxNy;
#pragma unroll
      for (int r = 0; r < KP; ++r) cen[r] = valid[r] ? ld(b + 1 + r) : 0.0;
      if (z <= 0 || z >= P.Nz - 1) {  // Dirichlet plane (uniform): x~ = 0
#pragma unroll
        for (int r = 0; r < KP; ++r) {
          P1[r] = 0.0;
          if (WQ) Qo[r] = 0.0;
        }
        return;
      }
      double v[3 * W];
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int t = 0; t < W; ++t) {
          const int s = W * j + t;
          const bool m = (mask >> s) & 1u;
          if (j == 1 && t >= 1 && t <= KP) v[s] = m ? cen[t - 1] : 0.0;
          else v[s] = m ? ld(b + (j - 1) * P.Nx + t) : 0.0;
        }
      double e[W];
#pragma unroll
      for (int t = 0; t < W; ++t) e[t] = v[t] + v[2 * W + t];
#pragma unroll
      for (int r = 0; r < KP; ++r) {
        const double a = v[W + 1 + r];
        const double sx = v[W + r] + v[W + r + 2];
        const double sy = e[1 + r];
        const double sxy = e[r] + e[r + 2];
        double p1 = P.w[4] * a;
        p1 = fma(P.w[5], sx, p1);
        p1 = fma(P.w[6], sy, p1);
        P1[r] = fma(P.w[7], sxy, p1);
        if (WQ) {
          double qv = fma(P.w[0], a, P1in[r]);
          qv = fma(P.w[1], sx, qv);
          qv = fma(P.w[2], sy, qv);
          Qo[r] = fma(P.w[3], sxy, qv);
        }
      }
    };
    using WithQ = std::true_type;
    using NoQ = std::false_type;

    double P1c[KP], Qc[KP], cc[KP];
#pragma unroll
    for (int r = 0; r < KP; ++r) P1c[r] = 0.0;
    if (za >= 1) {  // P1 of plane za - 1 (its Q is not needed)
      double cd[KP];
      plane(NoQ{}, za - 1, P1c, P1c, nullptr, cd);
    }
    {
      double P1n[KP];
      plane(WithQ{}, za, P1c, P1n, Qc, cc);
#pragma unroll
      for (int r = 0; r < KP; ++r) P1c[r] = P1n[r];
    }
    double* yp = P.y + (int64_t)za * P.NxNy + p0;
    // step z: plane z + 1 (its Q only when a later step needs it), then row z
    auto step = [&](auto withq, int z) {
      double P1n[KP], Qn[KP], cn[KP];
#pragma unroll
      for (int r = 0; r < KP; ++r) P1n[r] = Qn[r] = cn[r] = 0.0;
      if (z + 1 < P.Nz) plane(withq, z + 1, P1c, P1n, Qn, cn);
      double yv[KP];
      if (z == 0 || z == P.Nz - 1) {
#pragma unroll
        for (int r = 0; r < KP; ++r) yv[r] = P.dd * cc[r];
      } else {
#pragma unroll
        for (int r = 0; r < KP; ++r) yv[r] = Qc[r] + P1n[r];
        if (wb) {
#pragma unroll
          for (int r = 0; r < KP; ++r)
            if (bnd[r]) yv[r] = P.dd * cc[r];
        }
      }
#pragma unroll
      for (int r = 0; r < KP; ++r) {
        if (valid[r]) yp[r] = yv[r];
        if (DOT) dacc = fma(yv[r], cc[r], dacc);
      }
      yp += P.NxNy;
#pragma unroll
      for (int r = 0; r < KP; ++r) {
        P1c[r] = P1n[r];
        Qc[r] = Qn[r];
        cc[r] = cn[r];
      }
    };
    for (int z = za; z < zb - 1; ++z) step(WithQ{}, z);
    step(NoQ{}, zb - 1);  // the run's last row: the halo plane's Q goes unused
    q += zb - za;
  }
  if (!DOT) return;
  const double bt = block_sum(dacc, red);
  double total;
  if (grid_reduce_last(bt, P.partials, P.ticket, red, &total) && threadIdx.x == 0) {
    if (P.cg != nullptr) {
      P.cg->pAp = total;
      if (total < P.cg->brkdown_tol) P.cg->check_pending = 1;
    } else {
      *P.dot_out = total;
    }
  }
}

// four positions per thread: measured at 256^3, 0.484 ms per product
// against 0.493 ms with two (and no difference between the read-only and the
// L1-cached load paths)
constexpr int kKP = 4;

template <bool DOT>
mfe_status st64_launch(mfe_ctx* ctx, St64Params& P)
{
  P.ntile = (int)ceil_div(P.NxNy, (int64_t)kKP * kT64);
  const int64_t T = (int64_t)P.ntile * P.Nz;
  const int64_t res = std::min<int64_t>(
      resident_blocks(ctx, (const void*)k_spmv_st64<kKP, DOT>, kT64, 0),
      (int64_t)kSt64CtasPerSm * ctx->sm_count);
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>(T, res));
  k_spmv_st64<kKP, DOT><<<g, kT64, 0, ctx->stream>>>(P);
  return check_launch(ctx, "k_spmv_st64");
}

}  // namespace

mfe_status launch_spmv_st64(mfe_ctx* ctx, const mfe_csr* A, const double* w8, double dd,
                            const double* x, double* y, const DotSink* sink, void* cg_state)
{
  St64Params P;
  P.Nx = A->box_nx + 1;
  P.Ny = A->box_ny + 1;
  P.Nz = A->box_nz + 1;
  P.NxNy = P.Nx * P.Ny;
  for (int c = 0; c < 8; ++c) P.w[c] = w8[c];
  P.dd = dd;
  P.x = x;
  P.y = y;
  P.cg = static_cast<CgState*>(cg_state);
  P.partials = sink ? sink->partials : nullptr;
  P.ticket = sink ? sink->ticket : nullptr;
  P.dot_out = sink && !cg_state ? sink->out : nullptr;
  const bool dot = P.cg || P.dot_out;
  if (dot && (!P.partials || !P.ticket))
    return fail(ctx, MFE_BAD_ARG, "stencil SpMV: a dot needs reduction buffers");
  return dot ? st64_launch<true>(ctx, P) : st64_launch<false>(ctx, P);
}

}  // namespace mfe
