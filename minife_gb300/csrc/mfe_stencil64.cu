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
// Marching along z, each plane's class sums and P1 are formed once: with two
// adjacent positions per thread a plane costs 8 additions (class sums), 8
// operations for P1, 8 FMAs for Q, and a row 1 final addition and 1 FMA for
// p.Ap: 14 FP64 operations per row instead of 28.
//
// k_spmv_st64 works on the CG's natural-layout vectors.  A CTA owns 512
// consecutive positions of the xy plane (two per thread) and a run of z
// steps; the (plane tile, z) steps are split evenly over the grid.  Each
// thread reads its 3 x 4 window x[p-1 .. p+2] of lines y-1, y, y+1 of each
// plane with 8-byte loads (lines of odd length defeat wider ones), the
// neighbouring lines and planes coming from L1/L2: the kernel is bound by
// the FP64 pipe, not by memory.  Window entries that are not interior nodes
// are zeroed by per-thread masks fixed for the whole z run, Dirichlet planes
// take warp-uniform branches, and only warps holding a Dirichlet row replace
// its value by dd * x.  p.Ap is summed in FP64 per thread, then per block and
// over the grid in block order (deterministic for a fixed grid).
#include <algorithm>
#include <cmath>

#include "mfe_cgstate.cuh"
#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

namespace {

constexpr int kT64 = 256;       // threads per CTA
constexpr int kT64P = 2 * kT64;  // plane positions per CTA

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

// class sums and P1 of one interior plane for positions p, p + 1 from the
// window v[4j + t] = x~[p - 1 + t] of line y + j - 1
struct St64Sums {
  double a[2], sx[2], sy[2], sxy[2];
};

__device__ __forceinline__ void st64_sums(const double* v, St64Sums& S)
{
  double e[4];
#pragma unroll
  for (int t = 0; t < 4; ++t) e[t] = v[t] + v[8 + t];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    S.a[r] = v[5 + r];
    S.sx[r] = v[4 + r] + v[6 + r];
    S.sy[r] = e[1 + r];
    S.sxy[r] = e[r] + e[2 + r];
  }
}

__global__ void __launch_bounds__(kT64) k_spmv_st64(const __grid_constant__ St64Params P)
{
  __shared__ double red[32];
  const int64_t T = (int64_t)P.ntile * P.Nz;
  const int64_t q0 = T * blockIdx.x / gridDim.x, q1 = T * (blockIdx.x + 1) / gridDim.x;
  double dacc = 0.0;
  for (int64_t q = q0; q < q1;) {
    const int tile = (int)(q / P.Nz), za = (int)(q - (int64_t)tile * P.Nz);
    const int zb = (int)min((int64_t)P.Nz, za + (q1 - q));
    const int p0 = tile * kT64P + 2 * threadIdx.x;
    const bool v0 = p0 < P.NxNy, v1 = p0 + 1 < P.NxNy;
    // mask bit 4j + t: window entry (line y + j - 1, position p0 - 1 + t) is
    // an interior node of the plane (then its address lies inside the plane)
    unsigned mask = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t) {
      const int pp = p0 - 1 + t;
      if (pp >= 0 && pp < P.NxNy) {
        const int iy = pp / P.Nx, ix = pp - iy * P.Nx;
        const bool inx = ix >= 1 && ix <= P.Nx - 2;
#pragma unroll
        for (int j = 0; j < 3; ++j) {
          const int jy = iy + j - 1;
          if (inx && jy >= 1 && jy <= P.Ny - 2) mask |= 1u << (4 * j + t);
        }
      }
    }
    const bool bnd0 = !((mask >> 5) & 1u), bnd1 = !((mask >> 6) & 1u);  // Dirichlet rows
    const bool wb = __any_sync(0xffffffffu, (v0 && bnd0) || (v1 && bnd1));
    const double* xp = P.x + p0 - 1;  // window origin of plane 0

    // plane z: centres (unmasked), P1 and Q (chain from P1 of plane z - 1)
    auto plane = [&](int z, const double* P1in, double* P1, double* Qo, double* cen) {
      const double* b = xp + (int64_t)z * P.NxNy;
      cen[0] = v0 ? __ldg(b + 1) : 0.0;
      cen[1] = v1 ? __ldg(b + 2) : 0.0;
      if (z <= 0 || z >= P.Nz - 1) {  // Dirichlet plane (uniform): x~ = 0
        P1[0] = P1[1] = 0.0;
        Qo[0] = Qo[1] = 0.0;
        return;
      }
      double v[12];
#pragma unroll
      for (int j = 0; j < 3; ++j)
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          const int s = 4 * j + t;
          if (s == 5) v[s] = (mask >> 5) & 1u ? cen[0] : 0.0;
          else if (s == 6) v[s] = (mask >> 6) & 1u ? cen[1] : 0.0;
          else v[s] = (mask >> s) & 1u ? __ldg(b + (j - 1) * P.Nx + t) : 0.0;
        }
      St64Sums S;
      st64_sums(v, S);
#pragma unroll
      for (int r = 0; r < 2; ++r) {
        double p1 = P.w[4] * S.a[r];
        p1 = fma(P.w[5], S.sx[r], p1);
        p1 = fma(P.w[6], S.sy[r], p1);
        P1[r] = fma(P.w[7], S.sxy[r], p1);
        double qv = fma(P.w[0], S.a[r], P1in[r]);
        qv = fma(P.w[1], S.sx[r], qv);
        qv = fma(P.w[2], S.sy[r], qv);
        Qo[r] = fma(P.w[3], S.sxy[r], qv);
      }
    };

    double P1c[2] = {0.0, 0.0}, Qc[2], cc[2];
    if (za >= 1) {  // P1 of plane za - 1 (its Q is not needed)
      double zq[2] = {0.0, 0.0}, qd[2], cd[2];
      plane(za - 1, zq, P1c, qd, cd);
    }
    {
      double P1n[2];
      plane(za, P1c, P1n, Qc, cc);
      P1c[0] = P1n[0];
      P1c[1] = P1n[1];
    }
    double* yp = P.y + (int64_t)za * P.NxNy + p0;
    for (int z = za; z < zb; ++z) {
      double P1n[2] = {0.0, 0.0}, Qn[2] = {0.0, 0.0}, cn[2] = {0.0, 0.0};
      if (z + 1 < P.Nz) plane(z + 1, P1c, P1n, Qn, cn);
      double y0, y1;
      if (z == 0 || z == P.Nz - 1) {
        y0 = P.dd * cc[0];
        y1 = P.dd * cc[1];
      } else {
        y0 = Qc[0] + P1n[0];
        y1 = Qc[1] + P1n[1];
        if (wb) {
          if (bnd0) y0 = P.dd * cc[0];
          if (bnd1) y1 = P.dd * cc[1];
        }
      }
      if (v1) {
        yp[0] = y0;
        yp[1] = y1;
      } else if (v0) {
        yp[0] = y0;
      }
      dacc = fma(y0, cc[0], dacc);
      dacc = fma(y1, cc[1], dacc);
      yp += P.NxNy;
      P1c[0] = P1n[0];
      P1c[1] = P1n[1];
      Qc[0] = Qn[0];
      Qc[1] = Qn[1];
      cc[0] = cn[0];
      cc[1] = cn[1];
    }
    q += zb - za;
  }
  if (P.dot_out == nullptr && P.cg == nullptr) return;
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

}  // namespace

mfe_status launch_spmv_st64(mfe_ctx* ctx, const mfe_csr* A, const double* w8, double dd,
                            const double* x, double* y, const DotSink* sink, void* cg_state)
{
  St64Params P;
  P.Nx = A->box_nx + 1;
  P.Ny = A->box_ny + 1;
  P.Nz = A->box_nz + 1;
  P.NxNy = P.Nx * P.Ny;
  P.ntile = (int)ceil_div(P.NxNy, (int64_t)kT64P);
  for (int c = 0; c < 8; ++c) P.w[c] = w8[c];
  P.dd = dd;
  P.x = x;
  P.y = y;
  P.cg = static_cast<CgState*>(cg_state);
  P.partials = sink ? sink->partials : nullptr;
  P.ticket = sink ? sink->ticket : nullptr;
  P.dot_out = sink && !cg_state ? sink->out : nullptr;
  if ((P.cg || P.dot_out) && (!P.partials || !P.ticket))
    return fail(ctx, MFE_BAD_ARG, "stencil SpMV: a dot needs reduction buffers");
  const int64_t T = (int64_t)P.ntile * P.Nz;
  const int g = (int)std::max<int64_t>(
      1, std::min<int64_t>(T, (int64_t)resident_blocks(ctx, (const void*)k_spmv_st64, kT64, 0)));
  k_spmv_st64<<<g, kT64, 0, ctx->stream>>>(P);
  return check_launch(ctx, "k_spmv_st64");
}

}  // namespace mfe
