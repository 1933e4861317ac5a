// Structure generation, FE assembly, Dirichlet conditions, verification and
// the adjoint element contraction.
//
// This translation unit is compiled with -fmad=false: the Hex8 element math
// must round every multiply and add separately, as the reference does, so the
// assembled matrix and right-hand side are bit-identical to the reference's.
//
// Assembly is split in two passes (the reference's perform_element_loop does
// both in one serial loop with binary-search scatter, perform_element_loop.hpp
// :80-100, SparseMatrix_functions.hpp:183-255):
//   1. element pass: one thread per element computes its 36-entry symmetric
//      diffusion matrix and 8-entry source vector into a structure-of-arrays
//      scratch (coalesced writes); the Jacobian's three columns come from
//      per-axis tables (an element's x column depends on its x pair only),
//      computed once per box with the reference's operations in its order;
//   2. node gather: one thread per node row reads the rows of its (up to) 8
//      adjacent element matrices, in ascending element order, into 27 stencil
//      accumulators, applies both Dirichlet passes in registers, and writes
//      the CSR row (staged through shared memory for coalescing).
// The passes alternate over slabs of kSlab element planes: the scratch is a
// ring of kSlab + 1 element planes (element plane z in slot z mod (kSlab +
// 1)), so a slab's gather still finds the previous slab's last plane, and
// the scratch is (kSlab + 1) nx ny elements instead of nx ny nz.
// No atomics: every coefficient is summed in the reference's element order.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "mfe_box.cuh"
#include "mfe_common.cuh"
#include "mfe_hex8.cuh"
#include "mfe_internal.h"

namespace mfe {

__constant__ Hex8Tables c_hex8;

// ---------------------------------------------------------------------------
// closed-form 27-point structure (offsets: mfe_box.cuh)
// ---------------------------------------------------------------------------
int64_t box_nnz(int nx, int ny, int nz)
{
  return (3 * (int64_t)(nx + 1) - 2) * (3 * (int64_t)(ny + 1) - 2) * (3 * (int64_t)(nz + 1) - 2);
}

constexpr int kStructRows = 128;

// One thread per row: row offset (closed form) and the ascending in-box
// 27-point columns (MatrixInitOp.hpp:127-156), staged in shared memory so the
// block writes its contiguous column range coalesced.  vals are zeroed.
__global__ void __launch_bounds__(kStructRows)
    k_structure(int Nx, int Ny, int Nz, int64_t N, int32_t* __restrict__ ro,
                int32_t* __restrict__ cols)
{
  __shared__ int32_t s_cols[kStructRows * 27];
  const int64_t r0 = (int64_t)blockIdx.x * kStructRows;
  const int64_t r = r0 + threadIdx.x;
  const int64_t NxNy = (int64_t)Nx * Ny;
  const int64_t rend = min(r0 + (int64_t)kStructRows, N);
  const int64_t base =
      row_offset((int)(r0 % Nx), (int)((r0 / Nx) % Ny), (int)(r0 / NxNy), Nx, Ny, Nz);
  const int64_t endoff =
      rend == N ? (3 * (int64_t)Nx - 2) * (3 * (int64_t)Ny - 2) * (3 * (int64_t)Nz - 2)
                : row_offset((int)(rend % Nx), (int)((rend / Nx) % Ny), (int)(rend / NxNy), Nx,
                             Ny, Nz);
  if (r < N) {
    const int ix = (int)(r % Nx), iy = (int)((r / Nx) % Ny), iz = (int)(r / NxNy);
    const int64_t off = row_offset(ix, iy, iz, Nx, Ny, Nz);
    ro[r] = (int32_t)off;
    int k = (int)(off - base);
#pragma unroll
    for (int sz = -1; sz <= 1; ++sz)
#pragma unroll
      for (int sy = -1; sy <= 1; ++sy)
#pragma unroll
        for (int sx = -1; sx <= 1; ++sx) {
          const int jx = ix + sx, jy = iy + sy, jz = iz + sz;
          if (jx >= 0 && jx < Nx && jy >= 0 && jy < Ny && jz >= 0 && jz < Nz)
            s_cols[k++] = (int32_t)(r + sx + sy * (int64_t)Nx + sz * NxNy);
        }
    if (r == N - 1) ro[N] = (int32_t)endoff;
  }
  __syncthreads();
  const int total = (int)(endoff - base);
  for (int i = threadIdx.x; i < total; i += kStructRows) cols[base + i] = s_cols[i];
}

// ---------------------------------------------------------------------------
// element pass
// ---------------------------------------------------------------------------
constexpr int kElemThreads = 128;
constexpr int kSlab = 16;  // element planes per slab; the ring holds kSlab + 1

// Per-axis Jacobian columns: jc[(base_axis + i) * 24 + gp * 3 + a] for
// element index i along the axis (base: 0 for x, nx for y, nx + ny for z),
// with the coordinate pair of elem_corner().
__global__ void k_jcols(int nx, int ny, int nz, double* __restrict__ jc)
{
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = (nx + ny + nz) * 8;
  if (t >= n) return;
  const int gp = t % 8, row = t / 8;
  int axis, i;
  double c0, c1;
  if (row < nx) {
    axis = 0;
    i = row;
    c0 = (1.0 * (double)i) / (double)nx;
    c1 = c0 + 1.0 / nx;
  } else if (row < nx + ny) {
    axis = 1;
    i = row - nx;
    c0 = 1.0 * (double)i / (double)ny;
    c1 = c0 + 1.0 / ny;
  } else {
    axis = 2;
    i = row - nx - ny;
    c0 = (1.0 * (double)i) / (double)nz;
    c1 = c0 + 1.0 / nz;
  }
  double col[3];
  jacobian_column(c_hex8, axis, c0, c1, gp, col);
  double* o = jc + (int64_t)row * 24 + gp * 3;
  o[0] = col[0];
  o[1] = col[1];
  o[2] = col[2];
}

// Elements of planes ez0 .. ez0 + nplanes - 1 in BoxIterator order (x
// fastest).  Element (ex, ey, ez) goes to ring index ri = ((ez mod R) ny + ey)
// nx + ex: ke[k * RS + ri] (k < 36, upper triangle), fe[k * RS + ri] (k < 8),
// RS = R nx ny.  kappa (nullable) is indexed by the global element id.
__global__ void __launch_bounds__(kElemThreads)
    k_element(int nx, int ny, int nz, int ez0, int nplanes, int R, const double* __restrict__ kappa,
              const double* __restrict__ jc, double* __restrict__ ke, double* __restrict__ fe)
{
  const int64_t nxny = (int64_t)nx * ny;
  const int64_t el = (int64_t)blockIdx.x * kElemThreads + threadIdx.x;
  if (el >= nxny * nplanes) return;
  const int ex = (int)(el % nx);
  const int ey = (int)((el / nx) % ny);
  const int ez = ez0 + (int)(el / nxny);
  const int64_t e = ex + (int64_t)nx * (ey + (int64_t)ny * ez);
  const int64_t RS = (int64_t)R * nxny;
  const int64_t ri = ((int64_t)(ez % R) * ny + ey) * nx + ex;
  const double k = kappa ? kappa[e] : 1.0;
  const double* cx = jc + (int64_t)ex * 24;
  const double* cy = jc + ((int64_t)nx + ey) * 24;
  const double* cz = jc + ((int64_t)nx + ny + ez) * 24;
  double em[36], ev[8];
  element_matrix_vector_j(
      c_hex8,
      [&](int gp, double J[9]) {
        J[0] = __ldg(cx + gp * 3);
        J[3] = __ldg(cx + gp * 3 + 1);
        J[6] = __ldg(cx + gp * 3 + 2);
        J[1] = __ldg(cy + gp * 3);
        J[4] = __ldg(cy + gp * 3 + 1);
        J[7] = __ldg(cy + gp * 3 + 2);
        J[2] = __ldg(cz + gp * 3);
        J[5] = __ldg(cz + gp * 3 + 1);
        J[8] = __ldg(cz + gp * 3 + 2);
      },
      k, em, ev);
#pragma unroll
  for (int i = 0; i < 36; ++i) ke[i * RS + ri] = em[i];
#pragma unroll
  for (int i = 0; i < 8; ++i) fe[i * RS + ri] = ev[i];
}

// ---------------------------------------------------------------------------
// node gather + both Dirichlet passes
// ---------------------------------------------------------------------------
constexpr int kGatherRows = 128;

// Rows of node planes iz0 .. iz1 - 1; their adjacent elements are in the
// ring (ke, fe as k_element writes them).
__global__ void __launch_bounds__(kGatherRows)
    k_gather(int nx, int ny, int nz, int iz0, int iz1, int R, const double* __restrict__ ke,
             const double* __restrict__ fe, const int32_t* __restrict__ ro,
             double* __restrict__ vals, double* __restrict__ b, int impose_bc)
{
  __shared__ double s_vals[kGatherRows * 27];
  const int Nx = nx + 1, Ny = ny + 1, Nz = nz + 1;
  const int64_t NxNy = (int64_t)Nx * Ny;
  const int64_t RS = (int64_t)R * nx * ny;
  const int64_t R1 = NxNy * iz1;
  const int64_t r0 = NxNy * iz0 + (int64_t)blockIdx.x * kGatherRows;
  const int64_t r = r0 + threadIdx.x;
  const int64_t rend = min(r0 + (int64_t)kGatherRows, R1);
  const int64_t base = ro[r0];
  if (r < R1) {
    const int ix = (int)(r % Nx), iy = (int)((r / Nx) % Ny), iz = (int)(r / NxNy);
    const bool bc1 = (ix == Nx - 1);
    const bool bc0 = (ix == 0 || iy == 0 || iz == 0 || iy == Ny - 1 || iz == Nz - 1);
    const int64_t off = ro[r] - base;
    if (impose_bc && (bc0 || bc1)) {
      // zero_row_and_put_1_on_diagonal (SparseMatrix_functions.hpp:413-428),
      // b = prescribed value; the x=1 face (second pass) wins on shared edges
      int k = 0;
#pragma unroll
      for (int s = 0; s < 27; ++s) {
        const int jx = ix + s % 3 - 1, jy = iy + (s / 3) % 3 - 1, jz = iz + s / 9 - 1;
        if (jx >= 0 && jx < Nx && jy >= 0 && jy < Ny && jz >= 0 && jz < Nz)
          s_vals[off + k++] = (s == 13) ? 1.0 : 0.0;
      }
      b[r] = bc1 ? 1.0 : 0.0;
    } else {
      double acc[27];
#pragma unroll
      for (int s = 0; s < 27; ++s) acc[s] = 0.0;
      double bsum = 0.0;
      // adjacent elements in ascending element id: (ez, ey, ex) lexicographic
#pragma unroll
      for (int c = 0; c < 2; ++c) {
        const int ez = iz - 1 + c;
#pragma unroll
        for (int bb = 0; bb < 2; ++bb) {
          const int ey = iy - 1 + bb;
#pragma unroll
          for (int a = 0; a < 2; ++a) {
            const int ex = ix - 1 + a;
            if (ex < 0 || ex >= nx || ey < 0 || ey >= ny || ez < 0 || ez >= nz) continue;
            const int64_t e = ((int64_t)(ez % R) * ny + ey) * nx + ex;
            const int lr = local_node(1 - a, 1 - bb, 1 - c);
#pragma unroll
            for (int m = 0; m < 8; ++m) {
              const int mx = (m == 1 || m == 2 || m == 5 || m == 6);
              const int my = (m == 2 || m == 3 || m == 6 || m == 7);
              const int mz = (m >= 4);
              const int slot = (c + mz) * 9 + (bb + my) * 3 + (a + mx);
              acc[slot] += __ldg(&ke[(int64_t)sym_index(lr, m) * RS + e]);
            }
            bsum += __ldg(&fe[(int64_t)lr * RS + e]);
          }
        }
      }
      if (!impose_bc) {
        int k = 0;
#pragma unroll
        for (int s = 0; s < 27; ++s) {
          const int jx = ix + s % 3 - 1, jy = iy + (s / 3) % 3 - 1, jz = iz + s / 9 - 1;
          if (jx >= 0 && jx < Nx && jy >= 0 && jy < Ny && jz >= 0 && jz < Nz)
            s_vals[off + k++] = acc[s];
        }
        b[r] = bsum;
      } else {
        // interior row: all 27 columns exist.  impose_dirichlet pass 1
        // (value 0, faces x=0,y=0,z=0,y=1,z=1) then pass 2 (value 1, face
        // x=1), SparseMatrix_functions.hpp:460-479, in ascending column order
        double s0 = 0.0, s1 = 0.0;
#pragma unroll
        for (int s = 0; s < 27; ++s) {
          const int jx = ix + s % 3 - 1, jy = iy + (s / 3) % 3 - 1, jz = iz + s / 9 - 1;
          const bool c0 = (jx == 0 || jy == 0 || jz == 0 || jy == Ny - 1 || jz == Nz - 1);
          const bool c1 = (jx == Nx - 1);
          if (c0) s0 += acc[s];
          if (c1) s1 += c0 ? 0.0 : acc[s];  // pass 1 already zeroed c0 columns
          s_vals[off + s] = (c0 || c1) ? 0.0 : acc[s];
        }
        double bv = bsum;
        bv -= s0 * 0.0;
        bv -= s1 * 1.0;
        b[r] = bv;
      }
    }
  }
  __syncthreads();
  const int total = (int)(ro[rend] - base);
  for (int i = threadIdx.x; i < total; i += kGatherRows) vals[base + i] = s_vals[i];
}

// ---------------------------------------------------------------------------
// generic impose_dirichlet for any CSR (SparseMatrix_functions.hpp:434-480)
// ---------------------------------------------------------------------------
__global__ void k_bc_mark(int64_t n_bc, const int32_t* __restrict__ bc_rows, int64_t nrows,
                          uint8_t* __restrict__ mask, const int32_t* __restrict__ ro,
                          const int32_t* __restrict__ cols, double* __restrict__ vals,
                          double* __restrict__ b, double value)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_bc) return;
  const int32_t row = bc_rows[i];
  if (row < 0 || row >= nrows) return;  // rows outside the matrix are ignored
  mask[row] = 1;
  b[row] = value;
  for (int32_t j = ro[row]; j < ro[row + 1]; ++j) vals[j] = (cols[j] == row) ? 1.0 : 0.0;
}

__global__ void k_bc_lift(int64_t nrows, const uint8_t* __restrict__ mask,
                          const int32_t* __restrict__ ro, const int32_t* __restrict__ cols,
                          double* __restrict__ vals, double* __restrict__ b, double value)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows || mask[i]) return;
  double sum = 0.0;
  for (int32_t j = ro[i]; j < ro[i + 1]; ++j) {
    const int32_t c = cols[j];
    if (c >= 0 && c < nrows && mask[c]) {
      sum += vals[j];
      vals[j] = 0.0;
    }
  }
  b[i] -= sum * value;
}

__global__ void k_to_f32(const double* __restrict__ src, float* __restrict__ dst, int64_t n)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

// ---------------------------------------------------------------------------
// verify_solution (ref/fem/verify_solution.hpp:55-174) with the series of
// ref/fem/analytic_soln.hpp:66-112:
//   soln(x, y, z) = 16/pi^2 sum_p sum_q sinh(l x) sin_py / sinh(l) sin_qz,
//   l = pi sqrt((2p+1)^2 + (2q+1)^2), p, q = 0..300,
// where the q loop of a p stops at the first term that is NaN.  A term is
// NaN exactly when sinh(l x) overflows (then sinh(l) has overflowed too and
// sin_qz / sinh(l) is a signed zero), so where the q loop stops depends on
// (x, p) only, and the checked nodes form a product set X x Y x Z of
// coordinates.  The sum is therefore evaluated through tables instead of
// 90,601 sinh calls per node:
//   T[x][p,q] = sinh(l x), D[z][p,q] = sin_qz / sinh(l), S[y][p] = sin_py,
//   U[x][z][p] = sum over the q the reference sums of T * D,
//   soln = 16/pi^2 sum_p S[y][p] U[x][z][p];
// each quantity is the reference's expression, only the order of the
// products and additions differs (the result agrees to ~1e-15).
// ---------------------------------------------------------------------------
constexpr int kSerP = 301;             // p, q = 0..300 (verify_solution.hpp:111)
constexpr int kSerPQ = kSerP * kSerP;
constexpr double kPI = 3.141592653589793238462;

// node coordinate along a dimension of N nodes (get_coords, box_utils.hpp:64-82)
__host__ __device__ __forceinline__ double verify_coord(int i, int N)
{
  const int div = N > 1 ? N - 1 : 1;
  return (1.0 * (double)i) / div;
}

struct VerifyAxes {
  int x0, nxs, y0, nys, z0, nzs;  // checked index ranges [a0, a0 + n)
  int Nx, Ny, Nz;
};

// l and sinh(l) per (p, q) (analytic_soln.hpp fcn_l)
__global__ void k_ver_l(double* __restrict__ L, double* __restrict__ S2)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kSerPQ) return;
  const int p = i / kSerP, q = i - p * kSerP;
  const double PI_SQR = kPI * kPI;
  const double l = sqrt((2 * p + 1) * (2 * p + 1) * PI_SQR + (2 * q + 1) * (2 * q + 1) * PI_SQR);
  L[i] = l;
  S2[i] = sinh(l);
}

// T[xi][pq] = sinh(l x), D[zi][pq] = sin_qz(z) / sinh(l)
__global__ void k_ver_td(VerifyAxes A, const double* __restrict__ L, const double* __restrict__ S2,
                         double* __restrict__ T, double* __restrict__ D)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t nt = (int64_t)A.nxs * kSerPQ, nd = (int64_t)A.nzs * kSerPQ;
  if (i < nt) {
    const int xi = (int)(i / kSerPQ), pq = (int)(i - (int64_t)xi * kSerPQ);
    const double x = verify_coord(A.x0 + xi, A.Nx);
    T[i] = sinh(L[pq] * x);
  } else if (i < nt + nd) {
    const int64_t k = i - nt;
    const int zi = (int)(k / kSerPQ), pq = (int)(k - (int64_t)zi * kSerPQ);
    const int q = pq % kSerP;
    const double z = verify_coord(A.z0 + zi, A.Nz);
    const double q21z = (2 * q + 1) * kPI * z;
    const double sin_qz = sin(q21z) / (2 * q + 1);
    D[k] = sin_qz / S2[pq];
  }
}

// U[xi][zi][p] = sum over q < (first q with sinh(l x) = inf) of T * D, in
// q order; one warp per (xi, zi, p), lanes over q, fixed-order warp sum
__global__ void k_ver_u(VerifyAxes A, const double* __restrict__ T, const double* __restrict__ D,
                        double* __restrict__ U)
{
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int64_t nw = (int64_t)A.nxs * A.nzs * kSerP;
  if (w >= nw) return;
  const int p = (int)(w % kSerP);
  const int64_t xz = w / kSerP;
  const int zi = (int)(xz % A.nzs), xi = (int)(xz / A.nzs);
  const double* t = T + (int64_t)xi * kSerPQ + p * kSerP;
  const double* d = D + (int64_t)zi * kSerPQ + p * kSerP;
  // the first overflowing q (sinh(l x) grows with q)
  int qb = kSerP;
  for (int q0 = 0; q0 < kSerP; q0 += 32) {
    const int q = q0 + lane;
    const bool inf = q < kSerP && isinf(t[q]);
    const unsigned m = __ballot_sync(0xffffffffu, inf);
    if (m) {
      qb = q0 + __ffs(m) - 1;
      break;
    }
  }
  double s = 0.0;
  for (int q = lane; q < qb; q += 32) s += t[q] * d[q];
  s = warp_sum(s);
  if (lane == 0) U[w] = s;
}

// one thread per checked node: soln from S (formed here) and U, the
// reference's boundary values, |soln - x| folded into a bitwise maximum
__global__ void k_ver_node(VerifyAxes A, const double* __restrict__ U, const double* __restrict__ xv,
                           unsigned long long* __restrict__ max_bits)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t n = (int64_t)A.nxs * A.nys * A.nzs;
  if (i >= n) return;
  const int xi = (int)(i % A.nxs);
  const int yi = (int)((i / A.nxs) % A.nys);
  const int zi = (int)(i / ((int64_t)A.nxs * A.nys));
  const int ix = A.x0 + xi, iy = A.y0 + yi, iz = A.z0 + zi;
  const double x = verify_coord(ix, A.Nx), y = verify_coord(iy, A.Ny), z = verify_coord(iz, A.Nz);
  double a;
  if (x == 1.0) a = 1;
  else if (x == 0.0 || y == 0.0 || z == 0.0) a = 0;
  else if (y == 1.0 || z == 1.0) a = 0;
  else {
    const double* u = U + ((int64_t)xi * A.nzs + zi) * kSerP;
    double sum = 0.0;
    for (int p = 0; p < kSerP; ++p) {
      const double p21y = (2 * p + 1) * kPI * y;
      const double sin_py = sin(p21y) / (2 * p + 1);
      sum += sin_py * u[p];
    }
    a = 16.0 / (kPI * kPI) * sum;
  }
  const int64_t r = ((int64_t)iz * A.Ny + iy) * A.Nx + ix;
  const double err = fabs(a - xv[r]);
  // non-negative doubles order like their bit patterns
  atomicMax(max_bits, (unsigned long long)__double_as_longlong(err));
}

// ---------------------------------------------------------------------------
// adjoint contraction: g[e] = -lambda_e^T Khat_e u_e (k = 1 element matrix)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kElemThreads)
    k_elem_grad(int nx, int ny, int nz, int64_t E, const double* __restrict__ u,
                const double* __restrict__ lam, double* __restrict__ g)
{
  const int64_t e = (int64_t)blockIdx.x * kElemThreads + threadIdx.x;
  if (e >= E) return;
  const int ex = (int)(e % nx);
  const int ey = (int)((e / nx) % ny);
  const int ez = (int)(e / ((int64_t)nx * ny));
  const int Nx = nx + 1;
  const int64_t NxNy = (int64_t)Nx * (ny + 1);
  const int64_t n0 = ex + (int64_t)Nx * ey + NxNy * ez;
  const int64_t ids[8] = {n0, n0 + 1, n0 + Nx + 1, n0 + Nx,
                          n0 + NxNy, n0 + 1 + NxNy, n0 + Nx + NxNy + 1, n0 + Nx + NxNy};
  const ElemCorner c = elem_corner(ex, ey, ez, nx, ny, nz);
  double em[36], ev[8];
  element_matrix_vector(c_hex8, c, 1.0, em, ev);
  double ue[8], le[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    ue[i] = u[ids[i]];
    le[i] = lam[ids[i]];
  }
  double s = 0.0;
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    double t = 0.0;
#pragma unroll
    for (int n = 0; n < 8; ++n) t += em[sym_index(m, n)] * ue[n];
    s += le[m] * t;
  }
  g[e] = -s;
}

// v[r] = 0 on every Dirichlet row of the box (both boundary sets): the adjoint
// right-hand side must vanish there so that lambda_D = 0.
__global__ void k_zero_boundary(int Nx, int Ny, int Nz, double* __restrict__ v)
{
  const int64_t NxNy = (int64_t)Nx * Ny, N = NxNy * Nz;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < N;
       r += (int64_t)gridDim.x * blockDim.x) {
    const int ix = (int)(r % Nx), iy = (int)((r / Nx) % Ny), iz = (int)(r / NxNy);
    if (ix == 0 || ix == Nx - 1 || iy == 0 || iy == Ny - 1 || iz == 0 || iz == Nz - 1) v[r] = 0.0;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static bool g_tables_ready[64] = {};

// Hex8::gradients / shape_fns at the 2x2x2 Gauss points (Hex8.hpp:44-113,
// Hex8_ElemData.hpp:37-61).  Products and differences of constants only.
static void fill_tables(Hex8Tables& T)
{
  const double gpts[2] = {-kGaussPt, kGaussPt};
  for (int ig = 0; ig < 2; ++ig)
    for (int jg = 0; jg < 2; ++jg)
      for (int kg = 0; kg < 2; ++kg) {
        const int gp = ig * 4 + jg * 2 + kg;
        const double x0 = gpts[ig], x1 = gpts[jg], x2 = gpts[kg];
        const double u = 1.0 - x0, v = 1.0 - x1, w = 1.0 - x2;
        const double up1 = 1.0 + x0, vp1 = 1.0 + x1, wp1 = 1.0 + x2;
        double* g = &T.grad[gp][0][0];
        g[0] = -0.125 * v * w;     g[1] = -0.125 * u * w;     g[2] = -0.125 * u * v;
        g[3] = 0.125 * v * w;      g[4] = -0.125 * up1 * w;   g[5] = -0.125 * up1 * v;
        g[6] = 0.125 * vp1 * w;    g[7] = 0.125 * up1 * w;    g[8] = -0.125 * up1 * vp1;
        g[9] = -0.125 * vp1 * w;   g[10] = 0.125 * u * w;     g[11] = -0.125 * u * vp1;
        g[12] = -0.125 * v * wp1;  g[13] = -0.125 * u * wp1;  g[14] = 0.125 * u * v;
        g[15] = 0.125 * v * wp1;   g[16] = -0.125 * up1 * wp1; g[17] = 0.125 * up1 * v;
        g[18] = 0.125 * vp1 * wp1; g[19] = 0.125 * up1 * wp1; g[20] = 0.125 * up1 * vp1;
        g[21] = -0.125 * vp1 * wp1; g[22] = 0.125 * u * wp1;  g[23] = 0.125 * u * vp1;
        double* p = T.psi[gp];
        p[0] = 0.125 * u * v * w;
        p[1] = 0.125 * up1 * v * w;
        p[2] = 0.125 * up1 * vp1 * w;
        p[3] = 0.125 * u * vp1 * w;
        p[4] = 0.125 * u * v * wp1;
        p[5] = 0.125 * up1 * v * wp1;
        p[6] = 0.125 * up1 * vp1 * wp1;
        p[7] = 0.125 * u * vp1 * wp1;
      }
}

static mfe_status ensure_tables(mfe_ctx* ctx)
{
  if (ctx->device >= 0 && ctx->device < 64 && g_tables_ready[ctx->device]) return MFE_OK;
  Hex8Tables T;
  fill_tables(T);
  MFE_CUDA_TRY(ctx, cudaMemcpyToSymbol(c_hex8, &T, sizeof(T)));
  if (ctx->device >= 0 && ctx->device < 64) g_tables_ready[ctx->device] = true;
  return MFE_OK;
}

mfe_status launch_structure(mfe_ctx* ctx, int nx, int ny, int nz, int32_t* ro, int32_t* cols)
{
  const int Nx = nx + 1, Ny = ny + 1, Nz = nz + 1;
  const int64_t N = (int64_t)Nx * Ny * Nz;
  const int64_t blocks = ceil_div(N, kStructRows);
  k_structure<<<(unsigned)blocks, kStructRows, 0, ctx->stream>>>(Nx, Ny, Nz, N, ro, cols);
  return check_launch(ctx, "k_structure");
}

mfe_status launch_assemble(mfe_ctx* ctx, int nx, int ny, int nz, const double* kappa,
                           const int32_t* ro, double* vals, double* b, int impose_bc)
{
  MFE_TRY(ensure_tables(ctx));
  const int64_t nxny = (int64_t)nx * ny;
  const int64_t NxNy = (int64_t)(nx + 1) * (ny + 1);
  const int R = std::min(kSlab, nz) + 1;
  double* jc = static_cast<double*>(workspace(ctx, "assembly.jcols",
                                              sizeof(double) * 24 * (size_t)(nx + ny + nz)));
  double* ke = static_cast<double*>(workspace(ctx, "assembly.ring", sizeof(double) * 44 * R * nxny));
  if (!jc || !ke) return fail(ctx, MFE_OOM, "assembly scratch allocation failed");
  double* fe = ke + 36 * R * nxny;
  k_jcols<<<(unsigned)ceil_div((int64_t)(nx + ny + nz) * 8, 128), 128, 0, ctx->stream>>>(nx, ny, nz, jc);
  MFE_TRY(check_launch(ctx, "k_jcols"));
  for (int ez0 = 0; ez0 < nz; ez0 += kSlab) {
    const int np = std::min(kSlab, nz - ez0);
    k_element<<<(unsigned)ceil_div(nxny * np, kElemThreads), kElemThreads, 0, ctx->stream>>>(
        nx, ny, nz, ez0, np, R, kappa, jc, ke, fe);
    MFE_TRY(check_launch(ctx, "k_element"));
    // node planes whose elements are all in the ring: ez0 .. ez0 + np - 1,
    // and the last node plane with the last slab
    const int iz0 = ez0, iz1 = ez0 + np == nz ? nz + 1 : ez0 + np;
    k_gather<<<(unsigned)ceil_div(NxNy * (iz1 - iz0), kGatherRows), kGatherRows, 0, ctx->stream>>>(
        nx, ny, nz, iz0, iz1, R, ke, fe, ro, vals, b, impose_bc);
    MFE_TRY(check_launch(ctx, "k_gather"));
  }
  return MFE_OK;
}

mfe_status launch_impose_dirichlet(mfe_ctx* ctx, const mfe_csr* A, double* b, double value,
                                   const int32_t* bc_rows, int64_t n_bc)
{
  uint8_t* mask = static_cast<uint8_t*>(workspace(ctx, "bc.mask", (size_t)A->nrows + 1));
  if (!mask) return fail(ctx, MFE_OOM, "bc mask allocation failed");
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(mask, 0, (size_t)A->nrows, ctx->stream));
  double* vals = static_cast<double*>(A->vals);
  if (n_bc > 0) {
    k_bc_mark<<<(unsigned)ceil_div(n_bc, 256), 256, 0, ctx->stream>>>(
        n_bc, bc_rows, A->nrows, mask, A->row_offsets, A->cols, vals, b, value);
    MFE_TRY(check_launch(ctx, "k_bc_mark"));
  }
  k_bc_lift<<<(unsigned)ceil_div(A->nrows, 256), 256, 0, ctx->stream>>>(
      A->nrows, mask, A->row_offsets, A->cols, vals, b, value);
  return check_launch(ctx, "k_bc_lift");
}

mfe_status launch_convert_f32(mfe_ctx* ctx, const double* src, float* dst, int64_t n)
{
  const int64_t blocks = std::min<int64_t>(ceil_div(n, 256), (int64_t)ctx->sm_count * 16);
  k_to_f32<<<(unsigned)std::max<int64_t>(blocks, 1), 256, 0, ctx->stream>>>(src, dst, n);
  return check_launch(ctx, "k_to_f32");
}

// checked index range along a dimension of N nodes: all, or the nodes with
// |coord - 0.5| < 0.05 (verify_solution.hpp:97-105), a contiguous range
static void verify_range(int N, int whole, int* a0, int* n)
{
  if (whole) {
    *a0 = 0;
    *n = N;
    return;
  }
  int lo = -1, hi = -1;
  for (int i = 0; i < N; ++i)
    if (std::fabs(verify_coord(i, N) - 0.5) < 0.05) {
      if (lo < 0) lo = i;
      hi = i;
    }
  *a0 = lo < 0 ? 0 : lo;
  *n = lo < 0 ? 0 : hi - lo + 1;
}

mfe_status launch_verify(mfe_ctx* ctx, int nx, int ny, int nz, const double* x, int whole,
                         double* max_err_host)
{
  VerifyAxes A;
  A.Nx = nx + 1;
  A.Ny = ny + 1;
  A.Nz = nz + 1;
  verify_range(A.Nx, whole, &A.x0, &A.nxs);
  verify_range(A.Ny, whole, &A.y0, &A.nys);
  verify_range(A.Nz, whole, &A.z0, &A.nzs);
  unsigned long long* d = static_cast<unsigned long long*>(workspace(ctx, "verify.max", 8));
  if (!d) return fail(ctx, MFE_OOM, "verify scratch allocation failed");
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(d, 0, 8, ctx->stream));
  const int64_t nodes = (int64_t)A.nxs * A.nys * A.nzs;
  if (nodes > 0) {
    const int64_t nt = (int64_t)A.nxs * kSerPQ, nd = (int64_t)A.nzs * kSerPQ;
    const int64_t nu = (int64_t)A.nxs * A.nzs * kSerP;
    double* L = static_cast<double*>(workspace(ctx, "verify.l", sizeof(double) * 2 * kSerPQ));
    double* T = static_cast<double*>(workspace(ctx, "verify.td", sizeof(double) * (nt + nd)));
    double* U = static_cast<double*>(workspace(ctx, "verify.u", sizeof(double) * nu));
    if (!L || !T || !U) return fail(ctx, MFE_OOM, "verify table allocation failed");
    double* S2 = L + kSerPQ;
    double* D = T + nt;
    k_ver_l<<<(unsigned)ceil_div(kSerPQ, 256), 256, 0, ctx->stream>>>(L, S2);
    MFE_TRY(check_launch(ctx, "k_ver_l"));
    k_ver_td<<<(unsigned)ceil_div(nt + nd, 256), 256, 0, ctx->stream>>>(A, L, S2, T, D);
    MFE_TRY(check_launch(ctx, "k_ver_td"));
    k_ver_u<<<(unsigned)ceil_div(nu * 32, 256), 256, 0, ctx->stream>>>(A, T, D, U);
    MFE_TRY(check_launch(ctx, "k_ver_u"));
    k_ver_node<<<(unsigned)ceil_div(nodes, 128), 128, 0, ctx->stream>>>(A, U, x, d);
    MFE_TRY(check_launch(ctx, "k_ver_node"));
  }
  unsigned long long* h = static_cast<unsigned long long*>(host_scratch(ctx, 8));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(h, d, 8, cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  unsigned long long bits = *h;
  double v;
  static_assert(sizeof(v) == sizeof(bits), "");
  memcpy(&v, &bits, sizeof(v));
  *max_err_host = v;
  return MFE_OK;
}

mfe_status launch_zero_boundary(mfe_ctx* ctx, int nx, int ny, int nz, double* v)
{
  const int64_t N = (int64_t)(nx + 1) * (ny + 1) * (nz + 1);
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ceil_div(N, 256),
                                                                (int64_t)ctx->sm_count * 8));
  k_zero_boundary<<<(unsigned)blocks, 256, 0, ctx->stream>>>(nx + 1, ny + 1, nz + 1, v);
  return check_launch(ctx, "k_zero_boundary");
}

mfe_status launch_element_gradient(mfe_ctx* ctx, int nx, int ny, int nz, const double* u,
                                   const double* lambda, double* g)
{
  MFE_TRY(ensure_tables(ctx));
  const int64_t E = (int64_t)nx * ny * nz;
  k_elem_grad<<<(unsigned)ceil_div(E, kElemThreads), kElemThreads, 0, ctx->stream>>>(
      nx, ny, nz, E, u, lambda, g);
  return check_launch(ctx, "k_elem_grad");
}

}  // namespace mfe
