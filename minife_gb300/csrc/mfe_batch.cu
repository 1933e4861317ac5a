// Batched uneven boxes: nbox independent miniFE problems (each its own
// nx x ny x nz box, k = 1, the reference's boundary conditions) assembled
// into one concatenated store and solved with CG, all boxes advancing
// together: every iteration is one fixed sequence of launches over all
// boxes that are still iterating, captured once as a CUDA graph with a
// conditional while node.
//
// HBM layout.  Box b owns rows [row_base_b, row_base_b + n_b) of every
// concatenated vector and values [nnz_base_b, nnz_base_b + nnz_b) of the
// concatenated CSR values (FP64, plus an FP32 copy for the mixed solver);
// both bases are multiples of four elements, so every slice starts on a
// 16-byte boundary and the bulk copies of the box SpMV can round ranges
// outwards inside the slice.  Column indices are not stored: the box
// layout gives them in closed form (mfe_box.cuh).
//
// Work lists.  Each launch walks a list of boxes (those still iterating, or
// those taking a reliable update) in box order, with prefix sums of their
// SpMV tiles and vector chunks; one block rebuilds the lists after each
// iteration, so finished boxes cost nothing and the grid stays busy until
// the largest box converges.
//
// SpMV.  k_bx_spmv is the box SpMV of mfe_spmv_box.cu (warp-specialised:
// one producer lane stages a tile's values and nine x segments with bulk
// copies, consumer warps own one row per thread) over the global tile list
// of the launch.  Per-box dot products are deterministic: each consumer
// warp writes one partial per (box, CTA) it worked on; the last warp to
// finish a box (per-box counter) sums that box's partials in CTA order and
// forms the box's scalar (alpha or the true residual).
//
// Vectors.  k_bx_p / k_bx_update walk the chunk list (a tunable number of
// rows of one box per block pass); per-box r.r: one partial per chunk, the last block of
// the box sums them in chunk order.
//
// Solvers.  FP64: the reference's CG per box (cg_solve.hpp loop test with
// normr from the top of the iteration).  Mixed: FP32 values and vectors, FP64
// dots and scalars, FP64 solution; a box takes a reliable update (x += x32,
// r = b - A64 x in FP64, FP32 copy of r) when its recursive residual fell by
// inner_tol (default a hundredfold) since its last update, claims
// convergence, or after refine_k iterations, and it finishes only on its true
// FP64 residual (or after max_refine updates, when that cap is set).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "mfe_box.cuh"
#include "mfe_common.cuh"
#include "mfe_internal.h"
#include "mfe_stencil.cuh"

namespace mfe {

constexpr int kBxMaxBoxes = 1024;
constexpr int kBxVT = 256;       // vector-kernel block
constexpr int kBxPad = 4;        // slice alignment in elements

struct BoxDesc {
  int Nx, Ny, Nz, NxNy;
  int n;
  int ntiles32, ntiles64;  // SpMV tiles at the FP32 and FP64 shapes
  int nchunks, chunk_base;
  int64_t row_base;        // first row in the vectors (ghost zones either side)
  int64_t nnz_base;        // first value in the compressed FP64 values
  int64_t ell_base;        // first value in the padded FP32 values (27 per row)
};

struct BoxSt {
  double rr, rr_new, pAp, alpha, beta, rr_true, rr_upd, normr0, normr, tol_abs;
  double alpha_prev;  // mixed: alpha whose x32 += alpha p is still pending
  int open, gate, iters, since, brk;
  int x_pending;      // mixed: 1 while x32 += alpha_prev p is due
  int upd;            // mixed: reliable updates of this box
  unsigned cnt_mv, cnt_vec;
};

struct BatchCtl {
  int nbox, k, max_iter, refine_k, first, cont, status, updates, tol_mode;
  int max_refine;  // mixed: a box stops after this many updates (0: no cap)
  double delta2;
  unsigned err;
};

// Boxes taking part in a launch, in box order, with prefix sums of their
// tiles (FP32 and FP64 shapes) and vector chunks.
struct BxList {
  int* ids;
  int* tpre32;
  int* tpre64;
  int* cpre;
  int* count;
};

__host__ __device__ constexpr int bx_capv(int rows) { return ((rows * 27 + 8) + 3) & ~3; }
__host__ __device__ constexpr int bx_capx(int rows) { return ((rows + 2 + 8) + 3) & ~3; }
// dynamic shared memory of a box-SpMV launch shape (rows per tile, stages)
inline size_t bx_smem(size_t elem, int rows, int stages)
{
  return (size_t)stages * ((size_t)bx_capv(rows) + 9 * (size_t)bx_capx(rows)) * elem;
}
// FP64 products run at the one shape (FP64-FMA-bound); the FP32 shape is tunable
constexpr int kBx64Rows = 128, kBx64Stages = 2;

// position q of global index i in a prefix array pre[0..cnt] (pre[q] <= i <
// pre[q+1]), searching forward from a previous position
__device__ __forceinline__ int bx_advance(const int* pre, int cnt, int q, int i)
{
  if (q < 0 || __ldg(&pre[q]) > i) {
    int lo = 0, hi = cnt - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (__ldg(&pre[mid]) <= i) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  }
  while (q + 1 < cnt && __ldg(&pre[q + 1]) <= i) ++q;
  return q;
}

enum BxMode { BX_DOT = 1, BX_RESID = 2 };

template <typename T>
struct BxSpmvParams {
  const BoxDesc* boxes;
  BoxSt* st;
  const int* ids;
  const int* tpre;
  const int* count;
  const T* __restrict__ vals;
  const T* __restrict__ x;
  T* __restrict__ y;              // DOT output; RESID output when y32 is null
  const double* __restrict__ b;   // RESID
  float* __restrict__ y32;        // RESID output (FP32) when set
  double* slots;                  // [nbox][grid][consumer warps]
  unsigned* err;
};

// Tiles are split into contiguous ranges, one per CTA: CTA c takes tiles
// [bx_start(c), bx_start(c + 1)) of the launch's tile list.
__device__ __forceinline__ int bx_start(int c, int total, int G)
{
  return (int)(((int64_t)c * total) / G);
}

// Consumer warp cw of this CTA is done with box b (tiles [A, E) of the
// list): its partial goes to slot (b, CTA, cw); the last of the box's warps
// sums the slots of the CTAs whose ranges meet [A, E), in CTA order, and
// forms the box's scalar.
template <int MODE, int C>
__device__ void bx_flush(BoxSt* st, double* slots, int b, int A, int E, int total, int cw,
                         double dacc)
{
  const int lane = threadIdx.x & 31;
  const double v = warp_sum(dacc);
  const int G = gridDim.x;
  // first and last CTA whose range meets [A, E): bx_start(c) <= A < bx_start(c+1)
  const int c0 = (int)min((int64_t)(G - 1), ((int64_t)(A + 1) * G + total - 1) / total - 1);
  const int c1 = (int)min((int64_t)(G - 1), ((int64_t)E * G + total - 1) / total - 1);
  unsigned ranges = 0;  // CTAs in c0..c1 with a non-empty range
  if (total >= G) {
    ranges = (unsigned)(c1 - c0 + 1);
  } else {
    for (int c = c0 + lane; c <= c1; c += 32)
      ranges += bx_start(c + 1, total, G) > bx_start(c, total, G) ? 1u : 0u;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) ranges += __shfl_xor_sync(0xffffffffu, ranges, o);
  }
  double* slot = slots + (size_t)b * G * C;
  unsigned old = 0;
  if (lane == 0) {
    slot[(size_t)blockIdx.x * C + cw] = v;
    __threadfence();
    old = atomicAdd(&st[b].cnt_mv, 1u);
  }
  old = __shfl_sync(0xffffffffu, old, 0);
  if (old != ranges * C - 1) return;
  __threadfence();
  double sacc = 0.0;
  for (int c = c0 + lane; c <= c1; c += 32) {
    if (bx_start(c + 1, total, G) <= bx_start(c, total, G)) continue;
#pragma unroll
    for (int w = 0; w < C; ++w) sacc += __ldcg(&slot[(size_t)c * C + w]);
  }
  sacc = warp_sum(sacc);
  if (lane == 0) {
    BoxSt& bs = st[b];
    if (MODE == BX_DOT) {
      bs.pAp = sacc;
      if (sacc > 0.0) {
        bs.alpha = bs.rr / sacc;
      } else {
        bs.alpha = 0.0;
        bs.brk = 1;
      }
    } else {
      bs.rr_true = sacc;
    }
    bs.cnt_mv = 0u;
  }
}

// Box SpMV over the launch's tile list.  ELL: FP32 values in the padded
// 27-per-row layout (zeros for missing neighbours), so every row runs the
// unmasked 27-term code; otherwise the compressed CSR values with masked
// slots for boundary rows.  x has ghost zones of zeros around each box, so
// the nine segments are never clamped.
template <typename T, int MODE, bool ELL, int ROWS, int S>
__global__ void __launch_bounds__(ROWS + 32) k_bx_spmv(BxSpmvParams<T> P)
{
  constexpr int C = ROWS / 32;
  constexpr int capv = bx_capv(ROWS), capx = bx_capx(ROWS);
  constexpr int stage_elems = capv + 9 * capx;
  constexpr int VA = 16 / sizeof(T);
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t full[S], empty[S];
  __shared__ int s_vbase[S];
  __shared__ int s_xbase[S][9];
  __shared__ int s_ok[S];
  T* const st0 = reinterpret_cast<T*>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cnt = *P.count;
  if (cnt == 0) return;
  const int total = __ldg(&P.tpre[cnt]);
  const int t_begin = bx_start(blockIdx.x, total, gridDim.x);
  const int t_end = bx_start(blockIdx.x + 1, total, gridDim.x);
  if (t_begin >= t_end) return;
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], C);
    }
    fence_mbar_init();
  }
  __syncthreads();
  if (warp == 0) {
    if (lane == 0) {
      bool ok = true;
      int it = 0, q = -1;
      BoxDesc d{};
      int A = 0;
      for (int i = t_begin; i < t_end; ++i, ++it) {
        const int s = it % S;
        if (it >= S) ok = mbar_wait_bounded(&empty[s], (unsigned)(((it / S) - 1) & 1));
        if (!ok) break;
        const int nq = bx_advance(P.tpre, cnt, q, i);
        if (nq != q) {
          q = nq;
          d = P.boxes[__ldg(&P.ids[q])];
          A = __ldg(&P.tpre[q]);
        }
        const int lt = i - A;
        T* sv = st0 + (size_t)s * stage_elems;
        T* sx = sv + capv;
        const int r0 = lt * ROWS, r1 = min(d.n, r0 + ROWS);
        int av, bv;
        const T* vsrc;
        if (ELL) {
          av = 27 * r0;
          bv = (27 * r1 + VA - 1) & ~(VA - 1);
          vsrc = P.vals + d.ell_base;
        } else {
          const int a = (int)row_offset_of32(r0, d.Nx, d.Ny, d.Nz, d.NxNy);
          const int e = (int)row_offset_of32(r1, d.Nx, d.Ny, d.Nz, d.NxNy);
          av = a & ~(VA - 1);
          bv = (e + VA - 1) & ~(VA - 1);
          vsrc = P.vals + d.nnz_base;
        }
        bool fits = bv - av <= capv;
        int xlo[9], xhi[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const int off = (j / 3 - 1) * d.NxNy + (j % 3 - 1) * d.Nx;
          // inside the box's ghost zones: [-ghost, n + ghost)
          xlo[j] = (r0 + off - 1) & ~(VA - 1);
          xhi[j] = (r1 + off + 1 + VA - 1) & ~(VA - 1);
          fits = fits && xhi[j] - xlo[j] <= capx;
        }
        if (!fits) {
          // cannot happen for the stage capacities above
          atomicOr(P.err, ERR_TILE_OVERFLOW);
          s_ok[s] = 0;
          mbar_arrive_expect_tx(&full[s], 0);
          continue;
        }
        s_ok[s] = 1;
        s_vbase[s] = av;
        unsigned bytes = (unsigned)((bv - av) * sizeof(T));
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          s_xbase[s][j] = xlo[j];
          bytes += (unsigned)((xhi[j] - xlo[j]) * sizeof(T));
        }
        mbar_arrive_expect_tx(&full[s], bytes);
        bulk_g2s(sv, vsrc + av, (unsigned)((bv - av) * sizeof(T)), &full[s]);
#pragma unroll
        for (int j = 0; j < 9; ++j)
          bulk_g2s(sx + (size_t)j * capx, P.x + d.row_base + xlo[j],
                   (unsigned)((xhi[j] - xlo[j]) * sizeof(T)), &full[s]);
      }
      if (!ok) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        for (int st = 0; st < S && st < it; ++st)
          mbar_wait_bounded(&full[st], (unsigned)(((it - st + S - 1) / S - 1) & 1));
      }
    }
  } else {
    const int cw = warp - 1;
    const int lr = cw * 32 + lane;
    double dacc = 0.0;  // RESID, and DOT of FP64 operands
    DFAcc facc;         // DOT of FP32 operands
    int it = 0, q = -1, b = -1, A = 0, E = 0;
    BoxDesc d{};
    for (int i = t_begin; i < t_end; ++i, ++it) {
      const int s = it % S;
      const int nq = bx_advance(P.tpre, cnt, q, i);
      if (nq != q) {
        if (q >= 0) bx_flush<MODE, C>(P.st, P.slots, b, A, E, total, cw, dacc + facc.value());
        dacc = 0.0;
        facc = DFAcc{};
        q = nq;
        b = __ldg(&P.ids[q]);
        d = P.boxes[b];
        A = __ldg(&P.tpre[q]);
        E = __ldg(&P.tpre[q + 1]);
      }
      const int r = (i - A) * ROWS + lr;
      const bool active = r < d.n;
      int iz = 0, iy = 0, ix = 0, roff = 0;
      if (!ELL) {
        const int rr = active ? r : d.n - 1;
        iz = rr / d.NxNy;
        const int rem = rr - iz * d.NxNy;
        iy = rem / d.Nx;
        ix = rem - iy * d.Nx;
        roff = (int)row_offset(ix, iy, iz, d.Nx, d.Ny, d.Nz);
      } else {
        roff = 27 * r;
      }
      if (!mbar_wait_bounded(&full[s], (unsigned)((it / S) & 1))) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        break;
      }
      T sum = T(0), xr = T(0);
      const bool ok = active && s_ok[s] != 0;
      if (ok) {
        const T* sv = st0 + (size_t)s * stage_elems;
        const T* sx = sv + capv;
        const T* rowv = sv + (roff - s_vbase[s]);
        const T* xc = sx + 4 * capx + (r - s_xbase[s][4]);
        xr = xc[0];
        T s0 = T(0), s1 = T(0);
        const bool vxm = ELL || ix > 0, vxp = ELL || ix < d.Nx - 1;
        const bool vym = ELL || iy > 0, vyp = ELL || iy < d.Ny - 1;
        const bool vzm = ELL || iz > 0, vzp = ELL || iz < d.Nz - 1;
        // warps whose rows all have the full 27 columns take the unmasked code
        if (ELL || __all_sync(__activemask(), vxm && vxp && vym && vyp && vzm && vzp)) {
#pragma unroll
          for (int j = 0; j < 9; ++j) {
            const int off = (j / 3 - 1) * d.NxNy + (j % 3 - 1) * d.Nx;
            const T* seg = sx + j * capx + (r + off - s_xbase[s][j]);
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
              const int k = j * 3 + dx + 1;
              if (k & 1) s1 = fma(rowv[k], seg[dx], s1);
              else s0 = fma(rowv[k], seg[dx], s0);
            }
          }
        } else {
          const int cx = 1 + vxm + vxp, cy = 1 + vym + vyp, cxy = cx * cy;
          int slot = 0;
#pragma unroll
          for (int dz = -1; dz <= 1; ++dz) {
            const bool vz = dz < 0 ? vzm : (dz > 0 ? vzp : true);
            const int bz = dz < 0 ? 0 : (dz == 0 ? (int)vzm : (int)vzm + 1);
#pragma unroll
            for (int dy = -1; dy <= 1; ++dy) {
              const bool vy = dy < 0 ? vym : (dy > 0 ? vyp : true);
              const int by = dy < 0 ? 0 : (dy == 0 ? (int)vym : (int)vym + 1);
              const int j = (dz + 1) * 3 + (dy + 1);
              const int off = dz * d.NxNy + dy * d.Nx;
              const T* seg = sx + j * capx + (r + off - s_xbase[s][j]);
              const int pbase = bz * cxy + by * cx;
#pragma unroll
              for (int dx = -1; dx <= 1; ++dx) {
                const bool vx = dx < 0 ? vxm : (dx > 0 ? vxp : true);
                const int bx = dx < 0 ? 0 : (dx == 0 ? (int)vxm : (int)vxm + 1);
                const bool valid = vz && vy && vx;
                const T v = rowv[valid ? pbase + bx : 0];
                const T xv = *(valid ? seg + dx : xc);
                if (slot & 1) {
                  const T t1 = fma(v, xv, s1);
                  s1 = valid ? t1 : s1;
                } else {
                  const T t0 = fma(v, xv, s0);
                  s0 = valid ? t0 : s0;
                }
                ++slot;
              }
            }
          }
        }
        sum = s0 + s1;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (ok) {
        const int64_t g = d.row_base + r;
        if (MODE == BX_RESID) {
          const double res = P.b[g] - widen(sum);
          if (P.y32) P.y32[g] = (float)res;
          else P.y[g] = (T)res;
          dacc = fma(res, res, dacc);
        } else {
          P.y[g] = sum;
          if constexpr (sizeof(T) == 4)
            facc.add_product(sum, xr);
          else
            dacc = fma(sum, xr, dacc);
        }
      }
    }
    if (q >= 0) bx_flush<MODE, C>(P.st, P.slots, b, A, E, total, cw, dacc + facc.value());
  }
}

// FP32 values of box b in the padded 27-per-row layout (slot k = (dz, dy, dx)
// in the CSR column order; zero where the neighbour lies outside the box)
__global__ void k_bx_ell(BoxDesc d, const double* __restrict__ vals64, float* __restrict__ ell)
{
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < d.n; r += gridDim.x * blockDim.x) {
    const int iz = r / d.NxNy, rem = r - iz * d.NxNy, iy = rem / d.Nx, ix = rem - iy * d.Nx;
    int64_t k = d.nnz_base + row_offset(ix, iy, iz, d.Nx, d.Ny, d.Nz);
    float* out = ell + d.ell_base + (int64_t)27 * r;
    int slot = 0;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx, ++slot) {
          const bool in = ix + dx >= 0 && ix + dx < d.Nx && iy + dy >= 0 && iy + dy < d.Ny &&
                          iz + dz >= 0 && iz + dz < d.Nz;
          out[slot] = in ? (float)vals64[k++] : 0.0f;
        }
  }
}

// Batched FP32 stencil SpMV of the mixed solver, used when every box is a
// verified miniFE box operator (stencil_prepare_box): the z-marching kernel
// of mfe_stencil.cu over the (box, plane tile, z) steps of the listed boxes
// (tpre holds their prefix sums, box-major, then tile-major), in each box's
// natural layout inside its ghost zones (the per-plane copy phase follows the
// row's address mod 4), with the box's 27 interior coefficients in registers
// and its p.Ap finished by bx_flush.
struct BxStParams {
  const BoxDesc* boxes;
  BoxSt* st;
  const int* ids;
  const int* tpre;
  const int* count;
  const float* coef;  // [nbox][28]: interior stencil (slot order), Dirichlet diagonal
  const float* __restrict__ x;
  float* __restrict__ y;
  double* slots;      // [nbox][grid][kSC]
  unsigned* err;
};

// first float of the 16-byte aligned copy of line (z, dy = j - 1) of a box for
// plane positions [c0, c1), and one past its last
__device__ __forceinline__ int64_t bxs_lo(const BoxDesc& d, int z, int j, int c0)
{
  return ((int64_t)z * d.NxNy + (int64_t)(j - 1) * d.Nx + c0 - 1) & ~(int64_t)3;
}
__device__ __forceinline__ int64_t bxs_hi(const BoxDesc& d, int z, int j, int c1)
{
  return ((int64_t)z * d.NxNy + (int64_t)(j - 1) * d.Nx + c1 + 1 + 3) & ~(int64_t)3;
}

__global__ void __launch_bounds__(kSP + 32, 2) k_bx_stencil(const __grid_constant__ BxStParams P)
{
  extern __shared__ __align__(128) unsigned char bxs_smem[];
  float* const ring = reinterpret_cast<float*>(bxs_smem);
  __shared__ uint64_t full[kSS], empty[kSS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cnt = *P.count;
  if (cnt == 0) return;
  const int total = __ldg(&P.tpre[cnt]);
  const int t_begin = bx_start(blockIdx.x, total, gridDim.x);
  const int t_end = bx_start(blockIdx.x + 1, total, gridDim.x);
  if (t_begin >= t_end) return;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kSS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kSC);
    }
    fence_mbar_init();
  }
  __syncthreads();
  // Slot sequence of a run of rows za .. zb-1 of one plane tile: planes
  // (za-1, za), then z+1 .. z+min(3, zb-z) for z = za, za+3, ...
  if (warp == 0) {
    if (lane == 0) {
      bool ok = true;
      int it = 0, q = -1, A = 0, E = 0;
      BoxDesc d{};
      for (int i = t_begin; ok && i < t_end;) {
        const int nq = bx_advance(P.tpre, cnt, q, i);
        if (nq != q) {
          q = nq;
          d = P.boxes[__ldg(&P.ids[q])];
          A = __ldg(&P.tpre[q]);
          E = __ldg(&P.tpre[q + 1]);
        }
        const int tile = (i - A) / d.Nz, za = (i - A) - tile * d.Nz;
        const int zb = min(d.Nz, za + (min(t_end, E) - i));
        const int c0 = tile * kSP, c1 = min(d.NxNy, c0 + kSP);
        const float* xb = P.x + d.row_base;
        for (int z = za - 3; z < zb; z += 3, ++it) {
          const int zf = z < za ? za - 1 : z + 1;
          const int np = z < za ? 2 : min(3, zb - z);  // planes zf .. zf+np-1
          const int s = it % kSS;
          if (it >= kSS) ok = mbar_wait_bounded(&empty[s], (unsigned)(((it / kSS) - 1) & 1));
          if (!ok) break;
          unsigned bytes = 0;
          for (int pl = 0; pl < np; ++pl)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              bytes += (unsigned)((bxs_hi(d, zf + pl, j, c1) - bxs_lo(d, zf + pl, j, c0)) * sizeof(float));
          mbar_arrive_expect_tx(&full[s], bytes);
          for (int pl = 0; pl < np; ++pl)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const int64_t lo = bxs_lo(d, zf + pl, j, c0);
              bulk_g2s(ring + s * kSSlot + (pl * 3 + j) * kSCap, xb + lo,
                       (unsigned)((bxs_hi(d, zf + pl, j, c1) - lo) * sizeof(float)), &full[s]);
            }
        }
        i += zb - za;
      }
      if (!ok) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        for (int st = 0; st < kSS && st < it; ++st)
          mbar_wait_bounded(&full[st], (unsigned)(((it - st + kSS - 1) / kSS - 1) & 1));
      }
    }
  } else {
    const int cw = warp - 1;
    const int lr = cw * 32 + lane;
    bool ok = true;
    int it = 0, q = -1, b = -1, A = 0, E = 0;
    BoxDesc d{};
    DFAcc facc;
    float sv[27], dd = 0.0f;
    StPlane W0, W1, W2;
    int c = 0, cc = 0, c0 = 0;
    bool active = false, dir = false, mxl = false, mxh = false, myl = false, myh = false, wm = false;
    const float* sx = ring;
    auto wait_slot = [&]() {
      const int s = it % kSS;
      sx = ring + s * kSSlot + (cc - c0 + 1);
      return mbar_wait_bounded(&full[s], (unsigned)((it / kSS) & 1));
    };
    auto release_slot = [&]() {
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[it % kSS]);
      ++it;
    };
    // plane z (the slot's plane pl) around position cc into W, masked neighbours zeroed
    auto load_plane = [&](int pl, int z, StPlane& W) {
      const unsigned zb0 = (unsigned)z * (unsigned)d.NxNy + (unsigned)(c0 - 1);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        // the copy starts (base + c0 - 1) mod 4 floats before position c0 - 1
        const float* seg = sx + (pl * 3 + j) * kSCap + ((zb0 + (unsigned)((j - 1) * d.Nx)) & 3u);
        W.v[j * 3 + 0] = seg[-1];
        W.v[j * 3 + 1] = seg[0];
        W.v[j * 3 + 2] = seg[1];
      }
      if (wm) {  // the same for the whole warp
        if (mxl) W.v[0] = W.v[3] = W.v[6] = 0.0f;
        if (mxh) W.v[2] = W.v[5] = W.v[8] = 0.0f;
        if (myl) W.v[0] = W.v[1] = W.v[2] = 0.0f;
        if (myh) W.v[6] = W.v[7] = W.v[8] = 0.0f;
      }
    };
    const auto cf = [&](int k) { return sv[k]; };
    auto finish = [&](int z, float sum, const StPlane& B) {
      sum = dir ? dd * B.v[4] : sum;
      if (active) {
        P.y[d.row_base + (int64_t)z * d.NxNy + c] = sum;
        facc.add_product(sum, B.v[4]);
      }
    };
    auto row = [&](int z, const StPlane& A_, const StPlane& B, const StPlane& C) {
      finish(z, st_row_sum(cf, dd, z, d.Nz, A_, B, C), B);  // z is the same for the warp
    };
    for (int i = t_begin; ok && i < t_end;) {
      const int nq = bx_advance(P.tpre, cnt, q, i);
      if (nq != q) {
        if (q >= 0) bx_flush<BX_DOT, kSC>(P.st, P.slots, b, A, E, total, cw, facc.value());
        facc = DFAcc{};
        q = nq;
        b = __ldg(&P.ids[q]);
        d = P.boxes[b];
        A = __ldg(&P.tpre[q]);
        E = __ldg(&P.tpre[q + 1]);
#pragma unroll
        for (int k = 0; k < 27; ++k) sv[k] = __ldg(P.coef + (size_t)b * 28 + k);
        dd = __ldg(P.coef + (size_t)b * 28 + 27);
      }
      const int tile = (i - A) / d.Nz, za = (i - A) - tile * d.Nz;
      const int zb = min(d.Nz, za + (min(t_end, E) - i));
      c0 = tile * kSP;
      const int c1 = min(d.NxNy, c0 + kSP);
      c = c0 + lr;
      active = c < c1;
      cc = active ? c : c1 - 1;
      const int iy = cc / d.Nx, ix = cc - iy * d.Nx;
      dir = ix == 0 || ix == d.Nx - 1 || iy == 0 || iy == d.Ny - 1;
      mxl = ix == 1;
      mxh = ix == d.Nx - 2;
      myl = iy == 1;
      myh = iy == d.Ny - 2;
      wm = __any_sync(0xffffffffu, mxl || mxh || myl || myh);
      ok = wait_slot();
      if (!ok) break;
      load_plane(0, za - 1, W0);
      load_plane(1, za, W1);
      release_slot();
      for (int z = za; z < zb; z += 3) {
        if (!wait_slot()) {
          ok = false;
          break;
        }
        load_plane(0, z + 1, W2);
        row(z, W0, W1, W2);
        if (z + 1 < zb) {
          load_plane(1, z + 2, W0);
          row(z + 1, W1, W2, W0);
        }
        if (z + 2 < zb) {
          load_plane(2, z + 3, W1);
          row(z + 2, W2, W0, W1);
        }
        release_slot();
      }
      i += zb - za;
    }
    if (!ok) atomicOr(P.err, ERR_WAIT_TIMEOUT);
    if (q >= 0) bx_flush<BX_DOT, kSC>(P.st, P.slots, b, A, E, total, cw, facc.value());
  }
}

// Two adjacent plane positions per consumer thread (c - c0 even, c + 1) over
// 512-position tiles, for batches whose boxes all have mirror-symmetric
// stencils: a coefficient then depends only on (|dz|, |dy|, |dx|), so a box
// needs 8 weights in registers (w[4|dz| + 2|dy| + |dx|]); each plane of the
// window x[c-1 .. c+2] is reduced once to its per-class sums for the two
// rows (st_sep_reduce) and a row takes 8 FMAs (st_sep_rows).  Both y neighbours of a position are
// at -Nx / +Nx in the flattened plane, so a pair needs the same three lines;
// a pair that straddles two x lines is two Dirichlet rows (ix = Nx-1 and 0),
// whose results are replaced by dd * x.  Natural layout: four scalar loads
// per line (the copy phase follows the row's address mod 4).
constexpr int kB2P = 512;
constexpr int kB2Cap = ((kB2P + 9) + 3) & ~3;  // copies hold x[c0-1-phase .. c1+1]
constexpr int kB2Slot = kSKP * 3 * kB2Cap;
constexpr size_t kB2Smem = sizeof(float) * kSS * kB2Slot;
static_assert((kB2Cap * sizeof(float)) % 16 == 0, "bulk-copy destinations stay 16-byte aligned");

// one past the last float of the copy of line (z, dy = j - 1) for the pair
// kernel: its last row c1 - 1 reads x[c1 + 1]
__device__ __forceinline__ int64_t bxs_hi2(const BoxDesc& d, int z, int j, int c1)
{
  return ((int64_t)z * d.NxNy + (int64_t)(j - 1) * d.Nx + c1 + 2 + 3) & ~(int64_t)3;
}

struct BxPlane2 {
  float v[12];  // line j: x[c-1], x[c], x[c+1], x[c+2]
  float c0, c1;  // unmasked centres
};

__global__ void __launch_bounds__(kB2P / 2 + 32, 2) k_bx_stencil2(const __grid_constant__ BxStParams P)
{
  extern __shared__ __align__(128) unsigned char bx2_smem[];
  float* const ring = reinterpret_cast<float*>(bx2_smem);
  __shared__ uint64_t full[kSS], empty[kSS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int cnt = *P.count;
  if (cnt == 0) return;
  const int total = __ldg(&P.tpre[cnt]);
  const int t_begin = bx_start(blockIdx.x, total, gridDim.x);
  const int t_end = bx_start(blockIdx.x + 1, total, gridDim.x);
  if (t_begin >= t_end) return;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kSS; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kSC);
    }
    fence_mbar_init();
  }
  __syncthreads();
  if (warp == 0) {
    if (lane == 0) {
      bool ok = true;
      int it = 0, q = -1, A = 0, E = 0;
      BoxDesc d{};
      for (int i = t_begin; ok && i < t_end;) {
        const int nq = bx_advance(P.tpre, cnt, q, i);
        if (nq != q) {
          q = nq;
          d = P.boxes[__ldg(&P.ids[q])];
          A = __ldg(&P.tpre[q]);
          E = __ldg(&P.tpre[q + 1]);
        }
        const int tile = (i - A) / d.Nz, za = (i - A) - tile * d.Nz;
        const int zb = min(d.Nz, za + (min(t_end, E) - i));
        const int c0 = tile * kB2P, c1 = min(d.NxNy, c0 + kB2P);
        const float* xb = P.x + d.row_base;
        for (int z = za - 3; z < zb; z += 3, ++it) {
          const int zf = z < za ? za - 1 : z + 1;
          const int np = z < za ? 2 : min(3, zb - z);  // planes zf .. zf+np-1
          const int s = it % kSS;
          if (it >= kSS) ok = mbar_wait_bounded(&empty[s], (unsigned)(((it / kSS) - 1) & 1));
          if (!ok) break;
          unsigned bytes = 0;
          for (int pl = 0; pl < np; ++pl)
#pragma unroll
            for (int j = 0; j < 3; ++j)
              bytes += (unsigned)((bxs_hi2(d, zf + pl, j, c1) - bxs_lo(d, zf + pl, j, c0)) * sizeof(float));
          mbar_arrive_expect_tx(&full[s], bytes);
          for (int pl = 0; pl < np; ++pl)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
              const int64_t lo = bxs_lo(d, zf + pl, j, c0);
              bulk_g2s(ring + s * kB2Slot + (pl * 3 + j) * kB2Cap, xb + lo,
                       (unsigned)((bxs_hi2(d, zf + pl, j, c1) - lo) * sizeof(float)), &full[s]);
            }
        }
        i += zb - za;
      }
      if (!ok) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        for (int st = 0; st < kSS && st < it; ++st)
          mbar_wait_bounded(&full[st], (unsigned)(((it - st + kSS - 1) / kSS - 1) & 1));
      }
    }
  } else {
    const int cw = warp - 1;
    const int lr = cw * 32 + lane;
    bool ok = true;
    int it = 0, q = -1, b = -1, A = 0, E = 0;
    BoxDesc d{};
    DFAcc facc;
    float w[8] = {}, dd = 0.0f;
    StSep2 W0, W1, W2;
    int c = 0, c0 = 0, cc = 0;
    bool act0 = false, act1 = false, sp0 = false, sp1 = false;
    bool m1 = false, m2 = false, m3 = false, myl = false, myh = false, wm = false;
    const float* sx = ring;
    auto wait_slot = [&]() {
      const int s = it % kSS;
      sx = ring + s * kB2Slot + (cc - c0 + 1);
      return mbar_wait_bounded(&full[s], (unsigned)((it / kSS) & 1));
    };
    auto release_slot = [&]() {
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[it % kSS]);
      ++it;
    };
    // plane z (the slot's plane pl) around positions cc, cc + 1 into W
    auto load_plane = [&](int pl, int z, StSep2& Wo) {
      BxPlane2 W;
      const unsigned zb0 = (unsigned)z * (unsigned)d.NxNy + (unsigned)(c0 - 1);
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        // sx points at x[cc] of a copy starting at position c0 - 1 (phase 0)
        const float* seg = sx + (pl * 3 + j) * kB2Cap + ((zb0 + (unsigned)((j - 1) * d.Nx)) & 3u);
        W.v[4 * j] = seg[-1];
        W.v[4 * j + 1] = seg[0];
        W.v[4 * j + 2] = seg[1];
        W.v[4 * j + 3] = seg[2];
        if (j == 1) {
          W.c0 = seg[0];
          W.c1 = seg[1];
        }
      }
      if (wm) {  // the same for the whole warp
        if (m1) W.v[1] = W.v[5] = W.v[9] = 0.0f;   // x[c]: c is Dirichlet (ix = 0)
        if (m2) W.v[2] = W.v[6] = W.v[10] = 0.0f;  // x[c+1]: c + 1 is Dirichlet
        if (m3) W.v[3] = W.v[7] = W.v[11] = 0.0f;  // x[c+2]: Dirichlet, used by c + 1 only
        if (myl) W.v[0] = W.v[1] = W.v[2] = W.v[3] = 0.0f;
        if (myh) W.v[8] = W.v[9] = W.v[10] = W.v[11] = 0.0f;
      }
      st_sep_reduce(W.v, W.c0, W.c1, Wo);
    };
    // p.Ap: the pair's two products summed in FP32, the running sum in
    // double-float (act1 implies act0)
    auto finish = [&](int z, float s0, float s1, const StSep2& B) {
      s0 = sp0 ? dd * B.c0 : s0;
      s1 = sp1 ? dd * B.c1 : s1;
      const int64_t g = d.row_base + (int64_t)z * d.NxNy + c;
      if (act0) {
        P.y[g] = s0;
        float pr = s0 * B.c0;
        if (act1) {
          P.y[g + 1] = s1;
          pr = fmaf(s1, B.c1, pr);
        }
        facc.add(pr);
      }
    };
    const auto wf = [&](int k) { return w[k]; };
    auto row = [&](int z, const StSep2& A_, const StSep2& B, const StSep2& C) {
      float s0, s1;
      // z cases are the same for the whole warp
      if (z >= 2 && z <= d.Nz - 3) {
        st_sep_rows<true, true>(wf, A_, B, C, s0, s1);
      } else if (z == 0 || z == d.Nz - 1) {
        s0 = dd * B.c0;
        s1 = dd * B.c1;
      } else if (z == 1 && z == d.Nz - 2) {
        st_sep_rows<false, false>(wf, A_, B, C, s0, s1);
      } else if (z == 1) {
        st_sep_rows<false, true>(wf, A_, B, C, s0, s1);
      } else {
        st_sep_rows<true, false>(wf, A_, B, C, s0, s1);
      }
      finish(z, s0, s1, B);
    };
    for (int i = t_begin; ok && i < t_end;) {
      const int nq = bx_advance(P.tpre, cnt, q, i);
      if (nq != q) {
        if (q >= 0) bx_flush<BX_DOT, kSC>(P.st, P.slots, b, A, E, total, cw, facc.value());
        facc = DFAcc{};
        q = nq;
        b = __ldg(&P.ids[q]);
        d = P.boxes[b];
        A = __ldg(&P.tpre[q]);
        E = __ldg(&P.tpre[q + 1]);
#pragma unroll
        for (int k = 0; k < 8; ++k) w[k] = __ldg(P.coef + (size_t)b * 28 + k);
        dd = __ldg(P.coef + (size_t)b * 28 + 27);
      }
      const int tile = (i - A) / d.Nz, za = (i - A) - tile * d.Nz;
      const int zb = min(d.Nz, za + (min(t_end, E) - i));
      c0 = tile * kB2P;
      const int c1 = min(d.NxNy, c0 + kB2P);
      c = c0 + 2 * lr;
      act0 = c < c1;
      act1 = c + 1 < c1;
      cc = act0 ? c : c1 - 1;  // c1 - 1 >= c0, and cc + 2 stays inside the copy
      const int iy = cc / d.Nx, ix0 = cc - iy * d.Nx, ix1 = ix0 + 1;
      const bool dy = iy == 0 || iy == d.Ny - 1;
      sp0 = dy || ix0 == 0 || ix0 == d.Nx - 1;
      // ix1 == Nx: c + 1 starts the next x line (ix 0, a Dirichlet node)
      sp1 = dy || ix1 >= d.Nx - 1;
      m1 = ix1 == 1;
      m2 = ix0 == d.Nx - 2;
      m3 = ix1 == d.Nx - 2;
      myl = iy == 1;
      myh = iy == d.Ny - 2;
      wm = __any_sync(0xffffffffu, m1 || m2 || m3 || myl || myh);
      ok = wait_slot();
      if (!ok) break;
      load_plane(0, za - 1, W0);
      load_plane(1, za, W1);
      release_slot();
      for (int z = za; z < zb; z += 3) {
        if (!wait_slot()) {
          ok = false;
          break;
        }
        load_plane(0, z + 1, W2);
        row(z, W0, W1, W2);
        if (z + 1 < zb) {
          load_plane(1, z + 2, W0);
          row(z + 1, W1, W2, W0);
        }
        if (z + 2 < zb) {
          load_plane(2, z + 3, W1);
          row(z + 2, W2, W0, W1);
        }
        release_slot();
      }
      i += zb - za;
    }
    if (!ok) atomicOr(P.err, ERR_WAIT_TIMEOUT);
    if (q >= 0) bx_flush<BX_DOT, kSC>(P.st, P.slots, b, A, E, total, cw, facc.value());
  }
}

// ---------------------------------------------------------------------------
// vector kernels over the chunk list
// ---------------------------------------------------------------------------
// 16-byte vectors of the work arrays (chunks start on 16-byte boundaries)
template <typename V>
struct BxVec16;
template <>
struct BxVec16<float> {
  using type = float4;
  static constexpr int n = 4;
};
template <>
struct BxVec16<double> {
  using type = double2;
  static constexpr int n = 2;
};
template <typename V>
__device__ __forceinline__ V& bx_comp(typename BxVec16<V>::type& v, int c)
{
  return reinterpret_cast<V*>(&v)[c];
}

struct BxVecParams {
  const BoxDesc* boxes;
  BoxSt* st;
  BatchCtl* ctl;
  const int* ids;
  const int* cpre;
  const int* count;
  double* chunk_part;  // [total chunks], static chunk index
  int chunk;           // rows per chunk (multiple of 4)
};

// p = r + beta_b p (p = r on the first iteration).  Mixed (V = float): the
// box's previous x32 += alpha p is done here, where the old p is read anyway,
// unless its reliable update already folded it in (k_bx_xupdate).
template <typename V>
__global__ void __launch_bounds__(kBxVT)
    k_bx_p(BxVecParams Q, const V* __restrict__ r, V* __restrict__ p, float* __restrict__ x32)
{
  const int cnt = *Q.count;
  if (cnt == 0) return;
  const int total = __ldg(&Q.cpre[cnt]);
  const bool first = Q.ctl->first != 0;
  int q = -1;
  for (int c = blockIdx.x; c < total; c += gridDim.x) {
    q = bx_advance(Q.cpre, cnt, q, c);
    const int b = __ldg(&Q.ids[q]);
    const BoxDesc& d = Q.boxes[b];
    const int lc = c - __ldg(&Q.cpre[q]);
    const int64_t g0 = d.row_base + (int64_t)lc * Q.chunk;
    const int len = min(Q.chunk, d.n - lc * Q.chunk);
    const V beta = (V)Q.st[b].beta;
    const bool addx = sizeof(V) == 4 && !first && Q.st[b].x_pending != 0;
    const float alpha = (float)Q.st[b].alpha_prev;
    using VV = typename BxVec16<V>::type;
    constexpr int VW = BxVec16<V>::n;
    const VV* r4 = reinterpret_cast<const VV*>(r + g0);
    VV* p4 = reinterpret_cast<VV*>(p + g0);
    for (int k = threadIdx.x; k < len / VW; k += kBxVT) {
      const VV rv = r4[k];
      VV pv = rv;
      if (!first) {
        pv = p4[k];
        if constexpr (sizeof(V) == 4) {
          if (addx) {
            float4* x4 = reinterpret_cast<float4*>(x32 + g0);
            float4 xv = x4[k];
            const float4 po = reinterpret_cast<const float4&>(pv);
            xv.x = fmaf(alpha, po.x, xv.x);
            xv.y = fmaf(alpha, po.y, xv.y);
            xv.z = fmaf(alpha, po.z, xv.z);
            xv.w = fmaf(alpha, po.w, xv.w);
            x4[k] = xv;
          }
        }
#pragma unroll
        for (int c = 0; c < VW; ++c)
          bx_comp<V>(pv, c) = fma(beta, bx_comp<V>(pv, c), bx_comp<V>(const_cast<VV&>(rv), c));
      }
      p4[k] = pv;
    }
    for (int k = len / VW * VW + threadIdx.x; k < len; k += kBxVT) {
      const int64_t g = g0 + k;
      if constexpr (sizeof(V) == 4) {
        if (addx) x32[g] = fmaf(alpha, (float)p[g], x32[g]);
      }
      p[g] = first ? r[g] : fma(beta, p[g], r[g]);
    }
  }
}

// x += alpha_b p, r -= alpha_b Ap, rr_new_b = r.r over the box's chunks (x is
// x32 in the mixed solver, the FP64 solution otherwise)
template <typename V>
__global__ void __launch_bounds__(kBxVT)
    k_bx_update(BxVecParams Q, V* __restrict__ x, V* __restrict__ r, const V* __restrict__ p,
                const V* __restrict__ Ap)
{
  __shared__ double red[32];
  __shared__ bool last;
  const int cnt = *Q.count;
  if (cnt == 0) return;
  const int total = __ldg(&Q.cpre[cnt]);
  int q = -1;
  for (int c = blockIdx.x; c < total; c += gridDim.x) {
    q = bx_advance(Q.cpre, cnt, q, c);
    const int b = __ldg(&Q.ids[q]);
    const BoxDesc& d = Q.boxes[b];
    const int lc = c - __ldg(&Q.cpre[q]);
    const int64_t g0 = d.row_base + (int64_t)lc * Q.chunk;
    const int len = min(Q.chunk, d.n - lc * Q.chunk);
    const V alpha = (V)Q.st[b].alpha;
    double acc = 0.0;
    DFAcc facc;
    using VV = typename BxVec16<V>::type;
    constexpr int VW = BxVec16<V>::n;
    VV* x4 = reinterpret_cast<VV*>(x + g0);
    VV* r4 = reinterpret_cast<VV*>(r + g0);
    const VV* p4 = reinterpret_cast<const VV*>(p + g0);
    const VV* a4 = reinterpret_cast<const VV*>(Ap + g0);
    // mixed (V = float): x32 += alpha p is left pending (k_bx_p / k_bx_xupdate)
    constexpr bool kX = sizeof(V) == 8;
    for (int k = threadIdx.x; k < len / VW; k += kBxVT) {
      VV xv, rv = r4[k], pv, av = a4[k];
      if constexpr (kX) {
        xv = x4[k];
        pv = p4[k];
      }
#pragma unroll
      for (int c = 0; c < VW; ++c) {
        if constexpr (kX) bx_comp<V>(xv, c) = fma(alpha, bx_comp<V>(pv, c), bx_comp<V>(xv, c));
        const V rn = fma(-alpha, bx_comp<V>(av, c), bx_comp<V>(rv, c));
        bx_comp<V>(rv, c) = rn;
        if constexpr (sizeof(V) == 4)
          facc.add_product(rn, rn);
        else
          acc = fma(rn, rn, acc);
      }
      if constexpr (kX) x4[k] = xv;
      r4[k] = rv;
    }
    for (int k = len / VW * VW + threadIdx.x; k < len; k += kBxVT) {
      const int64_t g = g0 + k;
      if constexpr (kX) x[g] = fma(alpha, p[g], x[g]);
      const V rn = fma(-alpha, Ap[g], r[g]);
      r[g] = rn;
      if constexpr (sizeof(V) == 4)
        facc.add_product(rn, rn);
      else
        acc = fma(rn, rn, acc);
    }
    const double bt = block_sum(acc + facc.value(), red);
    if (threadIdx.x == 0) {
      Q.chunk_part[d.chunk_base + lc] = bt;
      __threadfence();
      last = atomicAdd(&Q.st[b].cnt_vec, 1u) == (unsigned)d.nchunks - 1;
    }
    __syncthreads();
    if (last) {
      __threadfence();
      double s = 0.0;
      for (int k = threadIdx.x; k < d.nchunks; k += kBxVT) s += __ldcg(&Q.chunk_part[d.chunk_base + k]);
      s = block_sum(s, red);
      if (threadIdx.x == 0) {
        Q.st[b].rr_new = s;
        Q.st[b].cnt_vec = 0u;
        if constexpr (!kX) {
          Q.st[b].alpha_prev = Q.st[b].alpha;
          Q.st[b].x_pending = 1;
        }
      }
    }
    __syncthreads();
  }
}

// x += x32 + alpha p (the pending update, the same FP32 FMA k_bx_p would do),
// x32 = 0 over the chunks of the listed (gated) boxes
__global__ void __launch_bounds__(kBxVT)
    k_bx_xupdate(BxVecParams Q, double* __restrict__ x, float* __restrict__ x32,
                 const float* __restrict__ p)
{
  const int cnt = *Q.count;
  if (cnt == 0) return;
  const int total = __ldg(&Q.cpre[cnt]);
  int q = -1;
  for (int c = blockIdx.x; c < total; c += gridDim.x) {
    q = bx_advance(Q.cpre, cnt, q, c);
    const int b = __ldg(&Q.ids[q]);
    const BoxDesc& d = Q.boxes[b];
    const int lc = c - __ldg(&Q.cpre[q]);
    const int64_t g0 = d.row_base + (int64_t)lc * Q.chunk;
    const int len = min(Q.chunk, d.n - lc * Q.chunk);
    const float alpha = (float)Q.st[b].alpha_prev;
    for (int k = threadIdx.x; k < len; k += kBxVT) {
      x[g0 + k] += f2d_exact(fmaf(alpha, p[g0 + k], x32[g0 + k]));
      x32[g0 + k] = 0.0f;
    }
    if (lc == 0 && threadIdx.x == 0) Q.st[b].x_pending = 0;  // read next by k_bx_p only
  }
}

// ---------------------------------------------------------------------------
// per-box bookkeeping: one block of 1024 threads, box b on thread b
// ---------------------------------------------------------------------------
// Rebuilds `list` from the boxes whose flag is set (block-wide exclusive scan
// of their tile and chunk counts).
__device__ void bx_build_list(const BoxDesc* boxes, int nbox, bool flag, BxList L)
{
  __shared__ int wsum[4][32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const bool f = t < nbox && flag;
  int v[4] = {f ? 1 : 0, f ? boxes[t].ntiles32 : 0, f ? boxes[t].ntiles64 : 0, f ? boxes[t].nchunks : 0};
  int inc[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    int x = v[k];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    inc[k] = x;
    if (lane == 31) wsum[k][w] = x;
  }
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      int x = wsum[k][lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      wsum[k][lane] = x;  // inclusive over warps
    }
  }
  __syncthreads();
  int ex[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) ex[k] = inc[k] - v[k] + (w > 0 ? wsum[k][w - 1] : 0);
  if (f) {
    L.ids[ex[0]] = t;
    L.tpre32[ex[0]] = ex[1];
    L.tpre64[ex[0]] = ex[2];
    L.cpre[ex[0]] = ex[3];
  }
  if (t == blockDim.x - 1) {
    const int n = ex[0] + v[0];
    *L.count = n;
    L.tpre32[n] = ex[1] + v[1];
    L.tpre64[n] = ex[2] + v[2];
    L.cpre[n] = ex[3] + v[3];
  }
  __syncthreads();
}

// after the initial residual: normr0, tolerances, open boxes
__global__ void __launch_bounds__(1024) k_bx_init(const BoxDesc* boxes, BoxSt* st, BatchCtl* ctl, BxList open)
{
  const int b = threadIdx.x;
  const int nbox = ctl->nbox;
  bool f = false;
  if (b < nbox) {
    BoxSt& s = st[b];
    const double nrm = sqrt(s.rr_true);
    s.normr0 = nrm;
    s.normr = nrm;
    if (ctl->tol_mode) s.tol_abs *= nrm;
    s.rr = s.rr_true;
    s.rr_upd = s.rr_true;
    s.iters = 0;
    s.since = 0;
    s.gate = 0;
    s.brk = 0;
    s.open = nrm > s.tol_abs && ctl->max_iter > 0;
    f = s.open;
  }
  __syncthreads();
  bx_build_list(boxes, nbox, f, open);
  if (b == 0) ctl->cont = *open.count > 0;
}

__global__ void k_bx_begin(const BatchCtl* ctl, cudaGraphConditionalHandle h)
{
  cudaGraphSetConditional(h, ctl->cont ? 1u : 0u);
}

// Mixed solver, after the update: which open boxes take a reliable update
// this iteration (gate list).
__global__ void __launch_bounds__(1024) k_bx_decide(const BoxDesc* boxes, BoxSt* st, BatchCtl* ctl, BxList gate)
{
  const int b = threadIdx.x;
  const int nbox = ctl->nbox;
  const int k = ctl->k + 1;
  bool f = false;
  if (b < nbox && st[b].open) {
    BoxSt& s = st[b];
    s.since += 1;
    const double t = s.rr_new;
    const bool ready = t < ctl->delta2 * s.rr_upd || t <= s.tol_abs * s.tol_abs;
    s.gate = !s.brk && (ready || s.since >= ctl->refine_k || k >= ctl->max_iter);
    f = s.gate;
  }
  __syncthreads();
  bx_build_list(boxes, nbox, f, gate);
}

// Mixed solver, end of iteration: finish boxes whose true residual meets
// the tolerance, restart the recursion of the others from it, rebuild the
// open list.
__global__ void __launch_bounds__(1024)
    k_bx_after(const BoxDesc* boxes, BoxSt* st, BatchCtl* ctl, BxList open,
               cudaGraphConditionalHandle h, int in_graph)
{
  const int b = threadIdx.x;
  const int nbox = ctl->nbox;
  const int k = ctl->k + 1;
  bool f = false;
  __shared__ int any_gate, any_brk;
  if (b == 0) {
    any_gate = 0;
    any_brk = 0;
  }
  __syncthreads();
  if (b < nbox && st[b].open) {
    BoxSt& s = st[b];
    if (s.brk) {
      // p.Ap <= 0 in iteration k (0 after an exact solve): stop with the k-1
      // completed updates, as the reference's breakdown exit does
      s.open = 0;
      s.iters = k - 1;
      atomicOr(&any_brk, 1);
    } else if (s.gate) {
      atomicOr(&any_gate, 1);
      s.normr = sqrt(s.rr_true);
      s.since = 0;
      s.upd += 1;
      if (s.normr <= s.tol_abs || (ctl->max_refine > 0 && s.upd >= ctl->max_refine)) {
        s.open = 0;
        s.iters = k;
      } else {
        s.beta = s.rr_true / s.rr;
        s.rr = s.rr_true;
        s.rr_upd = s.rr_true;
      }
      s.gate = 0;
    } else {
      s.beta = s.rr_new / s.rr;
      s.rr = s.rr_new;
    }
    if (s.open && k >= ctl->max_iter) {
      s.open = 0;
      s.iters = k;
    }
    f = s.open;
  }
  __syncthreads();
  bx_build_list(boxes, nbox, f, open);
  if (b == 0) {
    ctl->k = k;
    ctl->first = 0;
    if (any_gate) ctl->updates += 1;
    if (any_brk) ctl->status = MFE_BREAKDOWN;
    ctl->cont = *open.count > 0;
    if (in_graph) cudaGraphSetConditional(h, ctl->cont ? 1u : 0u);
  }
}

// FP64 solver, end of iteration k: the reference's loop test per box
// (iteration k+1 runs while k+1 <= max_iter and normr > tol, normr being
// |r| at the top of iteration k).
__global__ void __launch_bounds__(1024)
    k_bx_after64(const BoxDesc* boxes, BoxSt* st, BatchCtl* ctl, BxList open,
                 cudaGraphConditionalHandle h, int in_graph)
{
  const int b = threadIdx.x;
  const int nbox = ctl->nbox;
  const int k = ctl->k + 1;
  bool f = false;
  __shared__ int any_brk;
  if (b == 0) any_brk = 0;
  __syncthreads();
  if (b < nbox && st[b].open) {
    BoxSt& s = st[b];
    if (s.brk) {
      s.open = 0;
      s.iters = k - 1;
      atomicOr(&any_brk, 1);
    } else if (k + 1 <= ctl->max_iter && s.normr > s.tol_abs) {
      s.beta = s.rr_new / s.rr;
      s.rr = s.rr_new;
      s.normr = sqrt(s.rr_new);
    } else {
      s.open = 0;
      s.iters = k;
    }
    f = s.open;
  }
  __syncthreads();
  bx_build_list(boxes, nbox, f, open);
  if (b == 0) {
    ctl->k = k;
    ctl->first = 0;
    if (any_brk) ctl->status = MFE_BREAKDOWN;
    ctl->cont = *open.count > 0;
    if (in_graph) cudaGraphSetConditional(h, ctl->cont ? 1u : 0u);
  }
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------
}  // namespace mfe

// The batch handle: the assembled store of every box, owned device memory,
// and the launch shape the solves use.
struct mfe_batch {
  int device = 0;
  int nbox = 0;
  std::vector<int32_t> dims;
  std::vector<mfe::BoxDesc> hd;  // bases; tile and chunk counts filled per solve
  int64_t rows_tot = 0, nnz_tot = 0, ell_tot = 0, rows_real = 0, nnz_real = 0;
  double assembly_s = 0.0;
  mfe_batch_tuning tune{256, 2, 8192};
  bool ell_ready = false;
  int stencil_state = 0;   // 0: not checked, 1: every box verified, 2: not every box
  float* coef = nullptr;   // [nbox][28] when stencil_state == 1
  float* coef8 = nullptr;  // [nbox][28]: 8 mirror-class weights and dd (index 27) when
                           // every box's stencil is mirror-symmetric, else null
  // device memory
  mfe::BoxDesc* boxes = nullptr;
  mfe::BoxSt* st = nullptr;
  mfe::BatchCtl* ctl = nullptr;
  int* lists = nullptr;  // three lists (open, gate, all)
  double* slots = nullptr;
  size_t slots_bytes = 0;
  double* chunk_part = nullptr;
  size_t chunk_part_bytes = 0;
  double *vals64 = nullptr, *b = nullptr, *x = nullptr;
  float* ell32 = nullptr;
  void *r = nullptr, *p = nullptr, *Ap = nullptr;
  float* x32 = nullptr;
  size_t vec_bytes = 0;  // bytes of r, p, Ap as allocated
  std::vector<void*> owned;
};

namespace mfe {
namespace {

int64_t pad4(int64_t v) { return (v + kBxPad - 1) / kBxPad * kBxPad; }

// FP32 products read the padded 27-per-row values, FP64 ones the compressed CSR
template <int MODE, int R, int S>
cudaError_t bx_cfg32(int* per_sm)
{
  auto k = k_bx_spmv<float, MODE, true, R, S>;
  const size_t smem = bx_smem(sizeof(float), R, S);
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(per_sm, k, R + 32, smem);
  return e;
}

template <typename F>
auto bx_dispatch32(int rows, int stages, F&& f)
{
  if (rows == 128) {
    if (stages == 3) return f.template operator()<128, 3>();
    if (stages == 4) return f.template operator()<128, 4>();
    return f.template operator()<128, 2>();
  }
  if (stages == 3) return f.template operator()<256, 3>();
  if (stages == 4) return f.template operator()<256, 4>();
  return f.template operator()<256, 2>();
}

bool bx_shape_ok(const mfe_batch_tuning& t)
{
  return (t.spmv_rows == 128 || t.spmv_rows == 256) && t.spmv_stages >= 2 && t.spmv_stages <= 4 &&
         t.chunk_rows >= 1024 && t.chunk_rows <= (1 << 20) && t.chunk_rows % 4 == 0;
}

struct Grids {
  int g32, g64;
};

// grid sizes (resident CTAs) of the FP32 shape and the FP64 shape; the
// attributes are set here, before any graph capture
mfe_status bx_grids(mfe_ctx* ctx, const mfe_batch_tuning& t, Grids* g)
{
  int per32 = 1, pd = 1, pr = 1;
  cudaError_t e = bx_dispatch32(t.spmv_rows, t.spmv_stages,
                                [&]<int R, int S>() { return bx_cfg32<BX_DOT, R, S>(&per32); });
  const size_t smem64 = bx_smem(sizeof(double), kBx64Rows, kBx64Stages);
  auto kd = k_bx_spmv<double, BX_DOT, false, kBx64Rows, kBx64Stages>;
  auto kr = k_bx_spmv<double, BX_RESID, false, kBx64Rows, kBx64Stages>;
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem64);
  if (e == cudaSuccess) e = cudaFuncSetAttribute(kr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem64);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pd, kd, kBx64Rows + 32, smem64);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&pr, kr, kBx64Rows + 32, smem64);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched SpMV configuration");
  g->g32 = ctx->sm_count * std::max(per32, 1);
  g->g64 = ctx->sm_count * std::max(std::min(pd, pr), 1);
  return MFE_OK;
}

struct Run {
  mfe_batch* bt;
  BxList open, gate, all;
  Grids grid;
  bool mixed;
  bool stencil;  // FP32 products by k_bx_stencil (tpre32 then counts its steps)
  bool stencil2; // ... by k_bx_stencil2 (mirror-symmetric stencils, two rows per thread)
};

void* bx_alloc(mfe_batch* bt, size_t bytes);

// resident CTAs of the batched stencil SpMV (attribute set before any capture)
mfe_status bx_stencil_grid(mfe_ctx* ctx, bool pair, int* grid)
{
  const void* k = pair ? (const void*)k_bx_stencil2 : (const void*)k_bx_stencil;
  const size_t smem = pair ? kB2Smem : kStSmem;
  const int threads = pair ? kB2P / 2 + 32 : kSP + 32;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int per = 1;
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, threads, smem);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched stencil SpMV configuration");
  *grid = ctx->sm_count * std::max(per, 1);
  return MFE_OK;
}

// every box checked once per batch (its values never change after assembly)
mfe_status bx_stencil_prepare(mfe_ctx* ctx, mfe_batch* bt)
{
  if (bt->stencil_state != 0) return MFE_OK;
  std::vector<float> hc((size_t)bt->nbox * 28);
  bool all = true;
  for (int i = 0; i < bt->nbox && all; ++i) {
    const BoxDesc& d = bt->hd[i];
    bool ok = false;
    MFE_TRY(stencil_prepare_box(ctx, d.Nx, d.Ny, d.Nz, bt->vals64 + d.nnz_base, &hc[(size_t)i * 28], &ok));
    all = ok;
  }
  if (all) {
    bt->coef = static_cast<float*>(bx_alloc(bt, sizeof(float) * hc.size()));
    if (!bt->coef) return fail(ctx, MFE_OOM, "batch stencil allocation failed");
    MFE_CUDA_TRY(ctx, cudaMemcpy(bt->coef, hc.data(), sizeof(float) * hc.size(), cudaMemcpyHostToDevice));
    std::vector<float> h8(hc.size(), 0.0f);
    bool sym = true;
    for (int i = 0; i < bt->nbox && sym; ++i) {
      sym = stencil_mirror_classes(&hc[(size_t)i * 28], &h8[(size_t)i * 28]);
      h8[(size_t)i * 28 + 27] = hc[(size_t)i * 28 + 27];
    }
    if (sym) {
      bt->coef8 = static_cast<float*>(bx_alloc(bt, sizeof(float) * h8.size()));
      if (!bt->coef8) return fail(ctx, MFE_OOM, "batch stencil allocation failed");
      MFE_CUDA_TRY(ctx, cudaMemcpy(bt->coef8, h8.data(), sizeof(float) * h8.size(), cudaMemcpyHostToDevice));
    }
  }
  bt->stencil_state = all ? 1 : 2;
  return MFE_OK;
}

BxVecParams bx_vec(const Run& R, const BxList& L)
{
  return BxVecParams{R.bt->boxes, R.bt->st, R.bt->ctl, L.ids, L.cpre, L.count, R.bt->chunk_part,
                     R.bt->tune.chunk_rows};
}

template <typename T, int MODE>
BxSpmvParams<T> bx_params(const Run& R, const BxList& L, const T* vals, const T* x, T* y,
                          const double* b, float* y32)
{
  BxSpmvParams<T> P;
  P.boxes = R.bt->boxes;
  P.st = R.bt->st;
  P.ids = L.ids;
  P.tpre = sizeof(T) == 4 ? L.tpre32 : L.tpre64;
  P.count = L.count;
  P.vals = vals;
  P.x = x;
  P.y = y;
  P.b = b;
  P.y32 = y32;
  P.slots = R.bt->slots;
  P.err = &R.bt->ctl->err;
  return P;
}

mfe_status bx_spmv32(mfe_ctx* ctx, const Run& R, const BxList& L, const float* x, float* y)
{
  if (R.stencil) {
    BxStParams S;
    S.boxes = R.bt->boxes;
    S.st = R.bt->st;
    S.ids = L.ids;
    S.tpre = L.tpre32;
    S.count = L.count;
    S.coef = R.stencil2 ? R.bt->coef8 : R.bt->coef;
    S.x = x;
    S.y = y;
    S.slots = R.bt->slots;
    S.err = &R.bt->ctl->err;
    if (R.stencil2) {
      k_bx_stencil2<<<R.grid.g32, kB2P / 2 + 32, kB2Smem, ctx->stream>>>(S);
      return check_launch(ctx, "k_bx_stencil2");
    }
    k_bx_stencil<<<R.grid.g32, kSP + 32, kStSmem, ctx->stream>>>(S);
    return check_launch(ctx, "k_bx_stencil");
  }
  const BxSpmvParams<float> P = bx_params<float, BX_DOT>(R, L, R.bt->ell32, x, y, nullptr, nullptr);
  bx_dispatch32(R.bt->tune.spmv_rows, R.bt->tune.spmv_stages, [&]<int RW, int S>() {
    k_bx_spmv<float, BX_DOT, true, RW, S>
        <<<R.grid.g32, RW + 32, bx_smem(sizeof(float), RW, S), ctx->stream>>>(P);
    return 0;
  });
  return check_launch(ctx, "k_bx_spmv");
}

template <int MODE>
mfe_status bx_spmv64(mfe_ctx* ctx, const Run& R, const BxList& L, const double* x, double* y,
                     const double* b, float* y32)
{
  const BxSpmvParams<double> P = bx_params<double, MODE>(R, L, R.bt->vals64, x, y, b, y32);
  k_bx_spmv<double, MODE, false, kBx64Rows, kBx64Stages>
      <<<R.grid.g64, kBx64Rows + 32, bx_smem(sizeof(double), kBx64Rows, kBx64Stages), ctx->stream>>>(P);
  return check_launch(ctx, "k_bx_spmv");
}

// one wave of resident blocks of `kernel`
int bx_vgrid(mfe_ctx* ctx, const void* kernel) { return resident_blocks(ctx, kernel, kBxVT, 0); }

mfe_status bx_iter_mixed(mfe_ctx* ctx, const Run& R, cudaGraphConditionalHandle h, int in_graph)
{
  mfe_batch* bt = R.bt;
  float* r = static_cast<float*>(bt->r);
  float* p = static_cast<float*>(bt->p);
  float* Ap = static_cast<float*>(bt->Ap);
  k_bx_p<float><<<bx_vgrid(ctx, (const void*)k_bx_p<float>), kBxVT, 0, ctx->stream>>>(bx_vec(R, R.open), r, p,
                                                                                          bt->x32);
  MFE_TRY(check_launch(ctx, "k_bx_p"));
  MFE_TRY(bx_spmv32(ctx, R, R.open, p, Ap));
  k_bx_update<float><<<bx_vgrid(ctx, (const void*)k_bx_update<float>), kBxVT, 0, ctx->stream>>>(
      bx_vec(R, R.open), bt->x32, r, p, Ap);
  MFE_TRY(check_launch(ctx, "k_bx_update"));
  k_bx_decide<<<1, 1024, 0, ctx->stream>>>(bt->boxes, bt->st, bt->ctl, R.gate);
  MFE_TRY(check_launch(ctx, "k_bx_decide"));
  k_bx_xupdate<<<bx_vgrid(ctx, (const void*)k_bx_xupdate), kBxVT, 0, ctx->stream>>>(
      bx_vec(R, R.gate), bt->x, bt->x32, p);
  MFE_TRY(check_launch(ctx, "k_bx_xupdate"));
  MFE_TRY(bx_spmv64<BX_RESID>(ctx, R, R.gate, bt->x, nullptr, bt->b, r));
  k_bx_after<<<1, 1024, 0, ctx->stream>>>(bt->boxes, bt->st, bt->ctl, R.open, h, in_graph);
  return check_launch(ctx, "k_bx_after");
}

mfe_status bx_iter_f64(mfe_ctx* ctx, const Run& R, cudaGraphConditionalHandle h, int in_graph)
{
  mfe_batch* bt = R.bt;
  double* r = static_cast<double*>(bt->r);
  double* p = static_cast<double*>(bt->p);
  double* Ap = static_cast<double*>(bt->Ap);
  k_bx_p<double><<<bx_vgrid(ctx, (const void*)k_bx_p<double>), kBxVT, 0, ctx->stream>>>(bx_vec(R, R.open), r, p,
                                                                                            nullptr);
  MFE_TRY(check_launch(ctx, "k_bx_p"));
  MFE_TRY(bx_spmv64<BX_DOT>(ctx, R, R.open, p, Ap, nullptr, nullptr));
  k_bx_update<double><<<bx_vgrid(ctx, (const void*)k_bx_update<double>), kBxVT, 0, ctx->stream>>>(
      bx_vec(R, R.open), bt->x, r, p, Ap);
  MFE_TRY(check_launch(ctx, "k_bx_update"));
  k_bx_after64<<<1, 1024, 0, ctx->stream>>>(bt->boxes, bt->st, bt->ctl, R.open, h, in_graph);
  return check_launch(ctx, "k_bx_after64");
}

void* bx_alloc(mfe_batch* bt, size_t bytes)
{
  void* ptr = nullptr;
  if (cudaMalloc(&ptr, bytes) != cudaSuccess) return nullptr;
  bt->owned.push_back(ptr);
  return ptr;
}

BxList bx_list(int* base, int nbox, int which)
{
  const size_t per = (size_t)nbox + 2, stride = 4 * per + 4;
  int* a = base + which * stride;
  return BxList{a, a + per, a + 2 * per, a + 3 * per, a + 4 * per};
}

// Runs `body` as a CUDA graph with a conditional while node on ctl->cont (or,
// with MFE_CG_EAGER set, as a host loop reading cont back each iteration).
template <typename Body>
mfe_status bx_loop(mfe_ctx* ctx, BatchCtl* dctl, Body body)
{
  if (getenv("MFE_CG_EAGER") != nullptr) {
    BatchCtl* hctl = static_cast<BatchCtl*>(host_scratch(ctx, sizeof(BatchCtl)));
    if (!hctl) return fail(ctx, MFE_OOM, "pinned scratch allocation failed");
    for (;;) {
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hctl, dctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, ctx->stream));
      MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      if (!hctl->cont) return MFE_OK;
      MFE_TRY(body((cudaGraphConditionalHandle)0, 0));
    }
  }
  cudaStream_t run_stream = ctx->stream, s = ctx->own_stream;
  cudaGraph_t g = nullptr;
  cudaGraphExec_t ex = nullptr;
  cudaGraphConditionalHandle h = 0;
  mfe_status st = MFE_OK;
  cudaError_t e = cudaGraphCreate(&g, 0);
  if (e == cudaSuccess) e = cudaGraphConditionalHandleCreate(&h, g, 0, cudaGraphCondAssignDefault);
  if (e == cudaSuccess) {
    ctx->stream = s;
    e = cudaStreamBeginCaptureToGraph(s, g, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    if (e == cudaSuccess) {
      k_bx_begin<<<1, 1, 0, s>>>(dctl, h);
      e = cudaStreamEndCapture(s, &g);
    }
    cudaGraphNode_t nodes[4];
    size_t nn = 4;
    if (e == cudaSuccess) e = cudaGraphGetNodes(g, nodes, &nn);
    alignas(cudaGraphNodeParams) unsigned char cp_buf[sizeof(cudaGraphNodeParams)];
    memset(cp_buf, 0, sizeof(cp_buf));
    cudaGraphNodeParams* cp = reinterpret_cast<cudaGraphNodeParams*>(cp_buf);
    cp->type = cudaGraphNodeTypeConditional;
    cp->conditional.handle = h;
    cp->conditional.type = cudaGraphCondTypeWhile;
    cp->conditional.size = 1;
    cudaGraphNode_t cnode;
    if (e == cudaSuccess) e = cudaGraphAddNode(&cnode, g, &nodes[0], nullptr, 1, cp);
    if (e == cudaSuccess) {
      cudaGraph_t bg = cp->conditional.phGraph_out[0];
      e = cudaStreamBeginCaptureToGraph(s, bg, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
      if (e == cudaSuccess) {
        st = body(h, 1);
        cudaGraph_t tmp;
        const cudaError_t e2 = cudaStreamEndCapture(s, &tmp);
        if (e == cudaSuccess) e = e2;
      }
    }
    ctx->stream = run_stream;
    if (e == cudaSuccess && st == MFE_OK) e = cudaGraphInstantiate(&ex, g, 0);
    if (e == cudaSuccess && st == MFE_OK) e = cudaGraphLaunch(ex, ctx->stream);
  }
  if (ex) cudaGraphExecDestroy(ex);
  if (g) cudaGraphDestroy(g);
  if (st != MFE_OK) return st;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "batched CG graph");
  return MFE_OK;
}

}  // namespace

mfe_status batch_create(mfe_ctx* ctx, int nbox, const int32_t* dims, mfe_batch** out)
{
  *out = nullptr;
  if (nbox < 1 || nbox > kBxMaxBoxes) return fail(ctx, MFE_BAD_ARG, "nbox must be 1..1024");
  mfe_batch* bt = new mfe_batch();
  bt->device = ctx->device;
  bt->nbox = nbox;
  bt->dims.assign(dims, dims + 3 * nbox);
  bt->hd.resize(nbox);
  int64_t max_nnz = 0, max_rows = 0;
  for (int i = 0; i < nbox; ++i) {
    const int nx = dims[3 * i], ny = dims[3 * i + 1], nz = dims[3 * i + 2];
    int64_t n = 0, nnz = 0;
    if (mfe_box_dims(nx, ny, nz, &n, &nnz) != MFE_OK || nnz > INT32_MAX - 64 || 27 * n > INT32_MAX - 64) {
      delete bt;
      return fail(ctx, MFE_BAD_ARG, "bad box dimensions in the batch");
    }
    BoxDesc& d = bt->hd[i];
    memset(&d, 0, sizeof(d));
    d.Nx = nx + 1;
    d.Ny = ny + 1;
    d.Nz = nz + 1;
    d.NxNy = d.Nx * d.Ny;
    d.n = (int)n;
    // ghost zone: rows a tile's x segments reach outside the box, rounded to
    // the copy granule
    const int64_t ghost = pad4((int64_t)d.NxNy + d.Nx + 1 + kBxPad);
    d.row_base = bt->rows_tot + ghost;
    d.nnz_base = bt->nnz_tot;
    d.ell_base = bt->ell_tot;
    bt->rows_tot += ghost + pad4(n) + ghost;
    bt->nnz_tot += pad4(nnz);
    bt->ell_tot += pad4(27 * n);
    bt->rows_real += n;
    bt->nnz_real += nnz;
    max_nnz = std::max(max_nnz, nnz);
    max_rows = std::max(max_rows, n);
  }
  const size_t rows8 = (size_t)(bt->rows_tot + 8);
  bt->boxes = static_cast<BoxDesc*>(bx_alloc(bt, sizeof(BoxDesc) * nbox));
  bt->st = static_cast<BoxSt*>(bx_alloc(bt, sizeof(BoxSt) * nbox));
  bt->ctl = static_cast<BatchCtl*>(bx_alloc(bt, sizeof(BatchCtl)));
  bt->lists = static_cast<int*>(bx_alloc(bt, sizeof(int) * 3 * (4 * ((size_t)nbox + 2) + 4)));
  bt->vals64 = static_cast<double*>(bx_alloc(bt, sizeof(double) * (size_t)(bt->nnz_tot + 8)));
  bt->b = static_cast<double*>(bx_alloc(bt, sizeof(double) * rows8));
  bt->x = static_cast<double*>(bx_alloc(bt, sizeof(double) * rows8));
  int32_t* ro = static_cast<int32_t*>(workspace(ctx, "batch.ro", sizeof(int32_t) * (size_t)(max_rows + 1)));
  int32_t* cols = static_cast<int32_t*>(workspace(ctx, "batch.cols", sizeof(int32_t) * (size_t)(max_nnz + 4)));
  if (!bt->boxes || !bt->st || !bt->ctl || !bt->lists || !bt->vals64 || !bt->b || !bt->x || !ro || !cols) {
    batch_destroy(bt);
    return fail(ctx, MFE_OOM, "batch allocation failed");
  }
  mfe_status st = MFE_OK;
  auto cu = [&](cudaError_t e, const char* w) {
    if (st == MFE_OK && e != cudaSuccess) st = cuda_fail(ctx, e, w);
  };
  cu(cudaEventRecord(ctx->ev0, ctx->stream), "event");
  cu(cudaMemsetAsync(bt->vals64, 0, sizeof(double) * (size_t)(bt->nnz_tot + 8), ctx->stream), "memset");
  cu(cudaMemsetAsync(bt->b, 0, sizeof(double) * rows8, ctx->stream), "memset");
  for (int i = 0; i < nbox && st == MFE_OK; ++i) {
    const int nx = dims[3 * i], ny = dims[3 * i + 1], nz = dims[3 * i + 2];
    st = launch_structure(ctx, nx, ny, nz, ro, cols);
    if (st == MFE_OK)
      st = launch_assemble(ctx, nx, ny, nz, nullptr, ro, bt->vals64 + bt->hd[i].nnz_base,
                           bt->b + bt->hd[i].row_base, 1);
  }
  cu(cudaEventRecord(ctx->ev1, ctx->stream), "event");
  cu(cudaEventSynchronize(ctx->ev1), "assembly");
  if (st != MFE_OK) {
    batch_destroy(bt);
    return st;
  }
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  bt->assembly_s = ms * 1e-3;
  *out = bt;
  return MFE_OK;
}

void batch_destroy(mfe_batch* bt)
{
  if (!bt) return;
  int prev = -1;
  cudaGetDevice(&prev);
  cudaSetDevice(bt->device);
  for (void* p : bt->owned) cudaFree(p);
  if (prev >= 0) cudaSetDevice(prev);
  delete bt;
}

void batch_info(const mfe_batch* bt, int64_t* rows, int64_t* nnz, double* assembly_s,
                mfe_batch_tuning* tuning)
{
  if (rows) *rows = bt->rows_real;
  if (nnz) *nnz = bt->nnz_real;
  if (assembly_s) *assembly_s = bt->assembly_s;
  if (tuning) *tuning = bt->tune;
}

mfe_status batch_set_tuning(mfe_ctx* ctx, mfe_batch* bt, const mfe_batch_tuning* t)
{
  if (!bx_shape_ok(*t)) return fail(ctx, MFE_BAD_ARG, "spmv_rows 128|256, spmv_stages 2..4, chunk_rows 1024..2^20 (multiple of 4)");
  bt->tune = *t;
  return MFE_OK;
}

mfe_status batch_solve(mfe_ctx* ctx, mfe_batch* bt, const mfe_cg_opts* o, double* x_out,
                       mfe_cg_result* results)
{
  if (o->precision != MFE_PREC_MIXED && o->precision != MFE_PREC_F64)
    return fail(ctx, MFE_BAD_ARG, "unknown precision");
  if (bt->device != ctx->device) return fail(ctx, MFE_BAD_ARG, "batch belongs to another device");
  if (o->precision == MFE_PREC_MIXED && !mixed_opts_valid(o)) return fail(ctx, MFE_BAD_ARG, "inner_tol must lie in [0, 1) and max_refine must be >= 0");
  const int nbox = bt->nbox;
  Run R;
  R.bt = bt;
  R.mixed = o->precision == MFE_PREC_MIXED;
  if (R.mixed && o->mixed_operator == 0) MFE_TRY(bx_stencil_prepare(ctx, bt));
  R.stencil = R.mixed && o->mixed_operator == 0 && bt->stencil_state == 1;
  R.stencil2 = R.stencil && bt->coef8 != nullptr;
  R.open = bx_list(bt->lists, nbox, 0);
  R.gate = bx_list(bt->lists, nbox, 1);
  R.all = bx_list(bt->lists, nbox, 2);
  MFE_TRY(bx_grids(ctx, bt->tune, &R.grid));
  if (R.stencil) MFE_TRY(bx_stencil_grid(ctx, R.stencil2, &R.grid.g32));
  const size_t rows8 = (size_t)(bt->rows_tot + 8);

  // tiles (stencil steps) and chunks of each box at this launch shape
  int chunks_tot = 0;
  for (auto& d : bt->hd) {
    d.ntiles32 = R.stencil ? (int)(ceil_div(d.NxNy, (int64_t)(R.stencil2 ? kB2P : kSP)) * d.Nz)
                           : (int)ceil_div(d.n, bt->tune.spmv_rows);
    d.ntiles64 = (int)ceil_div(d.n, kBx64Rows);
    d.nchunks = (int)ceil_div(d.n, bt->tune.chunk_rows);
    d.chunk_base = chunks_tot;
    chunks_tot += d.nchunks;
  }
  // buffers that depend on the precision or the shape (grown, never shrunk)
  const size_t vb = (R.mixed ? sizeof(float) : sizeof(double)) * rows8;
  if (bt->vec_bytes < vb) {
    bt->r = bx_alloc(bt, vb);
    bt->p = bx_alloc(bt, vb);
    bt->Ap = bx_alloc(bt, vb);
    if (!bt->r || !bt->p || !bt->Ap) return fail(ctx, MFE_OOM, "batch vector allocation failed");
    bt->vec_bytes = vb;
  }
  if (R.mixed && !bt->x32) {
    bt->x32 = static_cast<float*>(bx_alloc(bt, sizeof(float) * rows8));
    if (!bt->x32) return fail(ctx, MFE_OOM, "batch FP32 allocation failed");
  }
  if (R.mixed && !R.stencil && !bt->ell32) {
    bt->ell32 = static_cast<float*>(bx_alloc(bt, sizeof(float) * (size_t)(bt->ell_tot + 8)));
    if (!bt->ell32) return fail(ctx, MFE_OOM, "batch FP32 allocation failed");
  }
  const size_t slots_b = sizeof(double) * (size_t)nbox * std::max(R.grid.g32, R.grid.g64) * 8;
  if (bt->slots_bytes < slots_b) {
    bt->slots = static_cast<double*>(bx_alloc(bt, slots_b));
    if (!bt->slots) return fail(ctx, MFE_OOM, "batch slot allocation failed");
    bt->slots_bytes = slots_b;
  }
  const size_t cp_b = sizeof(double) * (size_t)(chunks_tot + 1);
  if (bt->chunk_part_bytes < cp_b) {
    bt->chunk_part = static_cast<double*>(bx_alloc(bt, cp_b));
    if (!bt->chunk_part) return fail(ctx, MFE_OOM, "batch chunk allocation failed");
    bt->chunk_part_bytes = cp_b;
  }
  if (R.mixed && !R.stencil && !bt->ell_ready) {
    for (int i = 0; i < nbox; ++i) {
      k_bx_ell<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(bt->hd[i].n, 256),
                                                                  (int64_t)ctx->sm_count * 8)),
                 256, 0, ctx->stream>>>(bt->hd[i], bt->vals64, bt->ell32);
      MFE_TRY(check_launch(ctx, "k_bx_ell"));
    }
    bt->ell_ready = true;
  }

  // state: x = 0, ghosts and work vectors zero, per-box tolerances
  std::vector<BoxSt> hs(nbox);
  for (int i = 0; i < nbox; ++i) {
    memset(&hs[i], 0, sizeof(BoxSt));
    hs[i].tol_abs = o->tol;
  }
  BatchCtl hc{};
  hc.nbox = nbox;
  hc.max_iter = std::max(0, o->max_iter);
  hc.refine_k = o->refine_k > 0 ? o->refine_k : 50;
  hc.first = 1;
  hc.tol_mode = o->tol_mode == MFE_TOL_RELATIVE ? 1 : 0;
  hc.delta2 = mixed_delta2(o);
  hc.max_refine = o->max_refine;
  std::vector<int> hl(4 * ((size_t)nbox + 2) + 4, 0);
  {
    const size_t per = (size_t)nbox + 2;
    int t32 = 0, t64 = 0, ch = 0;
    for (int i = 0; i < nbox; ++i) {
      hl[i] = i;
      hl[per + i] = t32;
      hl[2 * per + i] = t64;
      hl[3 * per + i] = ch;
      t32 += bt->hd[i].ntiles32;
      t64 += bt->hd[i].ntiles64;
      ch += bt->hd[i].nchunks;
    }
    hl[per + nbox] = t32;
    hl[2 * per + nbox] = t64;
    hl[3 * per + nbox] = ch;
    hl[4 * per] = nbox;
  }
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(bt->boxes, bt->hd.data(), sizeof(BoxDesc) * nbox, cudaMemcpyHostToDevice, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(bt->st, hs.data(), sizeof(BoxSt) * nbox, cudaMemcpyHostToDevice, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(bt->ctl, &hc, sizeof(BatchCtl), cudaMemcpyHostToDevice, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(R.all.ids, hl.data(), sizeof(int) * hl.size(), cudaMemcpyHostToDevice, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(bt->x, 0, sizeof(double) * rows8, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(bt->r, 0, vb, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(bt->p, 0, vb, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(bt->Ap, 0, vb, ctx->stream));
  if (R.mixed) MFE_CUDA_TRY(ctx, cudaMemsetAsync(bt->x32, 0, sizeof(float) * rows8, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));

  // r = b - A x0 over all boxes, then the open list
  if (R.mixed)
    MFE_TRY(bx_spmv64<BX_RESID>(ctx, R, R.all, bt->x, nullptr, bt->b, static_cast<float*>(bt->r)));
  else
    MFE_TRY(bx_spmv64<BX_RESID>(ctx, R, R.all, bt->x, static_cast<double*>(bt->r), bt->b, nullptr));
  k_bx_init<<<1, 1024, 0, ctx->stream>>>(bt->boxes, bt->st, bt->ctl, R.open);
  MFE_TRY(check_launch(ctx, "k_bx_init"));
  // occupancy queries before the loop is captured
  for (const void* k : {(const void*)k_bx_p<float>, (const void*)k_bx_update<float>,
                        (const void*)k_bx_xupdate, (const void*)k_bx_p<double>,
                        (const void*)k_bx_update<double>})
    bx_vgrid(ctx, k);
  MFE_TRY(bx_loop(ctx, bt->ctl, [&](cudaGraphConditionalHandle h, int in_graph) -> mfe_status {
    return R.mixed ? bx_iter_mixed(ctx, R, h, in_graph) : bx_iter_f64(ctx, R, h, in_graph);
  }));
  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, ctx->stream));

  // results
  if (x_out) {
    int64_t out = 0;
    for (int i = 0; i < nbox; ++i) {
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(x_out + out, bt->x + bt->hd[i].row_base,
                                        sizeof(double) * bt->hd[i].n, cudaMemcpyDeviceToDevice, ctx->stream));
      out += bt->hd[i].n;
    }
  }
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs.data(), bt->st, sizeof(BoxSt) * nbox, cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(&hc, bt->ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  if (hc.err) return fail(ctx, MFE_TIMEOUT, "a bounded device wait gave up during the batched solve");
  mfe_status worst = MFE_OK;
  for (int i = 0; i < nbox; ++i) {
    const BoxSt& s = hs[i];
    mfe_cg_result& r = results[i];
    memset(&r, 0, sizeof(r));
    r.num_iters = s.open ? hc.k : s.iters;
    r.normr = s.normr;
    r.normr0 = s.normr0;
    r.final_resid = s.normr;
    r.times[0] = bt->assembly_s;  // assembly of the whole batch
    r.times[4] = ms * 1e-3;       // the batched solve
    r.refinements = hc.updates;
    r.inner_operator = !R.mixed ? MFE_INNER_NONE : (R.stencil ? MFE_INNER_STENCIL : MFE_INNER_PADDED);
    r.status = s.brk ? MFE_BREAKDOWN : (s.normr <= s.tol_abs ? MFE_OK : MFE_MAXITER);
    if (r.status != MFE_OK && worst == MFE_OK) worst = (mfe_status)r.status;
  }
  return worst;
}

mfe_status batch_solve_boxes(mfe_ctx* ctx, int nbox, const int32_t* dims, const mfe_cg_opts* o,
                             double* x_out, mfe_cg_result* results)
{
  mfe_batch* bt = nullptr;
  MFE_TRY(batch_create(ctx, nbox, dims, &bt));
  const mfe_status st = batch_solve(ctx, bt, o, x_out, results);
  batch_destroy(bt);
  return st;
}

}  // namespace mfe
