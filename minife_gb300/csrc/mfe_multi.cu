// Multi-right-hand-side CG on one box matrix: nrhs independent CG solves
// advanced together so every iteration reads the matrix once.
//
// Layout: X, B, and every work vector are row-major n x nrhs (X[i*nrhs + j]),
// so the rows a tile of the 27-point stencil touches are contiguous blocks of
// nrhs values.  k_spmm_box stages a tile's values and its nine x-row
// segments (all right-hand sides) into shared memory with bulk async copies
// (producer warp, full/empty mbarriers, as k_spmv_box) and runs one warp per
// row and one lane per right-hand side: the row's 27 values are broadcast to
// the warp, and lane j reads x[col*nrhs + j], so shared-memory reads are
// conflict-free.  Each lane accumulates its right-hand side's dot in FP64.
//
// The mixed solver is the one of mfe_mixed.cu applied per right-hand side:
// FP32 matrix copy, FP32 vectors, FP64 dots and scalars (alpha_j, beta_j),
// FP64 solution; reliable updates (x += x32, R = B - A X in FP64) happen for
// all right-hand sides together (see k_mr_decide).  The FP64 solver runs the
// reference's CG per right-hand side.  A finished right-hand side is frozen
// (alpha_j = 0).
// nrhs must divide 32 (1, 2, 4, 8, 16, 32).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <utility>

#include "mfe_box.cuh"
#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

constexpr int kMaxRhs = 32;
constexpr int kTileRowsM = 32;  // rows per tile (two per consumer warp)
constexpr int kConsM = 16;      // consumer warps per CTA
constexpr int kProdM = 2;       // producer warps per CTA (tiles alternate between them)
constexpr int kThreadsM = (kConsM + kProdM) * 32;
constexpr int kVT = 256;
constexpr int kMaxPartM = 2048;

// stage capacities (elements): a tile's values, and one x segment of
// kTileRowsM + 2 rows of nrhs values, each with room for rounding both ends
// to the 16-byte bulk-copy granule
__host__ __device__ constexpr int spmm_capv() { return ((kTileRowsM * 27 + 8) + 3) & ~3; }
__host__ __device__ constexpr int spmm_capx(int nrhs)
{
  return (((kTileRowsM + 2) * nrhs + 8) + 3) & ~3;
}
// pipeline depth (one stage per producer warp): a FP32 stage of 32
// right-hand sides is 42.6 KB, a FP64 one 85 KB
template <typename T>
__host__ __device__ constexpr int spmm_stages()
{
  return 2;
}

template <typename T>
struct Vec2;
template <>
struct Vec2<float> {
  using type = float2;
};
template <>
struct Vec2<double> {
  using type = double2;
};

struct MultiState {
  double rr[kMaxRhs], rr_new[kMaxRhs], pAp[kMaxRhs], beta[kMaxRhs];
  double alpha[kMaxRhs];  // rr / pAp (0 once finished), set with pAp
  double rr_true[kMaxRhs], rr_at_update[kMaxRhs], normr0[kMaxRhs], tol_abs[kMaxRhs];
  double normr_true[kMaxRhs];
  int done[kMaxRhs];
  int iters[kMaxRhs];  // iterations until each right-hand side converged
  int brk[kMaxRhs];    // p.Ap <= 0 met (the right-hand side stops alone)
  int nrhs, k, max_iter, since, refine_k, gate, cont, first, updates, status, tol_mode;
  int max_refine;  // mixed: stop after this many shared updates (0: no cap)
  unsigned err;
  int x_pending;  // mixed: x32 += alpha p of the last update not yet done
  double delta2;
};

enum MMode { MM_PLAIN = 0, MM_DOT = 1, MM_RESID = 2 };

template <typename T, typename RT>
struct SpmmParams {
  int n, Nx, Ny, Nz, NxNy, nrhs;
  int64_t nnz;
  const T* __restrict__ vals;
  const T* __restrict__ x;  // n x nrhs
  T* __restrict__ y;        // n x nrhs (DOT)
  const double* __restrict__ b;  // n x nrhs (RESID)
  RT* __restrict__ yres;         // RESID output: b - A x rounded to RT
  int capv, capx;                // stage capacities (elements)
  double* partials;              // [grid][32]
  unsigned* ticket;
  double* out;                   // [32] totals
  const int* gate;               // nullable
  unsigned* err;
  MultiState* cg;                // DOT mode in a solve: also set cg->alpha from out
};

// Per-lane dots of the block summed over its warps, then over blocks in
// block order by the last block: out[j] = total of lane j.  red: >= 33*32.
// With cg set (out = cg->pAp) the last block also forms cg->alpha.
__device__ void multi_dot_reduce(double v, double* red, double* partials, unsigned* ticket,
                                 double* out, int nlanes, MultiState* cg = nullptr)
{
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nw = blockDim.x >> 5;
  red[warp * 32 + lane] = v;
  __syncthreads();
  __shared__ bool am_last;
  if (threadIdx.x < 32) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w * 32 + threadIdx.x];
    partials[(size_t)blockIdx.x * 32 + threadIdx.x] = s;
  }
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) am_last = (atomicAdd(ticket, 1u) == gridDim.x - 1);
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  // every warp of the last block sums the partials of blocks warp,
  // warp + nw, ... (four accumulators keep four L2 loads in flight), then
  // the warps' sums are added in warp order: a fixed order for a fixed grid
  {
    const unsigned g = gridDim.x, uw = (unsigned)warp, unw = (unsigned)nw;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    unsigned bl = uw;
    for (; bl + 3 * unw < g; bl += 4 * unw) {
      s0 += __ldcg(&partials[(size_t)bl * 32 + lane]);
      s1 += __ldcg(&partials[(size_t)(bl + unw) * 32 + lane]);
      s2 += __ldcg(&partials[(size_t)(bl + 2 * unw) * 32 + lane]);
      s3 += __ldcg(&partials[(size_t)(bl + 3 * unw) * 32 + lane]);
    }
    for (; bl < g; bl += unw) s0 += __ldcg(&partials[(size_t)bl * 32 + lane]);
    red[warp * 32 + lane] = (s0 + s1) + (s2 + s3);
  }
  __syncthreads();
  if (threadIdx.x < nlanes) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += red[w * 32 + threadIdx.x];
    out[threadIdx.x] = s;
    if (cg)
      cg->alpha[threadIdx.x] = cg->done[threadIdx.x] || !(s > 0.0) ? 0.0 : cg->rr[threadIdx.x] / s;
  }
  if (threadIdx.x == 0) *ticket = 0u;
}

// NRC: nrhs as a compile-time constant (32), or 0 to read it from P
template <typename T, int MODE, typename RT, int NRC>
__global__ void __launch_bounds__(kThreadsM, NRC ? 2 : 1) k_spmm_box(SpmmParams<T, RT> P)
{
  constexpr int R = kTileRowsM, S = spmm_stages<T>();
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t full[S], empty[S];
  __shared__ uint32_t s_vbase[S];  // first staged value (low 32 bits of its index)
  __shared__ int64_t s_xbase[S][9];
  __shared__ int s_ok[S];    // stage holds the tile (capacities sufficed)
  __shared__ int s_fast[S];  // every x segment starts at its unclamped row
  // per row of the staged tile: low 32 bits of its CSR offset, and which of
  // its -x,+x,-y,+y,-z,+z neighbours exist (bits 0-5)
  __shared__ uint32_t s_rro[S][R];
  __shared__ int s_rflags[S][R];
  __shared__ double red[(kConsM + kProdM) * 32];
  static_assert(S % kProdM == 0, "each producer warp owns whole stages");
  constexpr int VA = 16 / sizeof(T);
  const int nr = NRC ? NRC : P.nrhs;
  const int capx = NRC ? spmm_capx(NRC) : P.capx;
  constexpr int capv = spmm_capv();
  const int stage_elems = capv + 9 * capx;
  T* const st0 = reinterpret_cast<T*>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = (P.n + R - 1) / R;
  if (P.gate != nullptr && *P.gate == 0) return;
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kConsM);
    }
    fence_mbar_init();
  }
  __syncthreads();
  double dacc = 0.0;  // FP64 products (RESID; DOT of FP64 operands)
  DFAcc facc;         // FP32 products (DOT of FP32 operands)
  if (warp < kProdM) {
    // producer warps: warp p stages the CTA's tiles it = p, p + kProdM, ...
    // (stages s = it % S).  Lane l follows row r0 + l of each tile (CSR
    // offset and neighbour flags, coordinates advanced incrementally: no
    // division per tile); lanes 0-8 also compute the nine x segments (lane
    // j: rows r0 + off_j - 1 .. r1 + off_j of offset j = (dz, dy)) and lane
    // 9 the values range; every lane announces and issues its own copy, lane
    // 0 arrives.
    const int p = warp;
    bool ok = true;
    const int64_t ntot = (int64_t)P.n * nr;
    static_assert(R == 32, "one producer lane per tile row");
    const int rl = lane;
    int ix = 0, iy = 0, iz = 0, sxs = 0, sys = 0, szs = 0;
    {
      const int64_t stride = (int64_t)kProdM * gridDim.x * R;
      szs = (int)(stride / P.NxNy);
      const int rs = (int)(stride - (int64_t)szs * P.NxNy);
      sys = rs / P.Nx;
      sxs = rs - sys * P.Nx;
      const int64_t rfirst = ((int64_t)blockIdx.x + (int64_t)p * gridDim.x) * R + rl;
      iz = (int)(rfirst / P.NxNy);
      const int rem = (int)(rfirst - (int64_t)iz * P.NxNy);
      iy = rem / P.Nx;
      ix = rem - iy * P.Nx;
    }
    int it = p;
    for (int tile = blockIdx.x + p * gridDim.x; tile < ntiles; tile += kProdM * gridDim.x, it += kProdM) {
      const int s = it % S;
      if (it >= S) {
        if (lane == 0) ok = mbar_wait_bounded(&empty[s], (unsigned)(((it / S) - 1) & 1));
        ok = __shfl_sync(0xffffffffu, ok, 0);
      }
      if (!ok) break;
      T* sv = st0 + (size_t)s * stage_elems;
      const int r0 = tile * R, r1 = min(P.n, r0 + R);
      const int64_t ro = row_offset(ix, iy, iz, P.Nx, P.Ny, P.Nz);
      const int cnt = nbr(ix, P.Nx) * nbr(iy, P.Ny) * nbr(iz, P.Nz);
      const int flags = (ix > 0) | (ix < P.Nx - 1) << 1 | (iy > 0) << 2 | (iy < P.Ny - 1) << 3 |
                        (iz > 0) << 4 | (iz < P.Nz - 1) << 5;
      const int64_t a = __shfl_sync(0xffffffffu, ro, 0);
      const int64_t e = __shfl_sync(0xffffffffu, ro + cnt, r1 - r0 - 1);
      // this lane's piece: elements [lo_e, bl_e) by bulk copy, [bl_e, hi_e)
      // (the unaligned end of the array) by plain loads
      int64_t lo_e = 0, bl_e = 0, hi_e = 0;
      const T* src = P.x;
      T* dst = sv;
      bool fits = true, fast = true;
      if (lane < 9) {
        const int off = (lane / 3 - 1) * P.NxNy + (lane % 3 - 1) * P.Nx;
        const int lo = min(max(r0 + off - 1, 0), P.n);
        int hi = min(r1 + off + 1, P.n);
        if (hi < lo) hi = lo;
        const int64_t elo = (int64_t)lo * nr;
        hi_e = (int64_t)hi * nr;
        lo_e = elo & ~(int64_t)(VA - 1);
        bl_e = min((hi_e + VA - 1) & ~(int64_t)(VA - 1), ntot & ~(int64_t)(VA - 1));
        if (bl_e < lo_e) bl_e = lo_e;
        fits = max(bl_e, hi_e) - lo_e <= capx;
        fast = lo == r0 + off - 1 && lo_e == elo;
        dst = sv + capv + lane * capx;
      } else if (lane == 9) {
        hi_e = e;
        lo_e = a & ~(int64_t)(VA - 1);
        bl_e = min((hi_e + VA - 1) & ~(int64_t)(VA - 1), P.nnz & ~(int64_t)(VA - 1));
        if (bl_e < lo_e) bl_e = lo_e;
        fits = max(bl_e, hi_e) - lo_e <= capv;
        src = P.vals;
      }
      fits = __all_sync(0xffffffffu, fits);
      fast = __all_sync(0xffffffffu, fast);
      {
        s_rro[s][rl] = (uint32_t)ro;
        s_rflags[s][rl] = r0 + rl < r1 ? flags : 0;
        ix += sxs;
        const int cx = ix >= P.Nx;
        ix -= cx ? P.Nx : 0;
        iy += sys + cx;
        const int cy = iy >= P.Ny;
        iy -= cy ? P.Ny : 0;
        iz += szs + cy;
      }
      if (!fits) {
        // cannot happen for the stage capacities the host computes
        if (lane == 0) {
          atomicOr(P.err, ERR_TILE_OVERFLOW);
          s_ok[s] = 0;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&full[s]);
        continue;
      }
      if (lane < 9) s_xbase[s][lane] = lo_e;
      if (lane == 9) s_vbase[s] = (uint32_t)lo_e;
      if (lane == 0) {
        s_ok[s] = 1;
        s_fast[s] = fast;
      }
      if (hi_e > bl_e) {
        for (int64_t k = bl_e; k < hi_e; ++k) dst[k - lo_e] = src[k];
        fence_proxy_async_smem();
      }
      const unsigned bytes = (unsigned)((bl_e - lo_e) * sizeof(T));
      if (bytes) {
        mbar_expect_tx(&full[s], bytes);
        bulk_g2s(dst, src + lo_e, bytes, &full[s]);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&full[s]);
    }
    if (!ok && lane == 0) {
      // wait (bounded) for the copies this warp issued: its tiles before
      // `it`, stage st (st = p mod kProdM) holding ceil((it - st) / S) of them
      atomicOr(P.err, ERR_WAIT_TIMEOUT);
      for (int st = p; st < S && st < it; st += kProdM)
        mbar_wait_bounded(&full[st], (unsigned)(((it - st + S - 1) / S - 1) & 1));
    }
  } else if constexpr (NRC == 32) {
    // consumer warp w: rows 2w (lanes 0-15) and 2w + 1 (lanes 16-31) of each
    // tile, lane h of a half holding right-hand sides 2h and 2h + 1 (paired
    // loads and stores; the row's values are broadcast to its half)
    using V2 = typename Vec2<T>::type;
    const int w = warp - kProdM, half = lane >> 4, h = lane & 15;
    const int lrow = 2 * w + half;
    double d0 = 0.0, d1 = 0.0;
    DFAcc f0, f1;
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      const int s = it % S;
      const int r = tile * R + lrow;
      if (!mbar_wait_bounded(&full[s], (unsigned)((it / S) & 1))) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        break;
      }
      const int flags = s_rflags[s][lrow];
      const bool ok = r < P.n && s_ok[s] != 0;
      const T* sv = st0 + (size_t)s * stage_elems;
      const T* sx = sv + capv;
      const T* rowv = sv + (s_rro[s][lrow] - s_vbase[s]);
      V2 sum{T(0), T(0)}, xr{T(0), T(0)};
      if (__all_sync(0xffffffffu, ok && flags == 63) && s_fast[s]) {
        // every segment of this stage starts at row r0 + off_j - 1, so the
        // row's x values sit at the same place in all nine: fixed offsets
        const T* xb = sx + (lrow + 1) * 32 + 2 * h;
        xr = *reinterpret_cast<const V2*>(xb + 4 * capx);
        V2 a0{T(0), T(0)}, a1{T(0), T(0)};
#pragma unroll
        for (int j = 0; j < 9; ++j) {
#pragma unroll
          for (int dx = -1; dx <= 1; ++dx) {
            const int slot = j * 3 + dx + 1;
            const T v = rowv[slot];
            const V2 xv = *reinterpret_cast<const V2*>(xb + j * capx + dx * 32);
            if (slot & 1) {
              a1.x = fma(v, xv.x, a1.x);
              a1.y = fma(v, xv.y, a1.y);
            } else {
              a0.x = fma(v, xv.x, a0.x);
              a0.y = fma(v, xv.y, a0.y);
            }
          }
        }
        sum.x = a0.x + a1.x;
        sum.y = a0.y + a1.y;
      } else if (ok) {
        const bool vxm = flags & 1, vxp = flags & 2, vym = flags & 4, vyp = flags & 8;
        const bool vzm = flags & 16, vzp = flags & 32;
        const int cx = 1 + vxm + vxp, cy = 1 + vym + vyp, cxy = cx * cy;
        const T* xc = sx + 4 * (size_t)capx + ((int64_t)r * 32 + 2 * h - s_xbase[s][4]);
        xr = *reinterpret_cast<const V2*>(xc);
        V2 a0{T(0), T(0)}, a1{T(0), T(0)};
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
            const int off = dz * P.NxNy + dy * P.Nx;
            const T* seg = sx + (size_t)j * capx + ((int64_t)(r + off) * 32 + 2 * h - s_xbase[s][j]);
            const int pbase = bz * cxy + by * cx;
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
              const bool vx = dx < 0 ? vxm : (dx > 0 ? vxp : true);
              const int bx = dx < 0 ? 0 : (dx == 0 ? (int)vxm : (int)vxm + 1);
              const bool valid = vz && vy && vx;
              const T v = valid ? rowv[pbase + bx] : T(0);
              const V2 xv = *reinterpret_cast<const V2*>(valid ? seg + dx * 32 : xc);
              if (slot & 1) {
                a1.x = fma(v, xv.x, a1.x);
                a1.y = fma(v, xv.y, a1.y);
              } else {
                a0.x = fma(v, xv.x, a0.x);
                a0.y = fma(v, xv.y, a0.y);
              }
              ++slot;
            }
          }
        }
        sum.x = a0.x + a1.x;
        sum.y = a0.y + a1.y;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
      if (ok) {
        const int64_t idx = (int64_t)r * 32 + 2 * h;
        if (MODE == MM_RESID) {
          const double2 b2 = *reinterpret_cast<const double2*>(P.b + idx);
          const double e0 = b2.x - widen(sum.x), e1 = b2.y - widen(sum.y);
          typename Vec2<RT>::type o;
          o.x = (RT)e0;
          o.y = (RT)e1;
          *reinterpret_cast<typename Vec2<RT>::type*>(P.yres + idx) = o;
          d0 = fma(e0, e0, d0);
          d1 = fma(e1, e1, d1);
        } else {
          *reinterpret_cast<V2*>(P.y + idx) = sum;
          if (MODE == MM_DOT) {
            if constexpr (sizeof(T) == 4) {
              f0.add_product(sum.x, xr.x);
              f1.add_product(sum.y, xr.y);
            } else {
              d0 = fma(sum.x, xr.x, d0);
              d1 = fma(sum.y, xr.y, d1);
            }
          }
        }
      }
    }
    // to one lane per right-hand side: j = 2h + c is held by lanes h, h + 16
    double t0 = d0 + f0.value(), t1 = d1 + f1.value();
    t0 += __shfl_xor_sync(0xffffffffu, t0, 16);
    t1 += __shfl_xor_sync(0xffffffffu, t1, 16);
    const double u0 = __shfl_sync(0xffffffffu, t0, lane >> 1);
    const double u1 = __shfl_sync(0xffffffffu, t1, lane >> 1);
    dacc = (lane & 1) ? u1 : u0;
  } else {
    // any nrhs dividing 32: consumer warp w handles rows w and w + 16 of each
    // tile, one lane per right-hand side
    const int w = warp - kProdM;
    const bool lane_on = lane < nr;
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      const int s = it % S;
      if (!mbar_wait_bounded(&full[s], (unsigned)((it / S) & 1))) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        break;
      }
      T sum[R / kConsM], xr[R / kConsM];
      bool okq[R / kConsM];
#pragma unroll
      for (int q = 0; q < R / kConsM; ++q) {
        const int lr = w + q * kConsM;
        const int r = tile * R + lr;
        const int flags = s_rflags[s][lr];
        const bool ok = r < P.n && s_ok[s] != 0;
        okq[q] = ok;
        sum[q] = T(0);
        xr[q] = T(0);
        const int lj = lane_on ? lane : 0;
        const T* sv = st0 + (size_t)s * stage_elems;
        const T* sx = sv + capv;
        const T* rowv = sv + (s_rro[s][lr] - s_vbase[s]);
        if (!ok) continue;
        const bool vxm = flags & 1, vxp = flags & 2, vym = flags & 4, vyp = flags & 8;
        const bool vzm = flags & 16, vzp = flags & 32;
        const int cx = 1 + vxm + vxp, cy = 1 + vym + vyp, cxy = cx * cy;
        const T* xc = sx + 4 * (size_t)capx + ((int64_t)r * nr + lj - s_xbase[s][4]);
        xr[q] = xc[0];
        T s0 = T(0), s1 = T(0);
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
            const int off = dz * P.NxNy + dy * P.Nx;
            const T* seg = sx + (size_t)j * capx + ((int64_t)(r + off) * nr + lj - s_xbase[s][j]);
            const int pbase = bz * cxy + by * cx;
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
              const bool vx = dx < 0 ? vxm : (dx > 0 ? vxp : true);
              const int bx = dx < 0 ? 0 : (dx == 0 ? (int)vxm : (int)vxm + 1);
              const bool valid = vz && vy && vx;
              const T v = valid ? rowv[pbase + bx] : T(0);
              const T xv = *(valid ? seg + (int64_t)dx * nr : xc);
              if (slot & 1)
                s1 = fma(v, xv, s1);
              else
                s0 = fma(v, xv, s0);
              ++slot;
            }
          }
        }
        sum[q] = s0 + s1;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
#pragma unroll
      for (int q = 0; q < R / kConsM; ++q) {
        if (!okq[q] || !lane_on) continue;
        const int64_t idx = (int64_t)(tile * R + w + q * kConsM) * nr + lane;
        if (MODE == MM_RESID) {
          const double res = P.b[idx] - widen(sum[q]);
          P.yres[idx] = (RT)res;
          dacc = fma(res, res, dacc);
        } else {
          P.y[idx] = sum[q];
          if (MODE == MM_DOT) {
            if constexpr (sizeof(T) == 4)
              facc.add_product(sum[q], xr[q]);
            else
              dacc = fma(sum[q], xr[q], dacc);
          }
        }
      }
    }
  }
  if (MODE != MM_PLAIN)
    multi_dot_reduce(warp < kProdM ? 0.0 : dacc + facc.value(), red, P.partials, P.ticket, P.out, nr,
                     MODE == MM_DOT ? P.cg : nullptr);
}

// ---------------------------------------------------------------------------
// FP32 A P for exactly 32 right-hand sides in the mixed solver: the matrix in a
// padded 28-per-row layout (the 27 stencil slots in (dz, dy, dx) order, zeros
// for missing neighbours, one zero pad so every row starts on 16 bytes) and P
// with ghost zones of zero rows around it, so no row needs a mask.  Each
// consumer warp owns four consecutive rows with one lane per right-hand side:
// the six x values of each of the nine lines serve all four rows (54 loads per
// 108 FMAs instead of one load per FMA), and each row's values come in seven
// 16-byte broadcast loads; shared-memory traffic per row is half that of
// k_spmm_box.
// ---------------------------------------------------------------------------
constexpr int kER = 32;                     // rows per tile
constexpr int kEW = 8;                      // consumer warps, four rows each
constexpr int kECapX = (kER + 2) * 32;      // floats per x segment
constexpr int kECapV = kER * 28;            // floats of a tile's values
constexpr int kEStage = kECapV + 9 * kECapX;
constexpr int kEThreads = (kEW + 2) * 32;

struct Ell32Params {
  int n, Nx, NxNy;
  const float* __restrict__ ell;  // [ceil(n/32)*32][28]
  const float* __restrict__ p;    // n x 32, ghost zones before and after
  float* __restrict__ Ap;
  double* partials;
  unsigned* ticket;
  MultiState* st;
  unsigned* err;
};

__global__ void __launch_bounds__(kEThreads, 2) k_spmm_ell32(Ell32Params P)
{
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t full[2], empty[2];
  __shared__ double red[(kEW + 2) * 32];
  float* const st0 = reinterpret_cast<float*>(smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = (P.n + kER - 1) / kER;
  if (threadIdx.x == 0) {
    for (int s = 0; s < 2; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], kEW);
    }
    fence_mbar_init();
  }
  __syncthreads();
  DFAcc facc;
  if (warp < 2) {
    // producer warp w stages the CTA's tiles it = w, w + 2, ... into stage w
    const int s = warp;
    bool ok = true;
    int it = warp;
    for (int tile = blockIdx.x + warp * gridDim.x; tile < ntiles; tile += 2 * gridDim.x, it += 2) {
      if (it >= 2) {
        if (lane == 0) ok = mbar_wait_bounded(&empty[s], (unsigned)(((it / 2) - 1) & 1));
        ok = __shfl_sync(0xffffffffu, ok, 0);
      }
      if (!ok) break;
      float* sv = st0 + (size_t)s * kEStage;
      const int64_t r0 = (int64_t)tile * kER;
      if (lane < 9) {
        const int64_t off = (int64_t)(lane / 3 - 1) * P.NxNy + (lane % 3 - 1) * P.Nx;
        const unsigned bytes = kECapX * sizeof(float);
        mbar_expect_tx(&full[s], bytes);
        bulk_g2s(sv + kECapV + lane * kECapX, P.p + (r0 + off - 1) * 32, bytes, &full[s]);
      } else if (lane == 9) {
        const unsigned bytes = kECapV * sizeof(float);
        mbar_expect_tx(&full[s], bytes);
        bulk_g2s(sv, P.ell + r0 * 28, bytes, &full[s]);
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&full[s]);
    }
    if (!ok && lane == 0) {
      // bounded wait for the copies of this warp's last issued tile
      atomicOr(P.err, ERR_WAIT_TIMEOUT);
      mbar_wait_bounded(&full[s], (unsigned)(((it - 2) / 2) & 1));
    }
  } else {
    const int cw = warp - 2;
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      const int s = it & 1;
      if (!mbar_wait_bounded(&full[s], (unsigned)((it >> 1) & 1))) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        break;
      }
      const float* sv = st0 + (size_t)s * kEStage;
      // segment j holds rows r0 + off_j - 1 .. r0 + off_j + 32: local row
      // 4cw + k is the neighbour dx = k - i - 1 of row 4cw + i
      const float* xs = sv + kECapV + (4 * cw) * 32 + lane;
      float xw[9][6];
#pragma unroll
      for (int j = 0; j < 9; ++j)
#pragma unroll
        for (int k = 0; k < 6; ++k) xw[j][k] = xs[j * kECapX + k * 32];
      float acc[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const float4* v4 = reinterpret_cast<const float4*>(sv + (4 * cw + i) * 28);
        float v[28];
#pragma unroll
        for (int q = 0; q < 7; ++q) {
          const float4 t = v4[q];
          v[4 * q] = t.x;
          v[4 * q + 1] = t.y;
          v[4 * q + 2] = t.z;
          v[4 * q + 3] = t.w;
        }
        float a0 = 0.0f, a1 = 0.0f;
#pragma unroll
        for (int k = 0; k < 27; ++k) {
          if (k & 1)
            a1 = fmaf(v[k], xw[k / 3][i + k % 3], a1);
          else
            a0 = fmaf(v[k], xw[k / 3][i + k % 3], a0);
        }
        acc[i] = a0 + a1;
      }
      __syncwarp();
      if (lane == 0) mbar_arrive(&empty[s]);
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const int64_t r = (int64_t)tile * kER + 4 * cw + i;
        if (r < P.n) {
          P.Ap[r * 32 + lane] = acc[i];
          facc.add_product(acc[i], xw[4][i + 1]);
        }
      }
    }
  }
  multi_dot_reduce(warp < 2 ? 0.0 : facc.value(), red, P.partials, P.ticket, P.st->pAp, 32, P.st);
}

// ---------------------------------------------------------------------------
// FP32 A P for exactly 32 right-hand sides on the verified FP32 stencil
// operator of the mixed solver (mfe_stencil.cu: every row dd * x_r or the
// interior stencil with Dirichlet neighbours zeroed, checked on the matrix
// on every call) with mirror-symmetric weights: P and AP are the only
// traffic, 256 bytes per row, instead of 368 with the padded values.  A
// warp owns four adjacent positions of the xy plane, one lane per
// right-hand side, and marches a chunk of z steps: each plane's window
// (lines y - 1, y, y + 1 at positions p - 1 .. p + 4) is six 128-byte rows
// per line, read coalesced, reduced once to the class sums a, sx, sy, sxy of
// its four rows, and combined as in the FP64 stencil kernel
// (mfe_stencil64.cu): P1(z) = w4 a + w5 sx + w6 sy + w7 sxy, Q(z) = P1(z-1)
// + w0 a + w1 sx + w2 sy + w3 sxy, AP(z) = Q(z) + P1(z+1).  The masks of
// Dirichlet neighbours are the same for the whole warp (one set of
// positions), so no lane diverges.  Work items are (z chunk, position
// tile), z-chunk major, so the warps resident together share lines through
// L2.  p.Ap per right-hand side in double-float, then multi_dot_reduce.
// ---------------------------------------------------------------------------
constexpr int kSMW = 8;    // warps per CTA
constexpr int kSMKP = 4;   // positions per warp
constexpr int kSMZC = 32;  // default z steps per work item (mfe_multi_set_tuning)

struct MSt32Params {
  int Nx, Ny, Nz, NxNy, ntile, nzc, zc;  // zc: z steps per work item
  float w[8];  // mirror-class weights, class 4|dz| + 2|dy| + |dx|
  float dd;    // Dirichlet diagonal
  const float* __restrict__ p;  // n x 32
  float* __restrict__ Ap;       // n x 32
  double* partials;
  unsigned* ticket;
  MultiState* st;
};

// One work item (positions p0 .. p0 + 3, planes za .. zb - 1) of
// k_spmm_st32.  MASKED: some window entry is not an interior node (masks and
// Dirichlet rows apply); otherwise every window entry of every plane is
// interior and the loads need neither predicates nor selects.  Rows of the
// item are row (z, r) = z NxNy + p0 + r, lane = right-hand side.
template <bool MASKED>
__device__ __forceinline__ void st32_item(const MSt32Params& P, int p0, int za, int zb, unsigned mask,
                                          DFAcc& facc)
{
  constexpr int KP = kSMKP, W = KP + 2;
  const int lane = threadIdx.x & 31;
  const int64_t line = (int64_t)P.Nx * 32, plane_stride = (int64_t)P.NxNy * 32;
  // element (plane z, line y + j - 1, position p0 - 1 + t) of lane's column:
  // pz + (j - 1) * line + 32 t, pz = the plane's window origin
  const float* const p_org = P.p + ((int64_t)p0 - 1) * 32 + lane;
  bool valid[KP], bnd[KP];
#pragma unroll
  for (int r = 0; r < KP; ++r) {
    valid[r] = !MASKED || p0 + r < P.NxNy;
    bnd[r] = MASKED && !((mask >> (W + 1 + r)) & 1u);
  }
  auto plane = [&](int z, const float* P1in, float* P1, float* Qo, float* cen) {
    const float* pz = p_org + (int64_t)z * plane_stride;
#pragma unroll
    for (int r = 0; r < KP; ++r) cen[r] = valid[r] ? __ldg(pz + 32 * (r + 1)) : 0.0f;
    if (z <= 0 || z >= P.Nz - 1) {  // a Dirichlet plane (uniform)
#pragma unroll
      for (int r = 0; r < KP; ++r) P1[r] = Qo[r] = 0.0f;
      return;
    }
    float v[3 * W];
#pragma unroll
    for (int j = 0; j < 3; ++j)
#pragma unroll
      for (int t = 0; t < W; ++t) {
        const int sl = W * j + t;
        if (j == 1 && t >= 1 && t <= KP) {
          v[sl] = MASKED && !((mask >> sl) & 1u) ? 0.0f : cen[t - 1];
        } else {
          const float* a = pz + (j - 1) * line + 32 * t;
          v[sl] = MASKED ? (((mask >> sl) & 1u) ? __ldg(a) : 0.0f) : __ldg(a);
        }
      }
    float e[W];
#pragma unroll
    for (int t = 0; t < W; ++t) e[t] = v[t] + v[2 * W + t];
#pragma unroll
    for (int r = 0; r < KP; ++r) {
      const float a = v[W + 1 + r];
      const float sx = v[W + r] + v[W + r + 2];
      const float sy = e[1 + r];
      const float sxy = e[r] + e[r + 2];
      float p1 = P.w[4] * a;
      p1 = fmaf(P.w[5], sx, p1);
      p1 = fmaf(P.w[6], sy, p1);
      P1[r] = fmaf(P.w[7], sxy, p1);
      float qv = fmaf(P.w[0], a, P1in[r]);
      qv = fmaf(P.w[1], sx, qv);
      qv = fmaf(P.w[2], sy, qv);
      Qo[r] = fmaf(P.w[3], sxy, qv);
    }
  };
  float P1c[KP], Qc[KP], cc[KP];
#pragma unroll
  for (int r = 0; r < KP; ++r) P1c[r] = 0.0f;
  if (za >= 1) {
    float zq[KP], qd[KP], cd[KP];
#pragma unroll
    for (int r = 0; r < KP; ++r) zq[r] = 0.0f;
    plane(za - 1, zq, P1c, qd, cd);
  }
  {
    float P1n[KP];
    plane(za, P1c, P1n, Qc, cc);
#pragma unroll
    for (int r = 0; r < KP; ++r) P1c[r] = P1n[r];
  }
  float* yz = P.Ap + ((int64_t)za * P.NxNy + p0) * 32 + lane;
  for (int z = za; z < zb; ++z) {
    float P1n[KP], Qn[KP], cn[KP];
#pragma unroll
    for (int r = 0; r < KP; ++r) P1n[r] = Qn[r] = cn[r] = 0.0f;
    if (z + 1 < P.Nz) plane(z + 1, P1c, P1n, Qn, cn);
    const bool dplane = z == 0 || z == P.Nz - 1;
#pragma unroll
    for (int r = 0; r < KP; ++r) {
      const float yv = (dplane || bnd[r]) ? P.dd * cc[r] : Qc[r] + P1n[r];
      if (valid[r]) {
        yz[32 * r] = yv;
        facc.add_product(yv, cc[r]);
      }
      P1c[r] = P1n[r];
      Qc[r] = Qn[r];
      cc[r] = cn[r];
    }
    yz += plane_stride;
  }
}

__global__ void __launch_bounds__(kSMW * 32) k_spmm_st32(const __grid_constant__ MSt32Params P)
{
  constexpr int KP = kSMKP, W = KP + 2;
  constexpr unsigned kAll = (1u << (3 * W)) - 1u;
  __shared__ double red[kSMW * 32];
  const int warp = threadIdx.x >> 5;
  const int64_t items = (int64_t)P.nzc * P.ntile;
  DFAcc facc;
  for (int64_t it = (int64_t)blockIdx.x * kSMW + warp; it < items; it += (int64_t)gridDim.x * kSMW) {
    const int zc = (int)(it / P.ntile), tile = (int)(it - (int64_t)zc * P.ntile);
    const int za = zc * P.zc, zb = min(P.Nz, za + P.zc);
    const int p0 = tile * KP;
    // bit W j + t: window entry (line y + j - 1, position p0 - 1 + t) is an
    // interior node (its row lies inside the plane), the same for all lanes
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
    if (mask == kAll)
      st32_item<false>(P, p0, za, zb, mask, facc);
    else
      st32_item<true>(P, p0, za, zb, mask, facc);
  }
  multi_dot_reduce(facc.value(), red, P.partials, P.ticket, P.st->pAp, 32, P.st);
}

// FP64 box CSR -> FP32 padded 28-per-row values (slot order, zeros outside
// the box and in the pad); rows n .. are left as the caller zeroed them
__global__ void k_mr_ell28(int Nx, int Ny, int Nz, const double* __restrict__ vals,
                           float* __restrict__ ell)
{
  const int n = Nx * Ny * Nz, NxNy = Nx * Ny;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const int iz = r / NxNy, rem = r - iz * NxNy, iy = rem / Nx, ix = rem - iy * Nx;
    int64_t k = row_offset(ix, iy, iz, Nx, Ny, Nz);
    float* out = ell + (int64_t)r * 28;
    int slot = 0;
    for (int dz = -1; dz <= 1; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx, ++slot) {
          const bool in = ix + dx >= 0 && ix + dx < Nx && iy + dy >= 0 && iy + dy < Ny &&
                          iz + dz >= 0 && iz + dz < Nz;
          out[slot] = in ? (float)vals[k++] : 0.0f;
        }
    out[27] = 0.0f;
  }
}

// lanes j, j+nrhs, j+2nrhs, ... of a warp hold right-hand side j: sum them
// into lane j (nrhs divides 32)
__device__ __forceinline__ double lane_group_sum(double v, int nrhs)
{
  for (int o = 16; o >= nrhs; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// 16-byte vectors of the work arrays: element e of the n x nrhs block
// belongs to right-hand side e % nrhs, so the VW components of a thread's
// vectors keep the same right-hand sides across its grid-stride loop
// (the stride is a multiple of 32 elements).
template <typename V>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
  static constexpr int n = 4;
};
template <>
struct Vec16<double> {
  using type = double2;
  static constexpr int n = 2;
};
template <typename V>
__device__ __forceinline__ V& comp(typename Vec16<V>::type& v, int c)
{
  return reinterpret_cast<V*>(&v)[c];
}

template <typename V>
__global__ void __launch_bounds__(kVT)
    k_mr_p(int64_t ntot, int nrhs, const V* __restrict__ r, V* __restrict__ p, float* __restrict__ x32,
           const MultiState* st)
{
  using VV = typename Vec16<V>::type;
  constexpr int VW = Vec16<V>::n;
  const int64_t g0 = (int64_t)blockIdx.x * kVT + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * kVT;
  const bool first = st->first != 0;
  // mixed (V = float): the last update's x32 += alpha p, done here where the
  // old p is read anyway (st->alpha still holds that update's alphas), unless
  // the reliable update already folded it in
  constexpr bool kX = sizeof(V) == 4;
  const bool addx = kX && !first && st->x_pending != 0;
  V beta[VW], alpha[VW];
#pragma unroll
  for (int c = 0; c < VW; ++c) {
    const int j = (VW * threadIdx.x + c) % nrhs;
    beta[c] = st->done[j] ? V(0) : (V)st->beta[j];
    alpha[c] = (V)st->alpha[j];
  }
  const int64_t nvec = ntot / VW;
  const VV* r4 = reinterpret_cast<const VV*>(r);
  VV* p4 = reinterpret_cast<VV*>(p);
  for (int64_t v = g0; v < nvec; v += stride) {
    const VV rv = r4[v];
    VV pv = first ? rv : p4[v];
    if (!first) {
      if constexpr (kX) {
        if (addx) {
          VV* x4 = reinterpret_cast<VV*>(x32);
          VV xv = x4[v];
#pragma unroll
          for (int c = 0; c < VW; ++c) comp<V>(xv, c) = fma(alpha[c], comp<V>(pv, c), comp<V>(xv, c));
          x4[v] = xv;
        }
      }
#pragma unroll
      for (int c = 0; c < VW; ++c) comp<V>(pv, c) = fma(beta[c], comp<V>(pv, c), comp<V>(const_cast<VV&>(rv), c));
    }
    p4[v] = pv;
  }
  if (g0 == nvec % stride) {
#pragma unroll
    for (int c = 0; c < VW; ++c) {
      const int64_t e = nvec * VW + c;
      if (e >= ntot) continue;
      if constexpr (kX) {
        if (addx) x32[e] = fma(alpha[c], p[e], x32[e]);
      }
      p[e] = first ? r[e] : fma(beta[c], p[e], r[e]);
    }
  }
}

// x += alpha_j p, r -= alpha_j Ap, rr_new_j = r_j.r_j; x is the FP32
// correction x32 in the mixed solver and the FP64 solution otherwise.  The
// FP32 squares are summed in double-float, the FP64 ones in FP64.
template <typename V>
__global__ void __launch_bounds__(kVT)
    k_mr_update(int64_t ntot, int nrhs, V* __restrict__ x, V* __restrict__ r,
                const V* __restrict__ p, const V* __restrict__ Ap, MultiState* st,
                double* partials, unsigned* ticket)
{
  using VV = typename Vec16<V>::type;
  constexpr int VW = Vec16<V>::n;
  __shared__ double red[(kVT / 32 + 1) * 32];
  __shared__ double ent[kVT * VW];
  const int64_t g0 = (int64_t)blockIdx.x * kVT + threadIdx.x;
  const int64_t stride = (int64_t)gridDim.x * kVT;
  V alpha[VW];
#pragma unroll
  for (int c = 0; c < VW; ++c) {
    alpha[c] = (V)st->alpha[(VW * threadIdx.x + c) % nrhs];
  }
  double acc[VW];
  DFAcc facc[VW];
#pragma unroll
  for (int c = 0; c < VW; ++c) acc[c] = 0.0;
  const int64_t nvec = ntot / VW;
  VV* x4 = reinterpret_cast<VV*>(x);
  VV* r4 = reinterpret_cast<VV*>(r);
  const VV* p4 = reinterpret_cast<const VV*>(p);
  const VV* a4 = reinterpret_cast<const VV*>(Ap);
  // mixed (V = float): x32 += alpha p is left pending (k_mr_p / k_mr_xupdate)
  constexpr bool kX = sizeof(V) == 8;
  for (int64_t v = g0; v < nvec; v += stride) {
    VV xv, rv = r4[v], pv, av = a4[v];
    if constexpr (kX) {
      xv = x4[v];
      pv = p4[v];
    }
#pragma unroll
    for (int c = 0; c < VW; ++c) {
      if constexpr (kX) comp<V>(xv, c) = fma(alpha[c], comp<V>(pv, c), comp<V>(xv, c));
      const V rn = fma(-alpha[c], comp<V>(av, c), comp<V>(rv, c));
      comp<V>(rv, c) = rn;
      if constexpr (sizeof(V) == 4)
        facc[c].add_product(rn, rn);
      else
        acc[c] = fma(rn, rn, acc[c]);
    }
    if constexpr (kX) x4[v] = xv;
    r4[v] = rv;
  }
  if (g0 == nvec % stride) {
#pragma unroll
    for (int c = 0; c < VW; ++c) {
      const int64_t e = nvec * VW + c;
      if (e >= ntot) continue;
      if constexpr (kX) x[e] = fma(alpha[c], p[e], x[e]);
      const V rn = fma(-alpha[c], Ap[e], r[e]);
      r[e] = rn;
      if constexpr (sizeof(V) == 4)
        facc[c].add_product(rn, rn);
      else
        acc[c] = fma(rn, rn, acc[c]);
    }
  }
  // entry VW*t + c holds right-hand side (VW*t + c) % nrhs; entries t + k*kVT
  // share thread t's right-hand side t % nrhs
#pragma unroll
  for (int c = 0; c < VW; ++c) ent[VW * threadIdx.x + c] = acc[c] + facc[c].value();
  __syncthreads();
  double a = 0.0;
#pragma unroll
  for (int k = 0; k < VW; ++k) a += ent[threadIdx.x + k * kVT];
  a = lane_group_sum(a, nrhs);
  if ((threadIdx.x & 31) >= nrhs) a = 0.0;
  multi_dot_reduce(a, red, partials, ticket, st->rr_new, nrhs);
}

__global__ void __launch_bounds__(kVT)
    k_mr_xupdate(int64_t ntot, int nrhs, double* __restrict__ x, float* __restrict__ x32,
                 const float* __restrict__ p, MultiState* st)
{
  if (st->gate == 0) return;
  // the pending x32 += alpha p folded in (the same FP32 FMA k_mr_p would do)
  for (int64_t i = (int64_t)blockIdx.x * kVT + threadIdx.x; i < ntot; i += (int64_t)gridDim.x * kVT) {
    const float alpha = (float)st->alpha[i % nrhs];
    x[i] += f2d_exact(fmaf(alpha, p[i], x32[i]));
    x32[i] = 0.0f;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) st->x_pending = 0;  // read next by k_mr_p only
}

// Mixed solver, one warp, after the update kernel: decide whether this
// iteration ends with a reliable update, which all right-hand sides share:
// when every open one has its recursive residual fallen by inner_tol since
// the last update or claims convergence, after refine_k iterations, or at the
// iteration limit.  (Waiting for the slowest keeps the update count near a
// single solve's; a right-hand side that claims convergence early keeps
// iterating on its recursion until the update checks its true residual.)
// Inside the graph (in_graph) the reliable update runs in a conditional node:
// this kernel sets its condition (h_upd) and, for an iteration without one,
// does k_mr_after's bookkeeping and sets the loop condition (h_loop).
__global__ void k_mr_decide(MultiState* st, cudaGraphConditionalHandle h_loop,
                            cudaGraphConditionalHandle h_upd, int in_graph)
{
  const int j = threadIdx.x;
  const int nr = st->nrhs;
  bool ready = true, brk = false;
  if (j < nr && !st->done[j]) {
    // p.Ap <= 0 (alpha was 0): this right-hand side stops at the reliable
    // update taken now, converged if its true residual says so
    brk = !(st->pAp[j] > 0.0);
    if (brk) st->brk[j] = 1;
    const double t = st->rr_new[j];
    ready = t < st->delta2 * st->rr_at_update[j] || t <= st->tol_abs[j] * st->tol_abs[j];
  }
  const bool all_ready = __all_sync(0xffffffffu, ready);
  const bool any_brk = __any_sync(0xffffffffu, brk);
  const int k = st->k + 1, since = st->since + 1;
  const bool gate = all_ready || any_brk || since >= st->refine_k || k >= st->max_iter;
  __syncwarp();
  if (j == 0) {
    st->k = k;
    st->since = since;
    st->first = 0;
    st->x_pending = 1;  // this iteration's x32 += alpha p (k_mr_p next, or k_mr_xupdate)
    st->gate = gate;
  }
  if (!in_graph) return;
  if (!gate) {
    if (j < nr && !st->done[j]) {
      st->beta[j] = st->rr_new[j] / st->rr[j];
      st->rr[j] = st->rr_new[j];
    }
    const bool open = __any_sync(0xffffffffu, j < nr && !st->done[j]);
    if (j == 0) {
      st->cont = open && k < st->max_iter;
      cudaGraphSetConditional(h_loop, st->cont ? 1u : 0u);
    }
  }
  if (j == 0) cudaGraphSetConditional(h_upd, gate ? 1u : 0u);
}

// Mixed solver, one warp, after the gated FP64 residual: per right-hand side
// beta and rr from the true residual (reliable update) or the recursive one.
__global__ void k_mr_after(MultiState* st, cudaGraphConditionalHandle h, int in_graph)
{
  const int j = threadIdx.x;
  const int nr = st->nrhs;
  const int gate = st->gate;
  if (j < nr && !st->done[j]) {
    if (gate) {
      st->normr_true[j] = sqrt(st->rr_true[j]);
      if (st->normr_true[j] <= st->tol_abs[j]) {
        st->done[j] = 1;
        st->iters[j] = st->k;
        st->brk[j] = 0;
      } else if (st->brk[j]) {
        st->done[j] = 1;
        st->iters[j] = st->k - 1;
      } else {
        st->beta[j] = st->rr_true[j] / st->rr[j];
        st->rr[j] = st->rr_true[j];
        st->rr_at_update[j] = st->rr_true[j];
      }
    } else {
      st->beta[j] = st->rr_new[j] / st->rr[j];
      st->rr[j] = st->rr_new[j];
    }
  }
  const bool open = __any_sync(0xffffffffu, j < nr && !st->done[j]);
  if (j == 0) {
    if (gate) {
      st->updates += 1;
      st->since = 0;
    }
    st->gate = 0;
    st->cont = open && st->k < st->max_iter &&
               !(gate && st->max_refine > 0 && st->updates >= st->max_refine);
    if (in_graph) cudaGraphSetConditional(h, st->cont ? 1u : 0u);
  }
}

// FP64 solver, one warp, after the update kernel of iteration k: the
// reference's loop test per right-hand side (cg_solve.hpp: the loop runs
// iteration k+1 while k+1 <= max_iter and normr > tol, normr being |r| at the
// top of iteration k, i.e. before its update).
__global__ void k_mr_after64(MultiState* st, cudaGraphConditionalHandle h, int in_graph)
{
  const int j = threadIdx.x;
  const int nr = st->nrhs;
  const int k = st->k + 1;
  if (j < nr && !st->done[j]) {
    if (!(st->pAp[j] > 0.0)) {
      // the reference reports a breakdown and returns with the k-1
      // completed iterations (cg_solve.hpp:186-198); the others go on
      st->brk[j] = 1;
      st->done[j] = 1;
      st->iters[j] = k - 1;
    } else if (k + 1 <= st->max_iter && st->normr_true[j] > st->tol_abs[j]) {
      const double rn = st->rr_new[j];
      st->beta[j] = rn / st->rr[j];
      st->rr[j] = rn;
      st->normr_true[j] = sqrt(rn);
    } else {
      st->done[j] = 1;
      st->iters[j] = k;
    }
  }
  const bool open = __any_sync(0xffffffffu, j < nr && !st->done[j]);
  if (j == 0) {
    st->k = k;
    st->first = 0;
    st->cont = open;
    if (in_graph) cudaGraphSetConditional(h, st->cont ? 1u : 0u);
  }
}

__global__ void k_mr_init(MultiState* st)
{
  const int j = threadIdx.x;
  const int nr = st->nrhs;
  if (j < nr) {
    const double nrm = sqrt(st->rr_true[j]);
    st->normr0[j] = nrm;
    st->normr_true[j] = nrm;
    if (st->tol_mode) st->tol_abs[j] *= nrm;
    st->rr[j] = st->rr_true[j];
    st->rr_at_update[j] = st->rr_true[j];
    st->done[j] = !(nrm > st->tol_abs[j]);
    st->iters[j] = 0;
  }
  const bool open = __any_sync(0xffffffffu, j < nr && !st->done[j]);
  if (j == 0) st->cont = open && st->max_iter > 0;
}

__global__ void k_mr_begin(const MultiState* st, cudaGraphConditionalHandle h)
{
  cudaGraphSetConditional(h, st->cont ? 1u : 0u);
}

// ---------------------------------------------------------------------------
// host
// ---------------------------------------------------------------------------
namespace {

template <typename T>
size_t spmm_smem(int nrhs)
{
  return (size_t)spmm_stages<T>() * ((size_t)spmm_capv() + 9 * (size_t)spmm_capx(nrhs)) * sizeof(T);
}

// Raises the dynamic shared memory limit of one kernel instantiation to what
// nrhs needs (the limit is per kernel, so it only grows) and returns its
// resident CTAs per SM for nrhs; cached per (device, nrhs) so launches
// recorded into a graph make no further runtime calls.
template <typename T, int MODE, typename RT, int NRC>
mfe_status spmm_setup_k(mfe_ctx* ctx, int nrhs, int* per_sm)
{
  static std::map<std::pair<int, int>, int> occ;
  static std::map<int, size_t> limit;
  static std::mutex mu;
  std::lock_guard<std::mutex> lock(mu);
  const auto key = std::make_pair(ctx->device, nrhs);
  auto it = occ.find(key);
  if (it == occ.end()) {
    const size_t smem = spmm_smem<T>(nrhs);
    size_t& lim = limit[ctx->device];
    if (smem > lim) {
      MFE_CUDA_TRY(ctx, cudaFuncSetAttribute(k_spmm_box<T, MODE, RT, NRC>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem));
      lim = smem;
    }
    int n = 1;
    MFE_CUDA_TRY(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                          &n, k_spmm_box<T, MODE, RT, NRC>, kThreadsM, smem));
    it = occ.emplace(key, std::max(n, 1)).first;
  }
  if (per_sm) *per_sm = it->second;
  return MFE_OK;
}

template <typename T, int MODE, typename RT>
mfe_status spmm_setup(mfe_ctx* ctx, int nrhs, int* per_sm)
{
  if (nrhs == 32) return spmm_setup_k<T, MODE, RT, 32>(ctx, nrhs, per_sm);
  return spmm_setup_k<T, MODE, RT, 0>(ctx, nrhs, per_sm);
}

template <typename T, int MODE, typename RT>
mfe_status launch_spmm_t(mfe_ctx* ctx, const mfe_csr* A, int nrhs, const T* X, T* Y,
                         const double* Bv, RT* yres, double* partials, unsigned* ticket,
                         double* out, const int* gate, unsigned* err, MultiState* cg = nullptr)
{
  SpmmParams<T, RT> P;
  P.Nx = A->box_nx + 1;
  P.Ny = A->box_ny + 1;
  P.Nz = A->box_nz + 1;
  P.NxNy = P.Nx * P.Ny;
  P.n = (int)A->nrows;
  P.nrhs = nrhs;
  P.nnz = A->nnz;
  P.vals = static_cast<const T*>(A->vals);
  P.x = X;
  P.y = Y;
  P.b = Bv;
  P.yres = yres;
  P.capv = spmm_capv();
  P.capx = spmm_capx(nrhs);
  P.partials = partials;
  P.ticket = ticket;
  P.out = out;
  P.gate = gate;
  P.err = err;
  P.cg = cg;
  const size_t smem = spmm_smem<T>(nrhs);
  const int threads = kThreadsM;
  int per_sm = 1;
  MFE_TRY((spmm_setup<T, MODE, RT>(ctx, nrhs, &per_sm)));
  const int64_t ntiles = ceil_div(A->nrows, (int64_t)kTileRowsM);
  const int grid = (int)std::max<int64_t>(
      1, std::min<int64_t>({ntiles, (int64_t)ctx->sm_count * per_sm, (int64_t)kMaxPartM}));
  if (nrhs == 32)
    k_spmm_box<T, MODE, RT, 32><<<grid, threads, smem, ctx->stream>>>(P);
  else
    k_spmm_box<T, MODE, RT, 0><<<grid, threads, smem, ctx->stream>>>(P);
  return check_launch(ctx, "k_spmm_box");
}

template <typename V>
struct MultiBufs {
  V *r, *p, *Ap;
  float* x32;  // mixed only
  MultiState* st;
  double* partials;  // [2][kMaxPartM][32]
  unsigned* tickets;
  unsigned* err;
  const float* ell = nullptr;  // mixed, 32 right-hand sides: padded values (p has ghost zones)
  int ell_grid = 0;
  // mixed, 32 right-hand sides, verified mirror-symmetric FP32 stencil:
  // k_spmm_st32 with these weights (takes precedence over ell)
  bool st32 = false;
  float w8[8] = {};
  float dd = 0.0f;
  int st32_grid = 0;
  int st32_zc = kSMZC;
};

size_t ell32_smem() { return (size_t)2 * kEStage * sizeof(float); }

// resident CTAs of k_spmm_ell32 on this device (attribute set once, before
// any capture)
mfe_status ell32_grid(mfe_ctx* ctx, int* grid)
{
  MFE_CUDA_TRY(ctx, cudaFuncSetAttribute(k_spmm_ell32, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)ell32_smem()));
  *grid = resident_blocks(ctx, (const void*)k_spmm_ell32, kEThreads, ell32_smem());
  return MFE_OK;
}

// One wave of resident blocks (a second, partial wave of a grid-stride
// kernel would run at a fraction of the bandwidth): the occupancy of the
// kernel times the SM count, cached per kernel and device.
template <typename K>
int vgrid(mfe_ctx* ctx, int64_t n, K kernel)
{
  static std::map<std::pair<const void*, int>, int> cache;
  static std::mutex mu;
  int per_sm = 0;
  {
    std::lock_guard<std::mutex> lock(mu);
    const auto key = std::make_pair(reinterpret_cast<const void*>(kernel), ctx->device);
    auto it = cache.find(key);
    if (it == cache.end()) {
      int b = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kernel, kVT, 0) != cudaSuccess) b = 4;
      it = cache.emplace(key, std::max(b, 1)).first;
    }
    per_sm = it->second;
  }
  return (int)std::max<int64_t>(
      1, std::min<int64_t>({ceil_div(std::max<int64_t>(n, 1), (int64_t)kVT),
                            (int64_t)ctx->sm_count * per_sm, (int64_t)kMaxPartM}));
}

// one iteration of the mixed solver up to the update decision: FP32 SpMM,
// FP32 vectors (h_upd: the graph condition of the reliable update)
mfe_status multi_iter_mixed(mfe_ctx* ctx, const mfe_csr& A32, const mfe_csr& A64, int nrhs,
                            const MultiBufs<float>& W, cudaGraphConditionalHandle h,
                            cudaGraphConditionalHandle h_upd, int in_graph)
{
  const int64_t ntot = A64.nrows * (int64_t)nrhs;
  k_mr_p<float><<<vgrid(ctx, ntot, k_mr_p<float>), kVT, 0, ctx->stream>>>(ntot, nrhs, W.r, W.p, W.x32, W.st);
  MFE_TRY(check_launch(ctx, "k_mr_p"));
  if (W.st32) {
    MSt32Params S;
    S.Nx = A64.box_nx + 1;
    S.Ny = A64.box_ny + 1;
    S.Nz = A64.box_nz + 1;
    S.NxNy = S.Nx * S.Ny;
    S.ntile = (int)ceil_div(S.NxNy, (int64_t)kSMKP);
    S.zc = W.st32_zc;
    S.nzc = (int)ceil_div(S.Nz, (int64_t)S.zc);
    for (int c = 0; c < 8; ++c) S.w[c] = W.w8[c];
    S.dd = W.dd;
    S.p = W.p;
    S.Ap = W.Ap;
    S.partials = W.partials;
    S.ticket = W.tickets;
    S.st = W.st;
    k_spmm_st32<<<W.st32_grid, kSMW * 32, 0, ctx->stream>>>(S);
    MFE_TRY(check_launch(ctx, "k_spmm_st32"));
  } else if (W.ell) {
    Ell32Params E;
    E.n = (int)A64.nrows;
    E.Nx = A64.box_nx + 1;
    E.NxNy = E.Nx * (A64.box_ny + 1);
    E.ell = W.ell;
    E.p = W.p;
    E.Ap = W.Ap;
    E.partials = W.partials;
    E.ticket = W.tickets;
    E.st = W.st;
    E.err = W.err;
    k_spmm_ell32<<<W.ell_grid, kEThreads, ell32_smem(), ctx->stream>>>(E);
    MFE_TRY(check_launch(ctx, "k_spmm_ell32"));
  } else {
    MFE_TRY((launch_spmm_t<float, MM_DOT, float>(ctx, &A32, nrhs, W.p, W.Ap, nullptr, nullptr,
                                                  W.partials, W.tickets, W.st->pAp, nullptr, W.err,
                                                  W.st)));
  }
  k_mr_update<float><<<vgrid(ctx, ntot, k_mr_update<float>), kVT, 0, ctx->stream>>>(
      ntot, nrhs, W.x32, W.r, W.p, W.Ap, W.st, W.partials + (size_t)kMaxPartM * 32, W.tickets + 1);
  MFE_TRY(check_launch(ctx, "k_mr_update"));
  k_mr_decide<<<1, 32, 0, ctx->stream>>>(W.st, h, h_upd, in_graph);
  return check_launch(ctx, "k_mr_decide");
}

// the gated FP64 reliable update (inside the graph: in a conditional node)
// and the bookkeeping
mfe_status multi_update_mixed(mfe_ctx* ctx, const mfe_csr& A64, int nrhs, const double* B,
                              double* X, const MultiBufs<float>& W, cudaGraphConditionalHandle h,
                              int in_graph)
{
  const int64_t ntot = A64.nrows * (int64_t)nrhs;
  k_mr_xupdate<<<vgrid(ctx, ntot, k_mr_xupdate), kVT, 0, ctx->stream>>>(ntot, nrhs, X, W.x32, W.p, W.st);
  MFE_TRY(check_launch(ctx, "k_mr_xupdate"));
  MFE_TRY((launch_spmm_t<double, MM_RESID, float>(ctx, &A64, nrhs, X, nullptr, B, W.r, W.partials,
                                                   W.tickets, W.st->rr_true, &W.st->gate, W.err)));
  k_mr_after<<<1, 32, 0, ctx->stream>>>(W.st, h, in_graph);
  return check_launch(ctx, "k_mr_after");
}

// one iteration of the FP64 solver (the reference's CG per right-hand side)
mfe_status multi_iter_f64(mfe_ctx* ctx, const mfe_csr& A64, int nrhs, double* X,
                          const MultiBufs<double>& W, cudaGraphConditionalHandle h, int in_graph)
{
  const int64_t ntot = A64.nrows * (int64_t)nrhs;
  k_mr_p<double><<<vgrid(ctx, ntot, k_mr_p<double>), kVT, 0, ctx->stream>>>(ntot, nrhs, W.r, W.p, nullptr,
                                                                             W.st);
  MFE_TRY(check_launch(ctx, "k_mr_p"));
  MFE_TRY((launch_spmm_t<double, MM_DOT, double>(ctx, &A64, nrhs, W.p, W.Ap, nullptr, nullptr,
                                                  W.partials, W.tickets, W.st->pAp, nullptr, W.err,
                                                  W.st)));
  k_mr_update<double><<<vgrid(ctx, ntot, k_mr_update<double>), kVT, 0, ctx->stream>>>(
      ntot, nrhs, X, W.r, W.p, W.Ap, W.st, W.partials + (size_t)kMaxPartM * 32, W.tickets + 1);
  MFE_TRY(check_launch(ctx, "k_mr_update"));
  k_mr_after64<<<1, 32, 0, ctx->stream>>>(W.st, h, in_graph);
  return check_launch(ctx, "k_mr_after64");
}

// Runs `body` (which launches one iteration on ctx->stream) as a CUDA graph
// with a conditional while node driven by the state's `cont`, or, with
// MFE_CG_EAGER set, as a host loop reading `cont` back each iteration.  With
// `update`, the body ends with a conditional IF node holding `update`, its
// condition set by the body (the handle passed as body's second argument).
template <typename Body, typename Update>
mfe_status run_loop(mfe_ctx* ctx, MultiState* dev_st, MultiState* host_st, Body body,
                    Update update, bool with_update)
{
  if (getenv("MFE_CG_EAGER") != nullptr) {
    for (;;) {
      MFE_CUDA_TRY(ctx, cudaMemcpyAsync(host_st, dev_st, sizeof(MultiState),
                                        cudaMemcpyDeviceToHost, ctx->stream));
      MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      if (!host_st->cont) return MFE_OK;
      MFE_TRY(body((cudaGraphConditionalHandle)0, (cudaGraphConditionalHandle)0, 0));
      if (with_update) MFE_TRY(update((cudaGraphConditionalHandle)0, 0));
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
      k_mr_begin<<<1, 1, 0, s>>>(dev_st, h);
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
      cudaGraph_t body_graph = cp->conditional.phGraph_out[0];
      cudaGraphConditionalHandle hu = 0;
      if (with_update) e = cudaGraphConditionalHandleCreate(&hu, body_graph, 0, 0);
      if (e == cudaSuccess)
        e = cudaStreamBeginCaptureToGraph(s, body_graph, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeRelaxed);
      cudaGraphNode_t leaf[4];
      size_t nleaf = 0;
      if (e == cudaSuccess) {
        st = body(h, hu, 1);
        cudaError_t e1 = cudaSuccess;
        if (with_update) {
          cudaStreamCaptureStatus cs;
          const cudaGraphNode_t* deps = nullptr;
          size_t nd = 0;
          e1 = cudaStreamGetCaptureInfo(s, &cs, nullptr, nullptr, &deps, nullptr, &nd);
          if (e1 == cudaSuccess && nd >= 1 && nd <= 4) {
            for (size_t i = 0; i < nd; ++i) leaf[i] = deps[i];
            nleaf = nd;
          } else if (e1 == cudaSuccess) {
            e1 = cudaErrorUnknown;
          }
        }
        cudaGraph_t tmp;
        const cudaError_t e2 = cudaStreamEndCapture(s, &tmp);
        if (e == cudaSuccess) e = e1;
        if (e == cudaSuccess) e = e2;
      }
      if (with_update && e == cudaSuccess && st == MFE_OK) {
        alignas(cudaGraphNodeParams) unsigned char up_buf[sizeof(cudaGraphNodeParams)];
        memset(up_buf, 0, sizeof(up_buf));
        cudaGraphNodeParams* up = reinterpret_cast<cudaGraphNodeParams*>(up_buf);
        up->type = cudaGraphNodeTypeConditional;
        up->conditional.handle = hu;
        up->conditional.type = cudaGraphCondTypeIf;
        up->conditional.size = 1;
        cudaGraphNode_t unode;
        e = cudaGraphAddNode(&unode, body_graph, leaf, nullptr, nleaf, up);
        if (e == cudaSuccess) {
          e = cudaStreamBeginCaptureToGraph(s, up->conditional.phGraph_out[0], nullptr, nullptr, 0,
                                            cudaStreamCaptureModeRelaxed);
          if (e == cudaSuccess) {
            st = update(h, 1);
            cudaGraph_t tmp;
            const cudaError_t e2 = cudaStreamEndCapture(s, &tmp);
            if (e == cudaSuccess) e = e2;
          }
        }
      }
    }
    ctx->stream = run_stream;
    if (e == cudaSuccess && st == MFE_OK) e = cudaGraphInstantiate(&ex, g, 0);
    if (e == cudaSuccess && st == MFE_OK) e = cudaGraphLaunch(ex, ctx->stream);
  }
  if (ex) cudaGraphExecDestroy(ex);
  if (g) cudaGraphDestroy(g);
  if (st != MFE_OK) return st;
  if (e != cudaSuccess) return cuda_fail(ctx, e, "multi-RHS CG graph");
  return MFE_OK;
}

}  // namespace

bool spmm_box_eligible(const mfe_csr* A, int nrhs, const void* X, const void* Y)
{
  return csr_is_box(A) && nrhs >= 1 && nrhs <= kMaxRhs && (32 % nrhs) == 0 &&
         !((uintptr_t)A->vals & 15u) && !((uintptr_t)X & 15u) && !((uintptr_t)Y & 15u);
}

mfe_status launch_spmm_box(mfe_ctx* ctx, const mfe_csr* A, int nrhs, const void* X, void* Y)
{
  unsigned* err = static_cast<unsigned*>(workspace(ctx, "spmv.err", sizeof(unsigned)));
  if (!err) return fail(ctx, MFE_OOM, "workspace allocation failed");
  if (A->dtype == MFE_F64)
    return launch_spmm_t<double, MM_PLAIN, double>(ctx, A, nrhs, static_cast<const double*>(X),
                                                   static_cast<double*>(Y), nullptr, nullptr,
                                                   nullptr, nullptr, nullptr, nullptr, err);
  return launch_spmm_t<float, MM_PLAIN, float>(ctx, A, nrhs, static_cast<const float*>(X),
                                               static_cast<float*>(Y), nullptr, nullptr, nullptr,
                                               nullptr, nullptr, nullptr, err);
}

mfe_status cg_multi(mfe_ctx* ctx, const mfe_csr* A64_in, int nrhs, const double* B, double* X,
                    const mfe_cg_opts* o, mfe_cg_result* results)
{
  if (nrhs < 1 || nrhs > kMaxRhs || (32 % nrhs) != 0)
    return fail(ctx, MFE_BAD_ARG, "nrhs must divide 32 (1, 2, 4, 8, 16 or 32)");
  if (o->precision != MFE_PREC_MIXED && o->precision != MFE_PREC_F64)
    return fail(ctx, MFE_BAD_ARG, "unknown precision");
  if (o->precision == MFE_PREC_MIXED && !mixed_opts_valid(o)) return fail(ctx, MFE_BAD_ARG, "inner_tol must lie in [0, 1) and max_refine must be >= 0");
  if (A64_in->dtype != MFE_F64) return fail(ctx, MFE_BAD_ARG, "A must be FP64");
  mfe_csr A64 = *A64_in;
  if (!csr_is_box(&A64)) {
    int bx, by, bz;
    MFE_TRY(detect_box(ctx, &A64, &bx, &by, &bz));
    A64.box_nx = bx;
    A64.box_ny = by;
    A64.box_nz = bz;
  }
  if (!csr_is_box(&A64))
    return fail(ctx, MFE_NOT_SUPPORTED, "multi-RHS CG needs a box-structured matrix");
  if (((uintptr_t)A64.vals & 15u) || ((uintptr_t)X & 15u) || ((uintptr_t)B & 15u))
    return fail(ctx, MFE_BAD_ARG, "matrix values, B and X must be 16-byte aligned");
  const bool mixed = o->precision == MFE_PREC_MIXED;
  const int64_t ntot = A64.nrows * nrhs;

  // mixed with 32 right-hand sides: the padded-values SpMM, which reads p
  // with ghost zones of zero rows on both sides (the stencil's reach plus a
  // partial tile).  The FP32 operator (padded or CSR values) is rebuilt on
  // every call: a cache keyed on the values pointer would go stale when an
  // allocator hands the same address to another matrix.
  // mixed with 32 right-hand sides on a verified mirror-symmetric FP32
  // stencil (every miniFE box with k = 1): the stencil SpMM, no FP32 matrix
  bool use_st32 = false;
  float coef32[28] = {}, w8[8] = {};
  if (mixed && nrhs == 32 && o->mixed_operator == 0 && getenv("MFE_MULTI_CSR") == nullptr) {
    MFE_TRY(stencil_prepare(ctx, &A64, coef32, &use_st32));
    use_st32 = use_st32 && stencil_mirror_classes(coef32, w8);
  }
  const bool use_ell = mixed && nrhs == 32 && !use_st32 && getenv("MFE_MULTI_CSR") == nullptr;
  mfe_csr A32 = A64;
  if (mixed && !use_ell) {
    float* v32 = static_cast<float*>(
        workspace(ctx, "mixed.vals32", sizeof(float) * (size_t)(A64.nnz + 4)));
    if (!v32) return fail(ctx, MFE_OOM, "FP32 matrix copy allocation failed");
    MFE_TRY(launch_convert_f32(ctx, static_cast<const double*>(A64.vals), v32, A64.nnz));
    A32.vals = v32;
    A32.dtype = MFE_F32;
  } else if (mixed) {
    A32.vals = nullptr;
    A32.dtype = MFE_F32;
  }
  int st32_grid = 0;
  const int st32_zc = ctx->multi_zchunk > 0 ? ctx->multi_zchunk : kSMZC;
  if (use_st32) {
    const int64_t items = ceil_div((int64_t)(A64.box_nx + 1) * (A64.box_ny + 1), (int64_t)kSMKP) *
                          ceil_div((int64_t)(A64.box_nz + 1), (int64_t)st32_zc);
    st32_grid = (int)std::max<int64_t>(
        1, std::min<int64_t>({ceil_div(items, (int64_t)kSMW),
                              (int64_t)resident_blocks(ctx, (const void*)k_spmm_st32, kSMW * 32, 0),
                              (int64_t)kMaxPartM}));
  }
  const size_t vb = (mixed ? sizeof(float) : sizeof(double)) * (size_t)(ntot + 8);
  void* r = workspace(ctx, "multi.r", vb);
  const int64_t Nx = A64.box_nx + 1, NxNy = Nx * (A64.box_ny + 1);
  const int64_t ghost = NxNy + Nx + 1 + kER;
  const size_t pb = use_ell ? sizeof(float) * (size_t)((A64.nrows + 2 * ghost) * 32 + 8) : vb;
  void* pbase = workspace(ctx, use_ell ? "multi.pg" : "multi.p", pb);
  void* p = use_ell && pbase ? static_cast<void*>(static_cast<float*>(pbase) + ghost * 32) : pbase;
  float* ell = nullptr;
  int ell_grid = 0;
  if (use_ell) {
    const int64_t ntl = (A64.nrows + kER - 1) / kER;
    const size_t eb = sizeof(float) * (size_t)(ntl * kER * 28 + 8);
    ell = static_cast<float*>(workspace(ctx, "multi.ell28", eb));
    if (!ell) return fail(ctx, MFE_OOM, "padded FP32 matrix allocation failed");
    MFE_CUDA_TRY(ctx, cudaMemsetAsync(ell, 0, eb, ctx->stream));
    k_mr_ell28<<<(unsigned)std::max<int64_t>(1, std::min<int64_t>(ceil_div(A64.nrows, (int64_t)256),
                                                                  (int64_t)ctx->sm_count * 8)),
                 256, 0, ctx->stream>>>((int)Nx, A64.box_ny + 1, A64.box_nz + 1,
                                        static_cast<const double*>(A64.vals), ell);
    MFE_TRY(check_launch(ctx, "k_mr_ell28"));
    MFE_TRY(ell32_grid(ctx, &ell_grid));
  }
  void* Ap = workspace(ctx, "multi.Ap", vb);
  float* x32 = mixed ? static_cast<float*>(workspace(ctx, "multi.x32", vb)) : nullptr;
  MultiState* dst = static_cast<MultiState*>(workspace(ctx, "multi.state", sizeof(MultiState)));
  double* partials =
      static_cast<double*>(workspace(ctx, "multi.partials", sizeof(double) * 2 * kMaxPartM * 32));
  const bool fresh = ctx->ws.find("multi.tickets") == ctx->ws.end();
  unsigned* tickets = static_cast<unsigned*>(workspace(ctx, "multi.tickets", sizeof(unsigned) * 4));
  unsigned* err = static_cast<unsigned*>(workspace(ctx, "multi.err", sizeof(unsigned)));
  if (!r || !pbase || !Ap || (mixed && !x32) || !dst || !partials || !tickets || !err)
    return fail(ctx, MFE_OOM, "multi-RHS workspace allocation failed");
  if (fresh) MFE_CUDA_TRY(ctx, cudaMemsetAsync(tickets, 0, sizeof(unsigned) * 4, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(err, 0, sizeof(unsigned), ctx->stream));

  MultiState* hs = static_cast<MultiState*>(host_scratch(ctx, sizeof(MultiState) + 64));
  if (!hs) return fail(ctx, MFE_OOM, "pinned scratch allocation failed");
  memset(hs, 0, sizeof(MultiState));
  hs->nrhs = nrhs;
  hs->max_iter = std::max(0, o->max_iter);
  hs->refine_k = o->refine_k > 0 ? o->refine_k : 50;
  hs->delta2 = mixed_delta2(o);
  hs->max_refine = o->max_refine;
  hs->first = 1;
  hs->tol_mode = o->tol_mode == MFE_TOL_RELATIVE ? 1 : 0;
  for (int j = 0; j < nrhs; ++j) hs->tol_abs[j] = o->tol;
  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev0, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(dst, hs, sizeof(MultiState), cudaMemcpyHostToDevice, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(pbase, 0, pb, ctx->stream));
  if (mixed) {
    MFE_CUDA_TRY(ctx, cudaMemsetAsync(x32, 0, vb, ctx->stream));
    MFE_TRY((launch_spmm_t<double, MM_RESID, float>(ctx, &A64, nrhs, X, nullptr, B,
                                                     static_cast<float*>(r), partials, tickets,
                                                     dst->rr_true, nullptr, err)));
  } else {
    MFE_TRY((launch_spmm_t<double, MM_RESID, double>(ctx, &A64, nrhs, X, nullptr, B,
                                                      static_cast<double*>(r), partials, tickets,
                                                      dst->rr_true, nullptr, err)));
  }
  k_mr_init<<<1, 32, 0, ctx->stream>>>(dst);
  MFE_TRY(check_launch(ctx, "k_mr_init"));

  // kernel attributes and occupancy are set up before the loop is captured
  if (mixed) {
    vgrid(ctx, ntot, k_mr_p<float>);
    vgrid(ctx, ntot, k_mr_update<float>);
    vgrid(ctx, ntot, k_mr_xupdate);
  } else {
    vgrid(ctx, ntot, k_mr_p<double>);
    vgrid(ctx, ntot, k_mr_update<double>);
  }
  if (mixed) {
    MFE_TRY((spmm_setup<float, MM_DOT, float>(ctx, nrhs, nullptr)));
  } else {
    MFE_TRY((spmm_setup<double, MM_DOT, double>(ctx, nrhs, nullptr)));
  }
  if (mixed) {
    MultiBufs<float> W{static_cast<float*>(r), static_cast<float*>(p), static_cast<float*>(Ap),
                       x32, dst, partials, tickets, err, ell, ell_grid};
    if (use_st32) {
      W.st32 = true;
      for (int c = 0; c < 8; ++c) W.w8[c] = w8[c];
      W.dd = coef32[27];
      W.st32_grid = st32_grid;
      W.st32_zc = st32_zc;
    }
    MFE_TRY(run_loop(
        ctx, dst, hs,
        [&](cudaGraphConditionalHandle h, cudaGraphConditionalHandle hu, int in_graph) {
          return multi_iter_mixed(ctx, A32, A64, nrhs, W, h, hu, in_graph);
        },
        [&](cudaGraphConditionalHandle h, int in_graph) {
          return multi_update_mixed(ctx, A64, nrhs, B, X, W, h, in_graph);
        },
        true));
  } else {
    MultiBufs<double> W{static_cast<double*>(r), static_cast<double*>(p),
                        static_cast<double*>(Ap), nullptr, dst, partials, tickets, err};
    MFE_TRY(run_loop(
        ctx, dst, hs,
        [&](cudaGraphConditionalHandle h, cudaGraphConditionalHandle, int in_graph) {
          return multi_iter_f64(ctx, A64, nrhs, X, W, h, in_graph);
        },
        [&](cudaGraphConditionalHandle, int) { return MFE_OK; }, false));
  }
  unsigned* herr = reinterpret_cast<unsigned*>(reinterpret_cast<unsigned char*>(hs) + sizeof(MultiState));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(hs, dst, sizeof(MultiState), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(herr, err, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaEventRecord(ctx->ev1, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaEventSynchronize(ctx->ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  if (*herr) return fail(ctx, MFE_TIMEOUT, "a bounded device wait gave up during multi-RHS CG");
  mfe_status worst = MFE_OK;
  for (int j = 0; j < nrhs; ++j) {
    mfe_cg_result& res = results[j];
    memset(&res, 0, sizeof(res));
    res.num_iters = hs->done[j] ? hs->iters[j] : hs->k;
    res.normr = hs->normr_true[j];
    res.normr0 = hs->normr0[j];
    res.final_resid = hs->normr_true[j];
    res.times[4] = ms * 1e-3;
    res.refinements = hs->updates;
    res.fp64_spmvs = mixed ? hs->updates + 1 : hs->k + 1;
    res.inner_operator = !mixed ? MFE_INNER_NONE
                                : (use_st32 ? MFE_INNER_STENCIL : (ell ? MFE_INNER_PADDED : MFE_INNER_VALUES));
    const bool converged = mixed ? hs->done[j] != 0 && !hs->brk[j]
                                 : !(hs->normr_true[j] > hs->tol_abs[j]);
    res.status = hs->brk[j] ? MFE_BREAKDOWN : (converged ? MFE_OK : MFE_MAXITER);
    if (res.status != MFE_OK && worst == MFE_OK) worst = (mfe_status)res.status;
  }
  return worst;
}

}  // namespace mfe
