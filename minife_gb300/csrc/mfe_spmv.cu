// CSR matrix-vector products on sm_103a.
//
// GB300 has a reduced FP64 pipe (about 2 FP64 FMA per clock per SM), which
// puts an FP64 CSR SpMV close to the FP64 issue limit as well as the HBM
// limit.  The main kernel therefore spends exactly one FP64 FMA per nonzero:
// one thread owns one row and accumulates it sequentially (no shuffle-add
// trees, which would cost 5 extra FP64 adds per lane), while the row's values
// and column indices arrive through shared memory so the HBM reads stay fully
// coalesced:
//   - a persistent grid walks tiles of ROWS consecutive rows; the nonzeros of
//     a tile are contiguous in CSR, so one thread issues two 1-D bulk async
//     copies (TMA, cp.async.bulk) for the tile's values and columns into a
//     shared-memory stage, completion tracked by an mbarrier;
//   - S stages are in flight per CTA, so the copies for the next tiles
//     overlap the current tile's FMAs;
//   - x is gathered through the read-only path (27-point rows touch three
//     x-planes, which stay L1/L2 resident).
// Two forms of that scheme: FP64 rows go through the warp-staged kernel (a
// warp per 32-row group with its own ring of stages and mbarriers, no block
// barrier), FP32 rows through the tiled kernel (a block per 128-row tile).
// The reference's row-major ELLMatrix has its own warp-staged kernel, whose
// groups start aligned.
// Epilogues: plain y = A x; y = A x with x.y (matvec_and_dot); and the CG
// residual r = b - A x with r.r.  Dots accumulate in FP64 and reduce
// deterministically (fixed grid, last block sums the block partials in order).
// Matrices with rows longer than 32 entries use a warp-per-row kernel.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "mfe_cgstate.cuh"
#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

constexpr int kMaxTileRowLen = 32;

static bool aligned16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

enum SpmvMode { SPMV_PLAIN = 0, SPMV_DOT = 1, SPMV_RESID = 2 };

template <typename T>
struct SpmvParams {
  int64_t n;
  int64_t nnz;
  const int32_t* __restrict__ ro;
  const int32_t* __restrict__ cols;
  const T* __restrict__ vals;
  const T* __restrict__ x;
  T* __restrict__ y;
  const double* __restrict__ b;  // SPMV_RESID: y = b - A x
  int cap;                       // elements per stage (multiple of 4)
  double* partials;
  unsigned* ticket;
  double* dot_out;  // used when cg == nullptr
  CgState* cg;      // CG bookkeeping in the last block (nullable)
  unsigned* err;
  // fault injection (mfe_inject_wait_timeout), warp-staged kernels: nonzero =
  // no copy is issued and the bounded waits give up after this many ns
  uint64_t withhold_ns;
};

// Row sum with one FMA per nonzero.  Rows of up to LMAX entries run the same
// fully unrolled, predicated code (no divergence between the 27-entry
// interior rows and the 8/12/18-entry boundary rows of a warp), and two
// interleaved partial sums (even / odd entries) halve the dependent-FMA
// chain, which the FP64 pipe's long latency otherwise exposes; one extra add
// joins them.  Longer rows continue in a plain loop.
//
// All LMAX column/value/x loads are issued unconditionally before the first
// FMA (indices past the row end are clamped to its last entry, so every load
// stays inside the row), letting the 27 x-gathers overlap; the FMAs past the
// row end are discarded by a select, so the sum is exactly that of the row's
// own entries.
// Read-only-path gathers written as volatile asm: the compiler treats
// __ldg results as rematerialisable and sinks each gather next to its FMA,
// which serialises the gathers' latency; volatile loads stay where they are
// issued, so all of a row's gathers are in flight together.
__device__ __forceinline__ double ld_gather(const double* p)
{
  double v;
  asm volatile("ld.global.nc.f64 %0, [%1];" : "=d"(v) : "l"(p));
  return v;
}
__device__ __forceinline__ float ld_gather(const float* p)
{
  float v;
  asm volatile("ld.global.nc.f32 %0, [%1];" : "=f"(v) : "l"(p));
  return v;
}

template <typename T, int LMAX>
__device__ __forceinline__ T row_dot(const T* __restrict__ rv, const int32_t* __restrict__ rc,
                                     int len, const T* __restrict__ x)
{
  if (len <= 0) return T(0);
  int32_t c[LMAX];
  T xv[LMAX], v[LMAX];
#pragma unroll
  for (int k = 0; k < LMAX; ++k) c[k] = rc[min(k, len - 1)];
#pragma unroll
  for (int k = 0; k < LMAX; ++k) xv[k] = ld_gather(&x[c[k]]);
#pragma unroll
  for (int k = 0; k < LMAX; ++k) v[k] = rv[min(k, len - 1)];
  T s0 = T(0), s1 = T(0);
#pragma unroll
  for (int k = 0; k < LMAX; k += 2) {
    const T t0 = fma(v[k], xv[k], s0);
    s0 = (k < len) ? t0 : s0;
    if (k + 1 < LMAX) {
      const T t1 = fma(v[k + 1], xv[k + 1], s1);
      s1 = (k + 1 < len) ? t1 : s1;
    }
  }
  for (int k = LMAX; k < len; ++k) s0 = fma(rv[k], __ldg(&x[rc[k]]), s0);
  return s0 + s1;
}

template <int MODE>
__device__ __forceinline__ void spmv_epilogue(double total, CgState* cg, double* dot_out)
{
  if (cg == nullptr) {
    if (MODE != SPMV_PLAIN) *dot_out = total;
    return;
  }
  if (MODE == SPMV_DOT) {
    // cg_solve.hpp:179-200: p.Ap and the breakdown pre-test
    cg->pAp = total;
    if (total < cg->brkdown_tol) cg->check_pending = 1;
  } else if (MODE == SPMV_RESID) {
    // cg_solve.hpp:124-144: r = b - A x, rtrans, normr, loop condition
    cg_resid_init(cg, total);
  }
}

// A minimum of two blocks per SM in the launch bounds (shared memory allows
// three or four) lets ptxas keep a row's gathers in flight at 96 registers
// instead of 32-40: the 256^3 FP32 product 0.638 against 0.714 ms
template <typename T, int ROWS, int S, int MODE>
__global__ void __launch_bounds__(ROWS, 2) k_spmv_tiled(SpmvParams<T> P)
{
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar[S];
  __shared__ int64_t s_base_v[S], s_base_c[S];
  __shared__ double red[32];
  constexpr int VA = 16 / sizeof(T);  // values per 16 bytes
  T* sv = reinterpret_cast<T*>(smem);
  int32_t* sc = reinterpret_cast<int32_t*>(smem + (size_t)S * P.cap * sizeof(T));

  const int tid = threadIdx.x;
  const int64_t ntiles = (P.n + ROWS - 1) / ROWS;
  if (tid == 0) {
    for (int s = 0; s < S; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // producer (thread 0): stage nonzeros [a, e) of one tile into stage s
  auto issue = [&](int64_t a, int64_t e, int s) {
    const int64_t av = a & ~(int64_t)(VA - 1);
    const int64_t ac = a & ~(int64_t)3;
    int64_t bv = min((e + VA - 1) & ~(int64_t)(VA - 1), P.nnz & ~(int64_t)(VA - 1));
    int64_t bc = min((e + 3) & ~(int64_t)3, P.nnz & ~(int64_t)3);
    if (bv < av) bv = av;
    if (bc < ac) bc = ac;
    if (max(bv, e) - av > P.cap || max(bc, e) - ac > P.cap) {
      // cannot happen when every row has <= max_len nonzeros (the host sizes
      // cap from max_len); record it and stage nothing
      atomicOr(P.err, ERR_TILE_OVERFLOW);
      s_base_v[s] = a;
      s_base_c[s] = a;
      mbar_arrive_expect_tx(&bar[s], 0);
      return;
    }
    s_base_v[s] = av;
    s_base_c[s] = ac;
    T* dv = sv + (size_t)s * P.cap;
    int32_t* dc = sc + (size_t)s * P.cap;
    // ragged tail past the last 16-byte boundary of the arrays: plain loads
    for (int64_t k = bv; k < e; ++k) dv[k - av] = P.vals[k];
    for (int64_t k = bc; k < e; ++k) dc[k - ac] = P.cols[k];
    fence_proxy_async_smem();
    const unsigned bytes_v = (unsigned)((bv - av) * sizeof(T));
    const unsigned bytes_c = (unsigned)((bc - ac) * sizeof(int32_t));
    mbar_arrive_expect_tx(&bar[s], bytes_v + bytes_c);
    if (bytes_v) bulk_g2s(dv, P.vals + av, bytes_v, &bar[s]);
    if (bytes_c) bulk_g2s(dc, P.cols + ac, bytes_c, &bar[s]);
  };
  auto tile_bounds = [&](int64_t t, int64_t& a, int64_t& e) {
    a = __ldg(&P.ro[t * ROWS]);
    e = __ldg(&P.ro[min(P.n, t * ROWS + ROWS)]);
  };

  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      const int64_t t = blockIdx.x + (int64_t)s * gridDim.x;
      if (t < ntiles) {
        int64_t a, e;
        tile_bounds(t, a, e);
        issue(a, e, s);
      }
    }
  }

  double dacc = 0.0;
  int it = 0;
  int64_t tile = blockIdx.x;
  // row offsets of this thread's row in the current tile (prefetched)
  int32_t ra = 0, rb = 0;
  {
    const int64_t r = tile * ROWS + tid;
    if (tile < ntiles && r < P.n) {
      ra = __ldg(&P.ro[r]);
      rb = __ldg(&P.ro[r + 1]);
    }
  }
  bool ok = true;
  for (; tile < ntiles; tile += gridDim.x, ++it) {
    const int s = it % S;
    const unsigned parity = (unsigned)((it / S) & 1);
    // prefetch the next tile's row offsets into registers
    const int64_t ntile = tile + gridDim.x;
    const int64_t nr = ntile * ROWS + tid;
    int32_t na = 0, nb = 0;
    if (ntile < ntiles && nr < P.n) {
      na = __ldg(&P.ro[nr]);
      nb = __ldg(&P.ro[nr + 1]);
    }
    // thread 0: bounds of the tile it will stage into s after this one
    const int64_t itile = tile + (int64_t)S * gridDim.x;
    int64_t ia = 0, ie = 0;
    if (tid == 0 && itile < ntiles) tile_bounds(itile, ia, ie);
    ok = mbar_wait_bounded(&bar[s], parity);
    ok = __syncthreads_and(ok);
    if (!ok) break;
    const int64_t r = tile * ROWS + tid;
    if (r < P.n) {
      const int len = rb - ra;
      const T* rv = sv + (size_t)s * P.cap + (ra - s_base_v[s]);
      const int32_t* rc = sc + (size_t)s * P.cap + (ra - s_base_c[s]);
      const T sum = row_dot<T, 27>(rv, rc, len, P.x);
      if (MODE == SPMV_RESID) {
        const double rr = P.b[r] - (double)sum;
        P.y[r] = (T)rr;
        dacc = fma(rr, rr, dacc);
      } else {
        P.y[r] = sum;
        if (MODE == SPMV_DOT) dacc = fma((double)sum, (double)__ldg(&P.x[r]), dacc);
      }
    }
    ra = na;
    rb = nb;
    __syncthreads();  // every thread is done reading stage s
    if (tid == 0 && itile < ntiles) issue(ia, ie, s);
  }
  if (!ok) {
    if (tid == 0) {
      atomicOr(P.err, ERR_WAIT_TIMEOUT);
      // drain: give every stage that may still have copies in flight a
      // bounded chance to complete before the block exits
      for (int s = 0; s < S; ++s) {
        const int j = it + s;
        mbar_wait_bounded(&bar[j % S], (unsigned)((j / S) & 1));
      }
    }
    return;
  }
  if (MODE != SPMV_PLAIN) {
    const double bt = block_sum(dacc, red);
    double total;
    if (grid_reduce_last(bt, P.partials, P.ticket, red, &total) && tid == 0)
      spmv_epilogue<MODE>(total, P.cg, P.dot_out);
  }
}

// Warp-staged products: a warp per group of 32 rows, whose nonzeros are
// contiguous in both layouts below (CSR: ro[32g] .. ro[32g+32]; the
// reference's ELLMatrix: 32 g K .. 32 (g+1) K, short rows padded).  Lane 0
// stages a group's values and columns with two 1-D bulk copies (TMA) into the
// warp's own ring of kStgStages shared-memory stages, each with its mbarrier
// (no block barrier in the loop), and every lane sums its own row from shared
// memory with row_dot.  With rows of 27 entries an FP64 stage is 10.5 KB and
// ten warps per SM each keep their next group in flight, where the tiled
// kernel's 128-row tiles hold two blocks per SM behind block barriers: the
// 256^3 FP64 product takes 1.14 ms against 2.09 ms through the tiled kernel
// (FP32 rows, half the bytes per stage, stay on the tiled kernel: 0.638
// ms, where the staged form took 0.75-0.80 ms before either kernel stated
// its blocks per SM).
constexpr int kStgWarps = 2;    // warps per block
constexpr int kStgStages = 2;   // stages per warp
constexpr int kStgMaxLen = 32;  // longer rows: the warp-per-row kernel

// Stage capacity (elements) for a group of 32 rows of at most max_len
// entries: ELL groups start aligned and hold exactly 32 K; CSR groups carry
// up to 3 elements of alignment slack at each end.  A multiple of 4, so the
// column part of a stage starts 16-byte aligned.
__host__ __device__ constexpr int stg_cap(int max_len, bool ell)
{
  return ell ? 32 * max_len : ((32 * max_len + 8) + 3) & ~3;
}

// CSR rows of at most max_len entries.  A stage starts on the 16-byte
// boundaries at or below its group's first nonzero, and the ragged end of
// the arrays arrives by plain loads, as in the tiled kernel.
// Five blocks per SM is the occupancy shared memory allows for 27-entry rows;
// stating it (any minimum does) lets ptxas keep a row's gathers in flight at
// 72 registers instead of 40: 1.14-1.16 against 1.40 ms for the 256^3 product
template <typename T, int MODE>
__global__ void __launch_bounds__(kStgWarps * 32, 5) k_spmv_staged(SpmvParams<T> P, int max_len)
{
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar[kStgWarps][kStgStages];
  __shared__ double red[32];
  constexpr int VA = 16 / sizeof(T);  // values per 16 bytes
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const int cap = stg_cap(max_len, false);
  const size_t vbytes = (size_t)cap * sizeof(T);
  const size_t sbytes = vbytes + (size_t)cap * sizeof(int32_t);
  unsigned char* wbase = smem + (size_t)w * kStgStages * sbytes;
  const int64_t ngroups = (P.n + 31) / 32;
  const int64_t nw = (int64_t)gridDim.x * kStgWarps;
  const int64_t g0 = (int64_t)blockIdx.x * kStgWarps + w;
  if (lane == 0) {
    for (int s = 0; s < kStgStages; ++s) mbar_init(&bar[w][s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // lane 0: nonzeros [a, e) of one group into stage s
  auto issue = [&](int64_t a, int64_t e, int s) {
    const int64_t av = a & ~(int64_t)(VA - 1);
    const int64_t ac = a & ~(int64_t)3;
    int64_t bv = min((e + VA - 1) & ~(int64_t)(VA - 1), P.nnz & ~(int64_t)(VA - 1));
    int64_t bc = min((e + 3) & ~(int64_t)3, P.nnz & ~(int64_t)3);
    if (bv < av) bv = av;
    if (bc < ac) bc = ac;
    if (max(bv, e) - av > cap || max(bc, e) - ac > cap) {
      // cannot happen when every row has <= the max_len the host passed;
      // record it and stage nothing
      atomicOr(P.err, ERR_TILE_OVERFLOW);
      mbar_arrive_expect_tx(&bar[w][s], 0);
      return;
    }
    T* dv = reinterpret_cast<T*>(wbase + (size_t)s * sbytes);
    int32_t* dc = reinterpret_cast<int32_t*>(wbase + (size_t)s * sbytes + vbytes);
    // ragged tail past the last 16-byte boundary of the arrays: plain loads
    for (int64_t k = bv; k < e; ++k) dv[k - av] = P.vals[k];
    for (int64_t k = bc; k < e; ++k) dc[k - ac] = P.cols[k];
    fence_proxy_async_smem();
    const unsigned bytes_v = (unsigned)((bv - av) * sizeof(T));
    const unsigned bytes_c = (unsigned)((bc - ac) * sizeof(int32_t));
    mbar_arrive_expect_tx(&bar[w][s], bytes_v + bytes_c);
    if (bytes_v) bulk_g2s(dv, P.vals + av, bytes_v, &bar[w][s]);
    if (bytes_c) bulk_g2s(dc, P.cols + ac, bytes_c, &bar[w][s]);
  };

  if (lane == 0 && P.withhold_ns == 0)
    for (int s = 0; s < kStgStages; ++s) {
      const int64_t g = g0 + (int64_t)s * nw;
      if (g < ngroups) issue(__ldg(&P.ro[g * 32]), __ldg(&P.ro[min(P.n, g * 32 + 32)]), s);
    }
  const uint64_t wait_ns = P.withhold_ns ? P.withhold_ns : kWaitLimitNs;
  double dacc = 0.0;
  bool ok = true;
  int it = 0;
  for (int64_t g = g0; g < ngroups; g += nw, ++it) {
    const int s = it % kStgStages;
    const int64_t r = g * 32 + lane;
    const int64_t gn = g + (int64_t)kStgStages * nw;  // the group stage s takes next
    // the group's and this lane's row bounds, and lane 0's bounds of the
    // next group, loaded before the wait so their latency overlaps it (the
    // next copy then starts as soon as the lanes are done)
    const int32_t a = __ldg(&P.ro[g * 32]);
    int32_t ra = 0, rb = 0;
    if (r < P.n) {
      ra = __ldg(&P.ro[r]);
      rb = __ldg(&P.ro[r + 1]);
    }
    int64_t na = 0, ne = 0;
    if (lane == 0 && gn < ngroups) {
      na = __ldg(&P.ro[gn * 32]);
      ne = __ldg(&P.ro[min(P.n, gn * 32 + 32)]);
    }
    ok = __all_sync(0xffffffffu, mbar_wait_bounded(&bar[w][s], (unsigned)((it / kStgStages) & 1), wait_ns));
    if (!ok) break;
    if (r < P.n) {
      const T* rv = reinterpret_cast<const T*>(wbase + (size_t)s * sbytes) + (ra - (a & ~(VA - 1)));
      const int32_t* rc =
          reinterpret_cast<const int32_t*>(wbase + (size_t)s * sbytes + vbytes) + (ra - (a & ~3));
      const T sum = row_dot<T, 27>(rv, rc, rb - ra, P.x);
      if (MODE == SPMV_RESID) {
        const double rr = P.b[r] - (double)sum;
        P.y[r] = (T)rr;
        dacc = fma(rr, rr, dacc);
      } else {
        P.y[r] = sum;
        if (MODE == SPMV_DOT) dacc = fma((double)sum, (double)__ldg(&P.x[r]), dacc);
      }
    }
    __syncwarp();  // every lane is done reading stage s
    if (lane == 0 && gn < ngroups) issue(na, ne, s);
  }
  if (!ok) {
    if (lane == 0) {
      atomicOr(P.err, ERR_WAIT_TIMEOUT);
      // drain: give each stage with a copy issued a bounded chance to land
      // before the block exits (an injected fault issued none)
      for (int j = it; j < it + kStgStages; ++j)
        if (P.withhold_ns == 0 && g0 + (int64_t)j * nw < ngroups)
          mbar_wait_bounded(&bar[w][j % kStgStages], (unsigned)((j / kStgStages) & 1));
    }
    __syncwarp();
  }
  // every warp reaches the block reduction, also after a timeout
  if (MODE != SPMV_PLAIN) {
    const double bt = block_sum(dacc, red);
    double total;
    if (grid_reduce_last(bt, P.partials, P.ticket, red, &total) && threadIdx.x == 0)
      spmv_epilogue<MODE>(total, P.cg, P.dot_out);
  }
}

// The reference's row-major ELL, K entries per row (K <= kStgMaxLen): group
// g's entries start at 32 g K, 16-byte aligned in both arrays, and row lane
// sits at lane K of its stage.  The stage size is computed from K here (not
// read from the parameter block), which lets the compiler fold each lane's
// stage addresses and keep a row's loads in flight together: 1.04 ms for the
// 256^3 product against 1.13 ms with the size read from P.  MODE: plain or
// the CG's initial residual.
// FP32 rows also name the five blocks per SM in the launch bounds (122
// registers: 0.579 against 0.595 ms at 256^3); FP64 rows name none (96
// registers; five blocks: 104 registers and 1.058 against 1.040 ms)
template <typename T>
constexpr int ell_min_blocks()
{
  return sizeof(T) == 4 ? 5 : 0;
}

template <typename T, int MODE>
__global__ void __launch_bounds__(kStgWarps * 32, ell_min_blocks<T>()) k_spmv_ell(SpmvParams<T> P, int K)
{
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t bar[kStgWarps][kStgStages];
  __shared__ double red[32];
  constexpr int VA = 16 / sizeof(T);
  const int lane = threadIdx.x & 31;
  const int w = threadIdx.x >> 5;
  const size_t sbytes = (size_t)32 * K * (sizeof(T) + sizeof(int32_t));
  const size_t vbytes = (size_t)32 * K * sizeof(T);
  unsigned char* wbase = smem + (size_t)w * kStgStages * sbytes;
  const int64_t ngroups = (P.n + 31) / 32;
  const int64_t nw = (int64_t)gridDim.x * kStgWarps;
  const int64_t g0 = (int64_t)blockIdx.x * kStgWarps + w;
  if (lane == 0) {
    for (int s = 0; s < kStgStages; ++s) mbar_init(&bar[w][s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // lane 0: group g into stage s; the ragged end past the last 16-byte
  // boundary of the matrix (last group only) by plain loads
  auto issue = [&](int64_t g, int s) {
    const int64_t a = g * 32 * K;
    const int64_t e = min(P.n, g * 32 + 32) * K;
    const int64_t bv = max(a, e & ~(int64_t)(VA - 1));
    const int64_t bc = max(a, e & ~(int64_t)3);
    T* dv = reinterpret_cast<T*>(wbase + (size_t)s * sbytes);
    int32_t* dc = reinterpret_cast<int32_t*>(wbase + (size_t)s * sbytes + vbytes);
    for (int64_t k = bv; k < e; ++k) dv[k - a] = P.vals[k];
    for (int64_t k = bc; k < e; ++k) dc[k - a] = P.cols[k];
    fence_proxy_async_smem();
    const unsigned bytes_v = (unsigned)((bv - a) * sizeof(T));
    const unsigned bytes_c = (unsigned)((bc - a) * sizeof(int32_t));
    mbar_arrive_expect_tx(&bar[w][s], bytes_v + bytes_c);
    if (bytes_v) bulk_g2s(dv, P.vals + a, bytes_v, &bar[w][s]);
    if (bytes_c) bulk_g2s(dc, P.cols + a, bytes_c, &bar[w][s]);
  };
  if (lane == 0 && P.withhold_ns == 0)
    for (int s = 0; s < kStgStages; ++s) {
      const int64_t g = g0 + (int64_t)s * nw;
      if (g < ngroups) issue(g, s);
    }
  const uint64_t wait_ns = P.withhold_ns ? P.withhold_ns : kWaitLimitNs;
  double dacc = 0.0;
  bool ok = true;
  int it = 0;
  for (int64_t g = g0; g < ngroups; g += nw, ++it) {
    const int s = it % kStgStages;
    ok = __all_sync(0xffffffffu, mbar_wait_bounded(&bar[w][s], (unsigned)((it / kStgStages) & 1), wait_ns));
    if (!ok) break;
    const int64_t r = g * 32 + lane;
    if (r < P.n) {
      const T* rv = reinterpret_cast<const T*>(wbase + (size_t)s * sbytes) + (size_t)lane * K;
      const int32_t* rc =
          reinterpret_cast<const int32_t*>(wbase + (size_t)s * sbytes + vbytes) + (size_t)lane * K;
      const T sum = row_dot<T, 27>(rv, rc, K, P.x);
      if (MODE == SPMV_RESID) {
        const double rr = P.b[r] - (double)sum;
        P.y[r] = (T)rr;
        dacc = fma(rr, rr, dacc);
      } else {
        P.y[r] = sum;
      }
    }
    __syncwarp();  // every lane is done reading stage s
    const int64_t gn = g + (int64_t)kStgStages * nw;
    if (lane == 0 && gn < ngroups) issue(gn, s);
  }
  if (!ok) {
    if (lane == 0) {
      atomicOr(P.err, ERR_WAIT_TIMEOUT);
      for (int j = it; j < it + kStgStages; ++j)
        if (P.withhold_ns == 0 && g0 + (int64_t)j * nw < ngroups)
          mbar_wait_bounded(&bar[w][j % kStgStages], (unsigned)((j / kStgStages) & 1));
    }
    __syncwarp();
  }
  if (MODE == SPMV_RESID) {
    const double bt = block_sum(dacc, red);
    double total;
    if (grid_reduce_last(bt, P.partials, P.ticket, red, &total) && threadIdx.x == 0)
      spmv_epilogue<MODE>(total, P.cg, P.dot_out);
  }
}

// Warp-per-row fallback for long rows (shuffle-reduced).
template <typename T, int MODE>
__global__ void __launch_bounds__(256) k_spmv_warp(SpmvParams<T> P)
{
  __shared__ double red[32];
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double dacc = 0.0;
  for (int64_t r = warp; r < P.n; r += nwarps) {
    const int32_t a = P.ro[r], e = P.ro[r + 1];
    T sum = T(0);
    for (int32_t k = a + lane; k < e; k += 32) sum = fma(P.vals[k], __ldg(&P.x[P.cols[k]]), sum);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) {
      if (MODE == SPMV_RESID) {
        const double rr = P.b[r] - (double)sum;
        P.y[r] = (T)rr;
        dacc = fma(rr, rr, dacc);
      } else {
        P.y[r] = sum;
        if (MODE == SPMV_DOT) dacc = fma((double)sum, (double)P.x[r], dacc);
      }
    }
  }
  if (MODE != SPMV_PLAIN) {
    const double bt = block_sum(dacc, red);
    double total;
    if (grid_reduce_last(bt, P.partials, P.ticket, red, &total) && threadIdx.x == 0)
      spmv_epilogue<MODE>(total, P.cg, P.dot_out);
  }
}

__global__ void k_max_row_len(int64_t n, const int32_t* __restrict__ ro, int* out)
{
  int m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, ro[i + 1] - ro[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// ---------------------------------------------------------------------------
// multi-RHS: Y = A X, X and Y row-major with nrhs columns; one thread per
// (row, rhs) pair walks the row, so A is read once per product through L1.
// ---------------------------------------------------------------------------
template <typename T>
__global__ void __launch_bounds__(256)
    k_spmm(int64_t n, int nrhs, const int32_t* __restrict__ ro, const int32_t* __restrict__ cols,
           const T* __restrict__ vals, const T* __restrict__ X, T* __restrict__ Y)
{
  const int64_t total = n * nrhs;
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < total;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t r = t / nrhs;
    const int j = (int)(t - r * nrhs);
    const int32_t a = ro[r], e = ro[r + 1];
    T sum = T(0);
    for (int32_t k = a; k < e; ++k) sum = fma(vals[k], __ldg(&X[(int64_t)cols[k] * nrhs + j]), sum);
    Y[t] = sum;
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
constexpr int kStages = 2;

// Rows per tile (= threads per CTA): 128 by default; MFE_SPMV_ROWS selects
// 64 or 256 for launch-shape sweeps.
static int tile_rows()
{
  static int rows = 0;
  if (rows == 0) {
    rows = 128;
    if (const char* v = getenv("MFE_SPMV_ROWS")) {
      const int r = atoi(v);
      if (r == 64 || r == 128 || r == 256) rows = r;
    }
  }
  return rows;
}

// Stage capacity (elements) for rows of at most max_len nonzeros: the tile's
// nonzeros plus the 16-byte alignment slack at both ends, kept a multiple of 4
// so every stage starts 16-byte aligned.
static int tile_cap(int rows, int max_len)
{
  return ((rows * max_len + 8) + 3) & ~3;
}

template <typename T>
static size_t tiled_smem(int rows, int max_len)
{
  return (size_t)kStages * tile_cap(rows, max_len) * (sizeof(T) + sizeof(int32_t));
}

template <typename T, int ROWS, int MODE>
static cudaError_t configure_one()
{
  return cudaFuncSetAttribute(k_spmv_tiled<T, ROWS, kStages, MODE>,
                              cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)tiled_smem<T>(ROWS, kMaxTileRowLen));
}

template <int ROWS>
static cudaError_t configure_rows()
{
  cudaError_t e = configure_one<float, ROWS, SPMV_PLAIN>();
  if (e == cudaSuccess) e = configure_one<float, ROWS, SPMV_DOT>();
  return e;
}

// Shared-memory opt-in for every tiled instantiation, once per device (a
// function attribute, so it is set before any stream capture uses them).
static cudaError_t configure_tiled(int device)
{
  static bool done[64] = {};
  if (device >= 0 && device < 64 && done[device]) return cudaSuccess;
  cudaError_t e = configure_rows<64>();
  if (e == cudaSuccess) e = configure_rows<128>();
  if (e == cudaSuccess) e = configure_rows<256>();
  if (e == cudaSuccess && device >= 0 && device < 64) done[device] = true;
  return e;
}

// CTAs per SM for the tiled kernel (MFE_SPMV_CTAS_PER_SM overrides, for
// launch-shape sweeps); limited by shared memory.
static int tiled_ctas_per_sm(size_t smem)
{
  int per_sm = (int)((227 * 1024) / (smem + 1024));
  if (const char* v = getenv("MFE_SPMV_CTAS_PER_SM")) {
    const int o = atoi(v);
    if (o > 0 && o < per_sm) per_sm = o;
  }
  return std::max(1, per_sm);
}

// ---- warp-staged kernels ----
mfe_status take_wait_injection(mfe_ctx* ctx, uint64_t* withhold_ns)
{
  *withhold_ns = 0;
  if (!ctx->inject_wait_ns) return MFE_OK;
  // one-shot, and only for a launch that runs now (not one being captured
  // into a graph, which would replay it)
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  MFE_CUDA_TRY(ctx, cudaStreamIsCapturing(ctx->stream, &cs));
  if (cs == cudaStreamCaptureStatusNone) {
    *withhold_ns = ctx->inject_wait_ns;
    ctx->inject_wait_ns = 0;
  }
  return MFE_OK;
}

template <typename T>
static size_t staged_smem(int max_len, bool ell)
{
  return (size_t)kStgWarps * kStgStages * stg_cap(max_len, ell) * (sizeof(T) + sizeof(int32_t));
}

template <typename T>
static int staged_grid(mfe_ctx* ctx, int64_t nrows, int max_len, bool ell)
{
  const size_t smem = staged_smem<T>(max_len, ell);
  const int per_sm = std::max(1, std::min(16, (int)((227 * 1024) / (smem + 1024))));
  return (int)std::max<int64_t>(1, std::min<int64_t>(ceil_div(ceil_div(nrows, (int64_t)32), (int64_t)kStgWarps),
                                                     (int64_t)ctx->sm_count * per_sm));
}

// shared-memory opt-in for the longest rows, once per device and kernel (a
// function attribute: set before any stream capture launches the kernel)
static mfe_status staged_configure(mfe_ctx* ctx, const void* kernel, size_t smem, bool* configured)
{
  const int dev = ctx->device;
  if (dev >= 0 && dev < 64 && configured[dev]) return MFE_OK;
  MFE_CUDA_TRY(ctx, cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  if (dev >= 0 && dev < 64) configured[dev] = true;
  return MFE_OK;
}

// P filled but for cap; rows of at most max_len <= kStgMaxLen entries
template <typename T, int MODE>
static mfe_status launch_staged(mfe_ctx* ctx, SpmvParams<T>& P, int max_len)
{
  static bool configured[64] = {};
  MFE_TRY(staged_configure(ctx, (const void*)k_spmv_staged<T, MODE>,
                           staged_smem<T>(kStgMaxLen, false), configured));
  P.cap = stg_cap(max_len, false);
  MFE_TRY(take_wait_injection(ctx, &P.withhold_ns));
  k_spmv_staged<T, MODE><<<staged_grid<T>(ctx, P.n, max_len, false), kStgWarps * 32,
                           staged_smem<T>(max_len, false), ctx->stream>>>(P, max_len);
  return check_launch(ctx, "k_spmv_staged");
}

int spmv_grid(mfe_ctx* ctx, const mfe_csr* A)
{
  const int max_len = A->max_row_len > 0 ? A->max_row_len : kStgMaxLen;
  if (max_len > kStgMaxLen)  // the warp-per-row kernel
    return (int)std::max<int64_t>(
        1, std::min<int64_t>(ceil_div(A->nrows * 32, 256), (int64_t)ctx->sm_count * 8));
  if (A->dtype == MFE_F64) return staged_grid<double>(ctx, A->nrows, max_len, false);
  const int rows = tile_rows();
  const int64_t ntiles = ceil_div(A->nrows, rows);
  const int per_sm = tiled_ctas_per_sm(tiled_smem<float>(rows, max_len));
  return (int)std::max<int64_t>(1, std::min<int64_t>(ntiles, (int64_t)ctx->sm_count * per_sm));
}

mfe_status ensure_max_row_len(mfe_ctx* ctx, const mfe_csr* A, int* max_len)
{
  if (A->max_row_len > 0) {
    *max_len = A->max_row_len;
    return MFE_OK;
  }
  int* d = static_cast<int*>(workspace(ctx, "spmv.maxlen", sizeof(int)));
  if (!d) return fail(ctx, MFE_OOM, "workspace allocation failed");
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(d, 0, sizeof(int), ctx->stream));
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ceil_div(A->nrows, 256),
                                                                (int64_t)ctx->sm_count * 8));
  k_max_row_len<<<(unsigned)blocks, 256, 0, ctx->stream>>>(A->nrows, A->row_offsets, d);
  MFE_TRY(check_launch(ctx, "k_max_row_len"));
  int* h = static_cast<int*>(host_scratch(ctx, sizeof(int)));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(h, d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  *max_len = *h;
  return MFE_OK;
}

template <typename T, int MODE>
static mfe_status launch_t(mfe_ctx* ctx, const mfe_csr* A, const T* x, T* y, const DotSink* sink,
                           const double* b, CgState* cg, int max_len)
{
  SpmvParams<T> P;
  P.n = A->nrows;
  P.nnz = A->nnz;
  P.ro = A->row_offsets;
  P.cols = A->cols;
  P.vals = static_cast<const T*>(A->vals);
  P.x = x;
  P.y = y;
  P.b = b;
  const int rows = tile_rows();
  P.cap = tile_cap(rows, std::max(max_len, 1));
  P.partials = sink ? sink->partials : nullptr;
  P.ticket = sink ? sink->ticket : nullptr;
  P.dot_out = sink ? sink->out : nullptr;
  P.cg = cg;
  P.withhold_ns = 0;
  P.err = static_cast<unsigned*>(workspace(ctx, "spmv.err", sizeof(unsigned)));
  if (!P.err) return fail(ctx, MFE_OOM, "workspace allocation failed");
  if (cg) P.err = &cg->err;
  if (A->nrows == 0) return MFE_OK;
  if (max_len <= kStgMaxLen && aligned16(A->vals) && aligned16(A->cols)) {
    if constexpr (sizeof(T) == 8) {
      return launch_staged<T, MODE>(ctx, P, max_len);
    } else {
      MFE_CUDA_TRY(ctx, configure_tiled(ctx->device));
      const size_t smem = tiled_smem<T>(rows, std::max(max_len, 1));
      const int64_t ntiles = ceil_div(A->nrows, rows);
      const int grid = (int)std::max<int64_t>(
          1, std::min<int64_t>(ntiles, (int64_t)ctx->sm_count * tiled_ctas_per_sm(smem)));
      if (rows == 64)
        k_spmv_tiled<T, 64, kStages, MODE><<<grid, 64, smem, ctx->stream>>>(P);
      else if (rows == 256)
        k_spmv_tiled<T, 256, kStages, MODE><<<grid, 256, smem, ctx->stream>>>(P);
      else
        k_spmv_tiled<T, 128, kStages, MODE><<<grid, 128, smem, ctx->stream>>>(P);
      return check_launch(ctx, "k_spmv_tiled");
    }
  }
  const int grid = (int)std::max<int64_t>(
      1, std::min<int64_t>(ceil_div(A->nrows * 32, 256), (int64_t)ctx->sm_count * 8));
  k_spmv_warp<T, MODE><<<grid, 256, 0, ctx->stream>>>(P);
  return check_launch(ctx, "k_spmv_warp");
}

mfe_status launch_spmv(mfe_ctx* ctx, const mfe_csr* A, const void* x, void* y,
                       const DotSink* sink, const double* resid_b, void* cg_state)
{
  // bulk async copies need 16-byte aligned sources
  if (csr_is_box(A) && aligned16(A->vals) && aligned16(x) &&
      getenv("MFE_SPMV_GENERIC") == nullptr)
    return launch_spmv_box(ctx, A, x, y, sink, resid_b, cg_state);
  int max_len = 0;
  MFE_TRY(ensure_max_row_len(ctx, A, &max_len));
  CgState* cg = static_cast<CgState*>(cg_state);
  if (A->dtype == MFE_F64) {
    const double* xd = static_cast<const double*>(x);
    double* yd = static_cast<double*>(y);
    if (resid_b) return launch_t<double, SPMV_RESID>(ctx, A, xd, yd, sink, resid_b, cg, max_len);
    if (sink) return launch_t<double, SPMV_DOT>(ctx, A, xd, yd, sink, nullptr, cg, max_len);
    return launch_t<double, SPMV_PLAIN>(ctx, A, xd, yd, nullptr, nullptr, cg, max_len);
  }
  if (A->dtype == MFE_F32) {
    const float* xf = static_cast<const float*>(x);
    float* yf = static_cast<float*>(y);
    if (resid_b) return fail(ctx, MFE_NOT_SUPPORTED, "FP32 residual SpMV is not provided");
    if (sink) return launch_t<float, SPMV_DOT>(ctx, A, xf, yf, sink, nullptr, cg, max_len);
    return launch_t<float, SPMV_PLAIN>(ctx, A, xf, yf, nullptr, nullptr, cg, max_len);
  }
  return fail(ctx, MFE_BAD_ARG, "unknown matrix dtype");
}

template <typename T, int MODE>
static mfe_status launch_ell_t(mfe_ctx* ctx, const mfe_ell* E, const T* x, T* y, const DotSink* sink,
                               const double* b, CgState* cg)
{
  static bool configured[64] = {};
  MFE_TRY(staged_configure(ctx, (const void*)k_spmv_ell<T, MODE>, staged_smem<T>(kStgMaxLen, true),
                           configured));
  SpmvParams<T> P;
  memset(&P, 0, sizeof(P));
  P.n = E->nrows;
  P.nnz = E->nrows * (int64_t)E->ncols_per_row;
  P.cols = E->cols;
  P.vals = static_cast<const T*>(E->vals);
  P.x = x;
  P.y = y;
  P.b = b;
  P.cap = stg_cap(E->ncols_per_row, true);
  P.partials = sink ? sink->partials : nullptr;
  P.ticket = sink ? sink->ticket : nullptr;
  P.dot_out = sink ? sink->out : nullptr;
  P.cg = cg;
  P.err = static_cast<unsigned*>(workspace(ctx, "spmv.err", sizeof(unsigned)));
  if (!P.err) return fail(ctx, MFE_OOM, "workspace allocation failed");
  if (cg) P.err = &cg->err;
  MFE_TRY(take_wait_injection(ctx, &P.withhold_ns));
  const int K = E->ncols_per_row;
  k_spmv_ell<T, MODE><<<staged_grid<T>(ctx, P.n, K, true), kStgWarps * 32, staged_smem<T>(K, true),
                        ctx->stream>>>(P, K);
  return check_launch(ctx, "k_spmv_ell");
}

mfe_status launch_spmv_ell(mfe_ctx* ctx, const mfe_ell* E, const void* x, void* y,
                           const DotSink* sink, const double* resid_b, void* cg_state)
{
  if (E->nrows == 0) return MFE_OK;
  // products with x.y (no caller on the ELL) also take the CSR view
  const bool dot_only = sink != nullptr && resid_b == nullptr;
  if (E->ncols_per_row > kStgMaxLen || !aligned16(E->vals) || !aligned16(E->cols) || dot_only) {
    mfe_csr V;
    MFE_TRY(ell_view(ctx, E, &V));
    return launch_spmv(ctx, &V, x, y, sink, resid_b, cg_state);
  }
  CgState* cg = static_cast<CgState*>(cg_state);
  if (E->dtype == MFE_F64) {
    const double* xd = static_cast<const double*>(x);
    double* yd = static_cast<double*>(y);
    if (resid_b) return launch_ell_t<double, SPMV_RESID>(ctx, E, xd, yd, sink, resid_b, cg);
    return launch_ell_t<double, SPMV_PLAIN>(ctx, E, xd, yd, nullptr, nullptr, cg);
  }
  if (E->dtype == MFE_F32) {
    const float* xf = static_cast<const float*>(x);
    float* yf = static_cast<float*>(y);
    if (resid_b) return fail(ctx, MFE_NOT_SUPPORTED, "FP32 residual SpMV is not provided");
    return launch_ell_t<float, SPMV_PLAIN>(ctx, E, xf, yf, nullptr, nullptr, cg);
  }
  return fail(ctx, MFE_BAD_ARG, "unknown matrix dtype");
}

mfe_status launch_spmm(mfe_ctx* ctx, const mfe_csr* A, int nrhs, const void* X, void* Y)
{
  if (A->nrows == 0) return MFE_OK;
  if (spmm_box_eligible(A, nrhs, X, Y) && getenv("MFE_SPMV_GENERIC") == nullptr)
    return launch_spmm_box(ctx, A, nrhs, X, Y);
  const int64_t total = A->nrows * (int64_t)nrhs;
  const int64_t blocks = std::max<int64_t>(1, std::min<int64_t>(ceil_div(total, 256),
                                                                (int64_t)ctx->sm_count * 16));
  if (A->dtype == MFE_F64)
    k_spmm<double><<<(unsigned)blocks, 256, 0, ctx->stream>>>(
        A->nrows, nrhs, A->row_offsets, A->cols, static_cast<const double*>(A->vals),
        static_cast<const double*>(X), static_cast<double*>(Y));
  else
    k_spmm<float><<<(unsigned)blocks, 256, 0, ctx->stream>>>(
        A->nrows, nrhs, A->row_offsets, A->cols, static_cast<const float*>(A->vals),
        static_cast<const float*>(X), static_cast<float*>(Y));
  return check_launch(ctx, "k_spmm");
}

mfe_status take_spmv_error(mfe_ctx* ctx)
{
  auto it = ctx->ws.find("spmv.err");
  if (it == ctx->ws.end() || !it->second.ptr) return MFE_OK;
  unsigned h = 0;
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(&h, it->second.ptr, sizeof(unsigned), cudaMemcpyDeviceToHost,
                                    ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (!h) return MFE_OK;
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(it->second.ptr, 0, sizeof(unsigned), ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return fail(ctx, MFE_TIMEOUT,
              (h & 1u) ? "a matrix-vector kernel gave up a bounded wait"
                       : "a matrix-vector kernel met a tile larger than its stage");
}

}  // namespace mfe
