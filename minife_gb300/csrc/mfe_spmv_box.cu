// SpMV for matrices with the 27-point box structure that miniFE assembles
// (generate_matrix_structure.hpp / MatrixInitOp.hpp): the CSR values are read
// in their CSR order, but column indices and row offsets are not read at all —
// they follow in closed form from the box dimensions (mfe_box.cuh).
//
// For a tile of ROWS consecutive rows r0..r1, every column a row can touch is
// r + dx + dy*Nx + dz*NxNy, so the tile needs exactly nine contiguous segments
// of x (one per (dy, dz)), each ROWS + 2 long.  One producer thread stages the
// tile's values and the nine x segments into shared memory with 1-D bulk
// async copies (TMA) tracked by an mbarrier, S stages deep; consumers then
// find every operand in shared memory, so the FMAs never wait on a global
// gather.  Each row runs the same 27-slot code: slots outside the box are
// masked (branch-free selects), which keeps the boundary rows of a warp from
// diverging.  One FP64 FMA per slot (two interleaved partial sums, one add).
//
// Bytes per FP64 product: 8 per nonzero + x and y once (5.797 GB of CSR
// traffic at 256^3 becomes 3.910 GB); the kernel is then bounded by the FP64
// FMA rate rather than by HBM.  The FP32 variant moves 1.955 GB.
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "mfe_box.cuh"
#include "mfe_cgstate.cuh"
#include "mfe_common.cuh"
#include "mfe_internal.h"

namespace mfe {

enum BoxMode { BOX_PLAIN = 0, BOX_DOT = 1, BOX_RESID = 2 };

template <typename T>
struct BoxParams {
  int n;               // rows = Nx*Ny*Nz (< 2^31)
  int Nx, Ny, Nz;
  int NxNy;
  int64_t nnz;
  const T* __restrict__ vals;
  const T* __restrict__ x;
  T* __restrict__ y;
  const double* __restrict__ b;
  int capv;            // value elements per stage
  int capx;            // x elements per segment
  double* partials;
  unsigned* ticket;
  double* dot_out;
  CgState* cg;
  unsigned* err;
  float* y32;          // BOX_RESID: when set, the residual is written as FP32 here
  int y32_pad;         // y32 rows are (Nx + y32_pad) long: row r goes to r + (r / Nx) * y32_pad
  const int* gate;     // when set and *gate == 0 the launch does nothing
  // fault injection (mfe_inject_wait_timeout): nonzero = the producer
  // issues no copy and arrives nowhere, and the consumers' bounded waits on
  // the first stage give up after this many nanoseconds
  uint64_t withhold_ns;
};

template <int MODE>
__device__ __forceinline__ void box_epilogue(double total, CgState* cg, double* dot_out)
{
  if (cg == nullptr) {
    if (MODE != BOX_PLAIN) *dot_out = total;
    return;
  }
  if (MODE == BOX_DOT) {
    cg->pAp = total;
    if (total < cg->brkdown_tol) cg->check_pending = 1;
  } else if (MODE == BOX_RESID) {
    cg_resid_init(cg, total);
  }
}

// Warp-specialised pipeline: warp 0 is the producer (lane 0 stages tiles),
// warps 1..C are consumers, one row per consumer thread (ROWS = 32 * C).
// full[s] completes when stage s holds its tile (expect_tx + bulk copies);
// empty[s] completes when all C consumer warps have finished reading it, so
// the producer runs up to S tiles ahead without any CTA-wide barrier.
template <typename T, int ROWS, int S, int MODE>
__global__ void __launch_bounds__(ROWS + 32) k_spmv_box(BoxParams<T> P)
{
  constexpr int C = ROWS / 32;  // consumer warps
  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t full[S], empty[S];
  __shared__ int s_vbase[S];     // first staged value index of each stage
  __shared__ int s_xbase[S][9];  // first staged x index of each segment
  __shared__ double red[32];
  constexpr int VA = 16 / sizeof(T);
  const size_t stage_elems = (size_t)P.capv + 9 * (size_t)P.capx;
  T* const st0 = reinterpret_cast<T*>(smem);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ntiles = (P.n + ROWS - 1) / ROWS;
  // gated launches (the mixed solver's reliable update inside its graph)
  // return at once, uniformly for the whole grid, when the gate is closed
  if (P.gate != nullptr && *P.gate == 0) return;
  if (threadIdx.x == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], C);
    }
    fence_mbar_init();
  }
  __syncthreads();

  double dacc = 0.0;
  bool ok = true;
  if (warp == 0) {
    // ---------------- producer ----------------
    if (lane == 0 && P.withhold_ns == 0) {
      int it = 0;
      unsigned issued[S];
      for (int s = 0; s < S; ++s) issued[s] = 0;
      for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++it) {
        const int s = it % S;
        if (it >= S) ok = mbar_wait_bounded(&empty[s], (unsigned)(((it / S) - 1) & 1));
        if (!ok) break;
        T* sv = st0 + (size_t)s * stage_elems;
        T* sx = sv + P.capv;
        const int r0 = tile * ROWS, r1 = min(P.n, r0 + ROWS);
        const int64_t a = row_offset_of32(r0, P.Nx, P.Ny, P.Nz, P.NxNy);
        const int64_t e = row_offset_of32(r1, P.Nx, P.Ny, P.Nz, P.NxNy);
        const int64_t av = a & ~(int64_t)(VA - 1);
        int64_t bv = min((e + VA - 1) & ~(int64_t)(VA - 1), P.nnz & ~(int64_t)(VA - 1));
        if (bv < av) bv = av;
        bool fits = (max(bv, e) - av <= P.capv);
        int xlo[9], xbl[9], xhi[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const int off = (j / 3 - 1) * P.NxNy + (j % 3 - 1) * P.Nx;
          // the segment [lo, hi) is clamped to [0, n] at both ends: near the
          // last rows r0 + off can lie past the end of x
          const int lo = min(max(r0 + off - 1, 0), P.n);
          int hi = min(r1 + off + 1, P.n);
          if (hi < lo) hi = lo;
          const int lal = lo & ~(VA - 1);
          int bl = min((hi + VA - 1) & ~(VA - 1), P.n & ~(VA - 1));
          if (bl < lal) bl = lal;
          xlo[j] = lal;
          xbl[j] = bl;
          xhi[j] = hi;
          fits = fits && (max(bl, hi) - lal <= P.capx);
        }
        ++issued[s];
        if (!fits) {
          // cannot happen for box dimensions the host accepted; record it
          atomicOr(P.err, ERR_TILE_OVERFLOW);
          s_vbase[s] = (int)a;
          for (int j = 0; j < 9; ++j) s_xbase[s][j] = 0;
          mbar_arrive_expect_tx(&full[s], 0);
          continue;
        }
        s_vbase[s] = (int)av;
        unsigned bytes = (unsigned)((bv - av) * sizeof(T));
        for (int64_t k = bv; k < e; ++k) sv[k - av] = P.vals[k];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          s_xbase[s][j] = xlo[j];
          T* dx = sx + (size_t)j * P.capx;
          for (int k = xbl[j]; k < xhi[j]; ++k) dx[k - xlo[j]] = P.x[k];
          bytes += (unsigned)((xbl[j] - xlo[j]) * sizeof(T));
        }
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&full[s], bytes);
        if (bv > av) bulk_g2s(sv, P.vals + av, (unsigned)((bv - av) * sizeof(T)), &full[s]);
#pragma unroll
        for (int j = 0; j < 9; ++j)
          if (xbl[j] > xlo[j])
            bulk_g2s(sx + (size_t)j * P.capx, P.x + xlo[j],
                     (unsigned)((xbl[j] - xlo[j]) * sizeof(T)), &full[s]);
      }
      if (!ok) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        // bounded drain: let the last copies issued into each stage land
        for (int s = 0; s < S; ++s)
          if (issued[s]) mbar_wait_bounded(&full[s], (issued[s] - 1) & 1u);
      }
    }
  } else {
    // ---------------- consumers ----------------
    const int lr = (warp - 1) * 32 + lane;
    int it = 0;
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
      const int s = it % S;
      // row coordinates and offsets do not depend on the staged data
      const int r = tile * ROWS + lr;
      const bool active = r < P.n;
      const int rr = active ? r : P.n - 1;
      const int iz = rr / P.NxNy;
      const int rem = rr - iz * P.NxNy;
      const int iy = rem / P.Nx;
      const int ix = rem - iy * P.Nx;
      const int64_t roff = row_offset(ix, iy, iz, P.Nx, P.Ny, P.Nz);
      if (!mbar_wait_bounded(&full[s], (unsigned)((it / S) & 1),
                             P.withhold_ns ? P.withhold_ns : kWaitLimitNs)) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        ok = false;
        break;
      }
      const bool vxm = ix > 0, vxp = ix < P.Nx - 1;
      const bool vym = iy > 0, vyp = iy < P.Ny - 1;
      const bool vzm = iz > 0, vzp = iz < P.Nz - 1;
      const bool interior = active && vxm && vxp && vym && vyp && vzm && vzp;
      // warps whose rows all have the full 27 columns (about three in four
      // at 256^3) take the unmasked code: value k of a row is rowv[k]
      const bool all_interior = __all_sync(0xffffffffu, interior);
      if (all_interior) {
        const T* sv = st0 + (size_t)s * stage_elems;
        const T* sx = sv + P.capv;
        const T* rowv = sv + (roff - s_vbase[s]);
        const T* xc = sx + 4 * (size_t)P.capx + (r - s_xbase[s][4]);
        T s0 = T(0), s1 = T(0);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
          const int off = (j / 3 - 1) * P.NxNy + (j % 3 - 1) * P.Nx;
          const T* seg = sx + (size_t)j * P.capx + (r + off - s_xbase[s][j]);
#pragma unroll
          for (int dx = -1; dx <= 1; ++dx) {
            const int k = j * 3 + dx + 1;
            if (k & 1) s1 = fma(rowv[k], seg[dx], s1);
            else s0 = fma(rowv[k], seg[dx], s0);
          }
        }
        const T sum = s0 + s1;
        const T xr = xc[0];
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);  // stage s no longer read by this warp
        if (MODE == BOX_RESID) {
          const double res = P.b[r] - widen(sum);
          if (P.y32 != nullptr)
            P.y32[P.y32_pad ? (int64_t)r + (int64_t)(r / P.Nx) * P.y32_pad : (int64_t)r] = (float)res;
          else P.y[r] = (T)res;
          dacc = fma(res, res, dacc);
        } else {
          P.y[r] = sum;
          if (MODE == BOX_DOT) dacc = fma(widen(sum), widen(xr), dacc);
        }
      } else if (active) {
        const T* sv = st0 + (size_t)s * stage_elems;
        const T* sx = sv + P.capv;
        const T* rowv = sv + (roff - s_vbase[s]);
        const int cx = 1 + vxm + vxp, cy = 1 + vym + vyp;
        const int cxy = cx * cy;
        // x[r] lives in the centre segment (j = 4) of every tile
        const T* xc = sx + 4 * (size_t)P.capx + (r - s_xbase[s][4]);
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
            const T* seg = sx + (size_t)j * P.capx + (r + off - s_xbase[s][j]);
            const int pbase = bz * cxy + by * cx;
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
              const bool vx = dx < 0 ? vxm : (dx > 0 ? vxp : true);
              const int bx = dx < 0 ? 0 : (dx == 0 ? (int)vxm : (int)vxm + 1);
              const bool valid = vz && vy && vx;
              // masked slots read the row's first value and x[r], both
              // staged (the addresses are selected: every load is in bounds)
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
        const T sum = s0 + s1;
        const T xr = xc[0];
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);  // stage s no longer read by this warp
        if (MODE == BOX_RESID) {
          const double res = P.b[r] - widen(sum);
          if (P.y32 != nullptr)
            P.y32[P.y32_pad ? (int64_t)r + (int64_t)(r / P.Nx) * P.y32_pad : (int64_t)r] = (float)res;
          else P.y[r] = (T)res;
          dacc = fma(res, res, dacc);
        } else {
          P.y[r] = sum;
          if (MODE == BOX_DOT) dacc = fma(widen(sum), widen(xr), dacc);
        }
      } else {
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
      }
    }
  }
  if (MODE != BOX_PLAIN) {
    const double bt = block_sum(dacc, red);
    double total;
    if (grid_reduce_last(bt, P.partials, P.ticket, red, &total) && threadIdx.x == 0)
      box_epilogue<MODE>(total, P.cg, P.dot_out);
  }
}

// Count rows whose CSR row (offsets and columns) differs from the box
// stencil's; zero means the closed-form layout describes the matrix.
__global__ void k_check_box(int n, int Nx, int Ny, int Nz, const int32_t* __restrict__ ro,
                            const int32_t* __restrict__ cols, unsigned* bad)
{
  const int NxNy = Nx * Ny;
  unsigned nbad = 0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < n; r += gridDim.x * blockDim.x) {
    const int iz = r / NxNy, rem = r - iz * NxNy, iy = rem / Nx, ix = rem - iy * Nx;
    const int64_t off = row_offset(ix, iy, iz, Nx, Ny, Nz);
    bool good = (ro[r] == off);
    if (r == n - 1) good = good && (ro[n] == row_offset_of(n, Nx, Ny, Nz));
    int64_t k = off;
    for (int dz = -1; dz <= 1 && good; ++dz)
      for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
          const int jx = ix + dx, jy = iy + dy, jz = iz + dz;
          if (jx < 0 || jx >= Nx || jy < 0 || jy >= Ny || jz < 0 || jz >= Nz) continue;
          good = good && (cols[k] == r + dx + dy * Nx + dz * NxNy);
          ++k;
        }
    nbad += good ? 0u : 1u;
  }
  if (nbad) atomicAdd(bad, nbad);
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
// Launch shape: rows per tile (64/128/256 = 2/4/8 consumer warps) and
// pipeline stages (2..4).  Defaults per value type come from launch-shape
// sweeps at 256^3; MFE_BOX_ROWS / MFE_BOX_STAGES override them for sweeps.
struct BoxShape {
  int rows, stages;
};

template <typename T>
static BoxShape box_shape()
{
  // measured at 256^3 on GB300: FP64 0.833 ms at {128, 2} (3 CTAs/SM keep
  // 12 consumer warps issuing FP64 FMAs), FP32 0.366 ms at {256, 2}
  BoxShape sh = sizeof(T) == 8 ? BoxShape{128, 2} : BoxShape{256, 2};
  if (const char* v = getenv("MFE_BOX_ROWS")) {
    const int r = atoi(v);
    if (r == 64 || r == 128 || r == 256) sh.rows = r;
  }
  if (const char* v = getenv("MFE_BOX_STAGES")) {
    const int st = atoi(v);
    if (st >= 2 && st <= 4) sh.stages = st;
  }
  if (sh.rows == 256 && sh.stages > 3) sh.stages = 3;
  return sh;
}

static int box_capv(int rows) { return ((rows * 27 + 8) + 3) & ~3; }
static int box_capx(int rows) { return ((rows + 2 + 8) + 3) & ~3; }

template <typename T>
static size_t box_smem(int rows, int stages)
{
  return (size_t)stages * ((size_t)box_capv(rows) + 9 * (size_t)box_capx(rows)) * sizeof(T);
}

// Calls F.template operator()<ROWS, S>() for the instantiated shape.
template <typename F>
static auto box_dispatch(BoxShape sh, F&& f)
{
  if (sh.rows == 64) {
    if (sh.stages == 2) return f.template operator()<64, 2>();
    if (sh.stages == 4) return f.template operator()<64, 4>();
    return f.template operator()<64, 3>();
  }
  if (sh.rows == 256) {
    if (sh.stages == 2) return f.template operator()<256, 2>();
    return f.template operator()<256, 3>();
  }
  if (sh.stages == 2) return f.template operator()<128, 2>();
  if (sh.stages == 4) return f.template operator()<128, 4>();
  return f.template operator()<128, 3>();
}

template <typename T, int MODE>
static cudaError_t box_configure_mode()
{
  const int shapes[8][2] = {{64, 2},  {64, 3},  {64, 4},  {128, 2},
                            {128, 3}, {128, 4}, {256, 2}, {256, 3}};
  for (auto& rs : shapes) {
    BoxShape sh{rs[0], rs[1]};
    const size_t smem = box_smem<T>(sh.rows, sh.stages);
    if (smem > 227 * 1024) continue;
    cudaError_t e = box_dispatch(sh, [&]<int R, int S>() {
      return cudaFuncSetAttribute(k_spmv_box<T, R, S, MODE>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    });
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

static cudaError_t box_configure(int device)
{
  static bool done[64] = {};
  if (device >= 0 && device < 64 && done[device]) return cudaSuccess;
  cudaError_t e = box_configure_mode<double, BOX_PLAIN>();
  if (e == cudaSuccess) e = box_configure_mode<double, BOX_DOT>();
  if (e == cudaSuccess) e = box_configure_mode<double, BOX_RESID>();
  if (e == cudaSuccess) e = box_configure_mode<float, BOX_PLAIN>();
  if (e == cudaSuccess) e = box_configure_mode<float, BOX_DOT>();
  if (e == cudaSuccess && device >= 0 && device < 64) done[device] = true;
  return e;
}

static int box_ctas_per_sm(size_t smem)
{
  int per_sm = (int)((227 * 1024) / (smem + 1024));
  if (const char* v = getenv("MFE_BOX_CTAS_PER_SM")) {
    const int o = atoi(v);
    if (o > 0 && o < per_sm) per_sm = o;
  }
  return std::max(1, per_sm);
}

bool csr_is_box(const mfe_csr* A)
{
  if (A->box_nx <= 0 || A->box_ny <= 0 || A->box_nz <= 0) return false;
  const int64_t Nx = A->box_nx + 1, Ny = A->box_ny + 1, Nz = A->box_nz + 1;
  return A->nrows == Nx * Ny * Nz && A->nnz == box_nnz(A->box_nx, A->box_ny, A->box_nz);
}

mfe_status detect_box(mfe_ctx* ctx, const mfe_csr* A, int* nx, int* ny, int* nz)
{
  *nx = *ny = *nz = 0;
  if (A->nrows < 8 || A->nnz < 8) return MFE_OK;
  // row 0 of a box matrix is node (0,0,0): columns 0, 1, Nx, Nx+1, NxNy, ...
  int32_t h[8];
  int32_t ro2[2];
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(ro2, A->row_offsets, sizeof(ro2), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(h, A->cols, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (ro2[0] != 0 || ro2[1] != 8 || h[0] != 0 || h[1] != 1) return MFE_OK;
  const int64_t Nx = h[2], NxNy = h[4];
  if (Nx < 2 || NxNy < 2 * Nx || NxNy % Nx != 0 || A->nrows % NxNy != 0) return MFE_OK;
  const int64_t Ny = NxNy / Nx, Nz = A->nrows / NxNy;
  if (Nz < 2 || box_nnz((int)Nx - 1, (int)Ny - 1, (int)Nz - 1) != A->nnz) return MFE_OK;
  unsigned* bad = static_cast<unsigned*>(workspace(ctx, "box.bad", sizeof(unsigned)));
  if (!bad) return fail(ctx, MFE_OOM, "workspace allocation failed");
  MFE_CUDA_TRY(ctx, cudaMemsetAsync(bad, 0, sizeof(unsigned), ctx->stream));
  const int blocks = std::max(1, std::min((int)ceil_div(A->nrows, 256), ctx->sm_count * 8));
  k_check_box<<<blocks, 256, 0, ctx->stream>>>((int)A->nrows, (int)Nx, (int)Ny, (int)Nz,
                                                A->row_offsets, A->cols, bad);
  MFE_TRY(check_launch(ctx, "k_check_box"));
  unsigned hb = 1;
  MFE_CUDA_TRY(ctx, cudaMemcpyAsync(&hb, bad, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
  MFE_CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (hb == 0) {
    *nx = (int)Nx - 1;
    *ny = (int)Ny - 1;
    *nz = (int)Nz - 1;
  }
  return MFE_OK;
}

template <typename T, int MODE>
static mfe_status box_launch_t(mfe_ctx* ctx, const mfe_csr* A, const T* x, T* y,
                               const DotSink* sink, const double* b, CgState* cg,
                               float* y32 = nullptr, const int* gate = nullptr, int y32_pad = 0)
{
  BoxParams<T> P;
  P.y32 = y32;
  P.y32_pad = y32_pad;
  P.gate = gate;
  P.Nx = A->box_nx + 1;
  P.Ny = A->box_ny + 1;
  P.Nz = A->box_nz + 1;
  P.NxNy = P.Nx * P.Ny;
  P.n = (int)A->nrows;
  P.nnz = A->nnz;
  P.vals = static_cast<const T*>(A->vals);
  P.x = x;
  P.y = y;
  P.b = b;
  const BoxShape sh = box_shape<T>();
  P.capv = box_capv(sh.rows);
  P.capx = box_capx(sh.rows);
  P.partials = sink ? sink->partials : nullptr;
  P.ticket = sink ? sink->ticket : nullptr;
  P.dot_out = sink ? sink->out : nullptr;
  P.cg = cg;
  P.err = static_cast<unsigned*>(workspace(ctx, "spmv.err", sizeof(unsigned)));
  if (!P.err) return fail(ctx, MFE_OOM, "workspace allocation failed");
  if (cg) P.err = &cg->err;
  MFE_TRY(take_wait_injection(ctx, &P.withhold_ns));
  MFE_CUDA_TRY(ctx, box_configure(ctx->device));
  const size_t smem = box_smem<T>(sh.rows, sh.stages);
  const int64_t ntiles = ceil_div(A->nrows, sh.rows);
  const int grid = (int)std::max<int64_t>(
      1, std::min<int64_t>(ntiles, (int64_t)ctx->sm_count * box_ctas_per_sm(smem)));
  box_dispatch(sh, [&]<int R, int S>() {
    k_spmv_box<T, R, S, MODE><<<grid, R + 32, smem, ctx->stream>>>(P);
    return 0;
  });
  return check_launch(ctx, "k_spmv_box");
}

mfe_status launch_spmv_box(mfe_ctx* ctx, const mfe_csr* A, const void* x, void* y,
                           const DotSink* sink, const double* resid_b, void* cg_state)
{
  CgState* cg = static_cast<CgState*>(cg_state);
  if (A->nrows == 0) return MFE_OK;
  if (A->dtype == MFE_F64) {
    const double* xd = static_cast<const double*>(x);
    double* yd = static_cast<double*>(y);
    if (resid_b) return box_launch_t<double, BOX_RESID>(ctx, A, xd, yd, sink, resid_b, cg);
    if (sink) return box_launch_t<double, BOX_DOT>(ctx, A, xd, yd, sink, nullptr, cg);
    return box_launch_t<double, BOX_PLAIN>(ctx, A, xd, yd, nullptr, nullptr, cg);
  }
  const float* xf = static_cast<const float*>(x);
  float* yf = static_cast<float*>(y);
  if (resid_b) return fail(ctx, MFE_NOT_SUPPORTED, "FP32 residual SpMV is not provided");
  if (sink) return box_launch_t<float, BOX_DOT>(ctx, A, xf, yf, sink, nullptr, cg);
  return box_launch_t<float, BOX_PLAIN>(ctx, A, xf, yf, nullptr, nullptr, cg);
}

mfe_status launch_box_resid_f32out(mfe_ctx* ctx, const mfe_csr* A64, const double* x,
                                   const double* b, float* r32, const DotSink* sink,
                                   const int* gate, int r32_pad)
{
  if (A64->nrows == 0) return MFE_OK;
  return box_launch_t<double, BOX_RESID>(ctx, A64, x, nullptr, sink, b, nullptr, r32, gate, r32_pad);
}

}  // namespace mfe
