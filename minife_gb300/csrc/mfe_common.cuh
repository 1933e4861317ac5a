// Shared device helpers for the minife_gb300 kernels (sm_103a).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "minife_gb300.h"

namespace mfe {

// ---------------------------------------------------------------------------
// error flags written by kernels instead of trapping: bit 0 = a bounded
// mbarrier wait gave up, bit 1 = a tile did not fit its shared-memory stage
// ---------------------------------------------------------------------------
enum : unsigned { ERR_WAIT_TIMEOUT = 1u, ERR_TILE_OVERFLOW = 2u };

// Upper bound on mbarrier polls before a wait gives up (each try_wait may
// suspend the thread for a hardware-chosen interval, so this is >> 1 s).
constexpr unsigned kMaxPolls = 1u << 26;

// ---------------------------------------------------------------------------
// reductions (deterministic for a fixed launch shape)
// ---------------------------------------------------------------------------
__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the block; result valid in thread 0.  scratch: >= 32 doubles.
__device__ __forceinline__ double block_sum(double v, double* scratch)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_sum(v);
  __syncthreads();  // scratch may be reused across calls
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  double s = 0.0;
  if (wid == 0) {
    s = lane < nw ? scratch[lane] : 0.0;
    s = warp_sum(s);
  }
  return s;
}

// Grid-level reduction tail: block partial -> partials[blockIdx.x]; the last
// block to finish (atomic ticket) sums the partials in block order and
// returns true with the total in *total (thread 0 only).  The ticket counter
// is re-armed to 0 by the last block, so consecutive launches reuse it.
__device__ __forceinline__ bool grid_reduce_last(double block_total, double* partials,
                                                 unsigned* ticket, double* scratch,
                                                 double* total)
{
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
    partials[blockIdx.x] = block_total;
    __threadfence();
    unsigned t = atomicAdd(ticket, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  double s = 0.0;
  for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x)
    s += __ldcg(&partials[i]);
  s = block_sum(s, scratch);
  if (threadIdx.x == 0) {
    *total = s;
    *ticket = 0u;
  }
  return true;
}

// ---------------------------------------------------------------------------
// mbarrier + bulk async copy (TMA, non-tensor form), inline PTX
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count)
{
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init()
{
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async_smem()
{
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes)
{
  asm volatile("mbarrier.arrive.expect_tx.release.cta.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Adds bytes to the current phase's expected transaction count without
// arriving (each lane of a producer warp announces its own copy).
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes)
{
  asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Plain arrival (count 1), release semantics: prior shared-memory reads by
// this thread are ordered before the phase can complete.
__device__ __forceinline__ void mbar_arrive(uint64_t* bar)
{
  asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity)
{
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.acquire.cta.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns()
{
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Longest a bounded wait may take before it gives up (nanoseconds).
constexpr uint64_t kWaitLimitNs = 2000000000ull;

// Bounded wait; returns false (and the caller records ERR_WAIT_TIMEOUT) if
// the phase did not complete within limit_ns (or kMaxPolls polls).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity,
                                                  uint64_t limit_ns = kWaitLimitNs)
{
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (unsigned i = 1; i < kMaxPolls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((i & 63u) == 0 && global_ns() - t0 > limit_ns) return false;
  }
  return false;
}

// 1-D bulk copy global -> shared, completion counted on bar (bytes, smem and
// gmem addresses must be multiples of 16).
__device__ __forceinline__ void bulk_g2s(void* smem_dst, const void* gmem_src, unsigned bytes,
                                         uint64_t* bar)
{
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(smem_dst)),
      "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// ---------------------------------------------------------------------------
// exact float -> double widening with integer operations only: on GB300 the
// FP64 pipe (which also executes F2F.F64.F32) is the scarce resource, so the
// FP64-accumulated dots of FP32 vectors spend their one FP64 operation per
// element on the FMA.  Built from the IEEE-754 binary32/binary64 layouts:
// the exponent is rebiased by 1023 - 127 = 896 and the 23-bit fraction moves
// to the top of the 52-bit one.  A subnormal float f * 2^-149 (0 < f < 2^23)
// is normal in binary64: with h the position of f's leading bit it is
// 2^(h - 149) * (f / 2^h), exponent field h - 149 + 1023, and f's bits below
// h become the top of the fraction.
// ---------------------------------------------------------------------------
__device__ __forceinline__ double f2d_exact(float f)
{
  const uint32_t u = __float_as_uint(f);
  const uint32_t e = (u >> 23) & 0xffu;
  const uint32_t f23 = u & 0x7fffffu;
  const uint64_t sign = (uint64_t)(u & 0x80000000u) << 32;
  const uint64_t frac = (uint64_t)f23 << 29;
  uint64_t bits;
  if (e == 0u) {
    if (f23 == 0u) {
      bits = sign;
    } else {
      const int h = 31 - __clz((int)f23);
      bits = sign | ((uint64_t)(h + 874) << 52) | (((uint64_t)f23 << (52 - h)) & 0xfffffffffffffull);
    }
  } else if (e == 0xffu) {
    bits = sign | 0x7ff0000000000000ull | frac;
  } else {
    bits = sign | ((uint64_t)(e + 896u) << 52) | frac;
  }
  return __longlong_as_double((long long)bits);
}

__device__ __forceinline__ double widen(double v) { return v; }
__device__ __forceinline__ double widen(float v) { return f2d_exact(v); }

// ---------------------------------------------------------------------------
// Double-float accumulator for sums of FP32 products, FP32 operations only
// (FP64 arithmetic on GB300 runs at 1/60 of the FP32 rate).  Each product is
// split exactly into p + pe with an FMA (Dekker's TwoProduct), p is added to
// hi with Knuth's TwoSum, and both rounding errors go to lo, so hi + lo holds
// the sum to about 48 significant bits.  The __f*_rn intrinsics keep the
// compiler from contracting the steps into FMAs, which would lose the error
// terms.
// ---------------------------------------------------------------------------
struct DFAcc {
  float hi = 0.0f, lo = 0.0f;
  __device__ __forceinline__ void add_product(float a, float b)
  {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    const float t = __fadd_rn(hi, p);
    const float bp = __fsub_rn(t, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    hi = t;
    lo = __fadd_rn(lo, __fadd_rn(err, pe));
  }
  // an FP32 term (already rounded) added with TwoSum
  __device__ __forceinline__ void add(float v)
  {
    const float t = __fadd_rn(hi, v);
    const float bp = __fsub_rn(t, hi);
    const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(v, bp));
    hi = t;
    lo = __fadd_rn(lo, err);
  }
  __device__ __forceinline__ double value() const { return f2d_exact(hi) + f2d_exact(lo); }
};

// Double-float reductions with FP32 operations only, so the tail of a kernel
// whose rows are summed in DFAcc does not queue on the FP64 pipe (1/64 of the
// FP32 rate on GB300): (hi, lo) += (h2, l2), TwoSum on the high parts.
__device__ __forceinline__ void df_add(float& hi, float& lo, float h2, float l2)
{
  const float t = __fadd_rn(hi, h2);
  const float bp = __fsub_rn(t, hi);
  const float err = __fadd_rn(__fsub_rn(hi, __fsub_rn(t, bp)), __fsub_rn(h2, bp));
  hi = t;
  lo = __fadd_rn(lo, __fadd_rn(l2, err));
}

__device__ __forceinline__ void warp_sum_df(float& hi, float& lo)
{
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float h2 = __shfl_xor_sync(0xffffffffu, hi, o);
    const float l2 = __shfl_xor_sync(0xffffffffu, lo, o);
    df_add(hi, lo, h2, l2);
  }
}

// block sum of double-float pairs, valid in thread 0; scratch >= 32 pairs
__device__ __forceinline__ void block_sum_df(float& hi, float& lo, float2* scratch)
{
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  warp_sum_df(hi, lo);
  __syncthreads();  // scratch may be reused across calls
  if (lane == 0) scratch[wid] = make_float2(hi, lo);
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  hi = 0.0f;
  lo = 0.0f;
  if (wid == 0) {
    if (lane < nw) {
      hi = scratch[lane].x;
      lo = scratch[lane].y;
    }
    warp_sum_df(hi, lo);
  }
}

// grid_reduce_last on double-float pairs: each block's pair goes to its
// 8-byte slot of partials, the last block sums them in block order and thread
// 0 gets hi + lo in FP64 (the one FP64 operation).
__device__ __forceinline__ bool grid_reduce_last_df(const DFAcc& a, double* partials, unsigned* ticket,
                                                    float2* scratch, double* total)
{
  float hi = a.hi, lo = a.lo;
  block_sum_df(hi, lo, scratch);
  float2* slots = reinterpret_cast<float2*>(partials);
  __shared__ bool am_last;
  if (threadIdx.x == 0) {
    slots[blockIdx.x] = make_float2(hi, lo);
    __threadfence();
    const unsigned t = atomicAdd(ticket, 1u);
    am_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return false;
  __threadfence();
  hi = 0.0f;
  lo = 0.0f;
  for (unsigned i = threadIdx.x; i < gridDim.x; i += blockDim.x) {
    const float2 v = __ldcg(&slots[i]);
    df_add(hi, lo, v.x, v.y);
  }
  block_sum_df(hi, lo, scratch);
  if (threadIdx.x == 0) {
    *total = f2d_exact(hi) + f2d_exact(lo);
    *ticket = 0u;
  }
  return true;
}

// ---------------------------------------------------------------------------
// misc
// ---------------------------------------------------------------------------
template <typename T>
__device__ __forceinline__ T ldg(const T* p) { return __ldg(p); }

__host__ __device__ __forceinline__ int64_t ceil_div(int64_t a, int64_t b)
{
  return (a + b - 1) / b;
}

}  // namespace mfe
