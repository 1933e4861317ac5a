// Allocation-free FP64 dot product: mfe_dot_noalloc (include/minife_gb300.h).
//
// Every other reduction in this library keeps its per-block partial sums in
// workspace that an mfe_ctx allocates with cudaMalloc on first use.  Some
// callers cannot allow that: applications whose device memory is owned by
// another allocator (a framework or host program that reserves the GPU's
// memory in its own pool up front and does not let a plugin allocate beside
// it), and latency-critical loops that cannot take the implicit device-wide
// synchronisation a cudaMalloc / cudaFree may cause.  For them this file
// provides a dot product that needs no context and allocates nothing: its
// scratch -- one partial sum per block plus the last-block ticket -- is the
// file-scope device array below.  That array is part of the library's device
// image, so every GPU that loads the library holds it (about 512 KiB) until
// the process exits.
//
// Layout and limits: block b of the grid sums elements [b*kChunk, (b+1)*kChunk)
// (the grid never strides), so the scratch caps the vector length at
// kMaxBlocks * kChunk = 2^29 elements; longer vectors are rejected with
// MFE_BAD_ARG before anything is launched.  Because the chunking does not
// depend on the GPU, results are deterministic for a given n.
//
// Sharing: all calls in the process use the same array on a device and the
// array keeps the last call's partial sums.  The ticket is cleared on the
// caller's stream before every launch; the partials need no clearing (every
// launched block overwrites its own slot before the last block reads them).
// Calls that overlap on the GPU (on different streams, or from several host
// threads without ordering) race on the scratch and must not be issued.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "mfe_common.cuh"
#include "minife_gb300.h"

namespace mfe {
namespace {

constexpr int kChunk = 8192;         // elements per block
constexpr int kMaxBlocks = 65536;    // one partial per block
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;
static_assert((int64_t)kMaxBlocks * kChunk == MFE_DOT_NOALLOC_MAX_N, "limit mismatch");

// kMaxBlocks partials followed by the ticket (stored in the next slot).
static __device__ __align__(256) double g_noalloc_scratch[kMaxBlocks + 32];

__global__ void __launch_bounds__(kThreads)
    k_dot_noalloc(int64_t n, const double* __restrict__ x, const double* __restrict__ y,
                  double* scratch, double* result)
{
  __shared__ double red[32];
  const int64_t begin = (int64_t)blockIdx.x * kChunk;
  const int64_t end = min(n, begin + kChunk);
  double acc = 0.0;
  for (int64_t i = begin + threadIdx.x; i < end; i += kThreads) acc = fma(x[i], y[i], acc);
  const double bt = block_sum(acc, red);
  unsigned* ticket = reinterpret_cast<unsigned*>(scratch + kMaxBlocks);
  double total;
  if (grid_reduce_last(bt, scratch, ticket, red, &total) && threadIdx.x == 0) *result = total;
}

// Device address of g_noalloc_scratch per device.  Resolved at set-up (the
// first call on the device), and again on every call that is not being
// captured into a graph: the lookup allocates nothing, and a device reset
// (cudaDeviceReset, a new primary context) loads the module again at another
// address, which a cached pointer would miss.  Calls during a capture use
// the address resolved before it.
struct DeviceScratch {
  bool ready = false;
  double* ptr = nullptr;
};
DeviceScratch g_scratch[kMaxDevices];
std::mutex g_scratch_mu;

}  // namespace
}  // namespace mfe

extern "C" mfe_status mfe_dot_noalloc(int64_t n, const double* x, const double* y,
                                      double* result, void* stream)
{
  using namespace mfe;
  if (n < 0 || n > MFE_DOT_NOALLOC_MAX_N || !result || (n > 0 && (!x || !y)))
    return MFE_BAD_ARG;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return MFE_CUDA_ERR;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    cudaGetLastError();
    return MFE_CUDA_ERR;
  }
  double* scratch = nullptr;
  {
    // set-up with that device current: the host-side name g_noalloc_scratch
    // is only a stand-in, the kernel needs the device address
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch[dev].ready || cs == cudaStreamCaptureStatusNone) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || p == nullptr) {
        cudaGetLastError();
        return MFE_CUDA_ERR;
      }
      g_scratch[dev].ptr = static_cast<double*>(p);
      g_scratch[dev].ready = true;
    }
    scratch = g_scratch[dev].ptr;
  }
  // the ticket must start at zero; it may hold a stale count if an earlier
  // launch on this device did not complete
  if (cudaMemsetAsync(scratch + kMaxBlocks, 0, sizeof(double), s) != cudaSuccess) {
    cudaGetLastError();
    return MFE_CUDA_ERR;
  }
  if (n == 0) {
    if (cudaMemsetAsync(result, 0, sizeof(double), s) != cudaSuccess) {
      cudaGetLastError();
      return MFE_CUDA_ERR;
    }
    return MFE_OK;
  }
  const unsigned blocks = (unsigned)((n + kChunk - 1) / kChunk);
  k_dot_noalloc<<<blocks, kThreads, 0, s>>>(n, x, y, scratch, result);
  if (cudaGetLastError() != cudaSuccess) return MFE_CUDA_ERR;
  return MFE_OK;
}
