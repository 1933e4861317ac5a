// Device pieces shared by the FP32 stencil SpMVs of the mixed solvers (one
// box: mfe_stencil.cu; batched boxes: mfe_batch.cu).  The operator model and
// its verification are described in mfe_stencil.cu.
#pragma once

#include <cstdint>

namespace mfe {

constexpr int kSP = 256;                  // plane positions per CTA (one per consumer thread)
constexpr int kSC = kSP / 32;             // consumer warps
constexpr int kSS = 4;                    // ring slots
constexpr int kSKP = 3;                   // planes per slot
constexpr int kSCap = ((kSP + 2 + 6) + 3) & ~3;  // floats per line segment: 16-byte multiple
constexpr int kSSlot = kSKP * 3 * kSCap;  // three y lines per plane
constexpr size_t kStSmem = sizeof(float) * kSS * kSSlot;  // the ring (dynamic shared memory)
static_assert((kSCap * sizeof(float)) % 16 == 0 && kSCap >= kSP + 8,
              "bulk-copy destinations in shared memory must stay 16-byte aligned");

// coordinate class along a dimension of N nodes: first, second, interior,
// second-last, last
__host__ __device__ __forceinline__ int st_cls(int i, int N)
{
  return i == 0 ? 0 : (i == N - 1 ? 4 : (i == 1 ? 1 : (i == N - 2 ? 3 : 2)));
}

// nine values of one plane around a position, q = 3 * (dy + 1) + (dx + 1)
struct StPlane {
  float v[9];
};

// interior-stencil row sum over planes A (dz = -1), B (dz = 0), C (dz = +1);
// HA / HC false: that plane is a Dirichlet plane and contributes nothing.
// cf(k) is coefficient k in slot order (dz, dy, dx).
template <bool HA, bool HC, typename CF>
__device__ __forceinline__ float st_sum(CF cf, const StPlane& A, const StPlane& B, const StPlane& C)
{
  float a[6] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int k = 0; k < 9; ++k) {
    if (HA) a[k & 1] = fmaf(cf(k), A.v[k], a[k & 1]);
    a[2 + (k & 1)] = fmaf(cf(9 + k), B.v[k], a[2 + (k & 1)]);
    if (HC) a[4 + (k & 1)] = fmaf(cf(18 + k), C.v[k], a[4 + (k & 1)]);
  }
  return ((a[0] + a[1]) + (a[2] + a[3])) + (a[4] + a[5]);
}

// row z's sum with the warp-uniform z boundary cases: Dirichlet planes give
// dd * x, the planes next to them drop the Dirichlet neighbour plane
template <typename CF>
__device__ __forceinline__ float st_row_sum(CF cf, float dd, int z, int Nz, const StPlane& A,
                                            const StPlane& B, const StPlane& C)
{
  if (z >= 2 && z <= Nz - 3) return st_sum<true, true>(cf, A, B, C);
  if (z == 0 || z == Nz - 1) return dd * B.v[4];
  if (z == 1 && z == Nz - 2) return st_sum<false, false>(cf, A, B, C);
  if (z == 1) return st_sum<false, true>(cf, A, B, C);
  return st_sum<true, false>(cf, A, B, C);
}

}  // namespace mfe
