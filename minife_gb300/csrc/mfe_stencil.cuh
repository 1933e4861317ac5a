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

// Mirror-symmetric stencils: one weight per class 4|dz| + 2|dy| + |dx|.
// A plane of the two-row window around positions c, c + 1 (line j = dy + 1,
// v[4j .. 4j+3] = x[c-1 .. c+2], masked neighbours already zeroed) reduces
// to u[k][r]: for row c + r, the sum of the plane's values of in-plane class
// k = 2|dy| + |dx| (8 additions per plane).  A row is then
// sum_k w(k) u_B[k][r] + w(4 + k) (u_A + u_C)[k][r]: 8 FMAs, with the four
// plane sums u_A + u_C shared by both rows, instead of 27 FMAs.
struct StSep2 {
  float u[4][2];
  float c0, c1;  // unmasked centres x[c], x[c+1]
};

__device__ __forceinline__ void st_sep_reduce(const float* v, float c0, float c1, StSep2& R)
{
  float m[4], e[4];  // line y; lines y - 1 and y + 1 added
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    m[i] = v[4 + i];
    e[i] = v[i] + v[8 + i];
  }
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    R.u[0][r] = m[1 + r];
    R.u[1][r] = m[r] + m[r + 2];
    R.u[2][r] = e[1 + r];
    R.u[3][r] = e[r] + e[r + 2];
  }
  R.c0 = c0;
  R.c1 = c1;
}

// rows c, c + 1 over reduced planes A (dz = -1), B (dz = 0), C (dz = +1);
// HA / HC false: that plane is a Dirichlet plane and contributes nothing
template <bool HA, bool HC, typename WF>
__device__ __forceinline__ void st_sep_rows(WF w, const StSep2& A, const StSep2& B, const StSep2& C,
                                            float& s0, float& s1)
{
  float s[2];
#pragma unroll
  for (int r = 0; r < 2; ++r) {
    float a = w(0) * B.u[0][r];
    float b = w(1) * B.u[1][r];
    a = fmaf(w(2), B.u[2][r], a);
    b = fmaf(w(3), B.u[3][r], b);
    if (HA || HC) {
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float zk = HA && HC ? A.u[k][r] + C.u[k][r] : (HA ? A.u[k][r] : C.u[k][r]);
        if (k & 1)
          b = fmaf(w(4 + k), zk, b);
        else
          a = fmaf(w(4 + k), zk, a);
      }
    }
    s[r] = a + b;
  }
  s0 = s[0];
  s1 = s[1];
}

}  // namespace mfe
