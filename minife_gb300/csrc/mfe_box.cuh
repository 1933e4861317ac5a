// Closed-form CSR layout of the 27-point node box (one rank).
//
// generate_matrix_structure (ref/src/generate_matrix_structure.hpp:98-125)
// and MatrixInitOp<CSR> (ref/src/MatrixInitOp.hpp:127-156) count and list each
// row's in-box neighbours one row at a time; the counts factor per dimension,
// so every row's offset and every nonzero's position follow in closed form.
#pragma once

#include <cstdint>

namespace mfe {

// Nonzeros contributed by node coordinates < i along a dimension of n nodes:
// sum_{j<i} (1 + [j>0] + [j<n-1]).
__host__ __device__ __forceinline__ int64_t pre_count(int64_t i, int64_t n)
{
  return i + (i > 0 ? i - 1 : 0) + (i < n - 1 ? i : n - 1);
}

// In-box neighbours (itself included) of coordinate i along n nodes.
__host__ __device__ __forceinline__ int nbr(int i, int n)
{
  return 1 + (i > 0) + (i < n - 1);
}

// CSR offset of node (ix, iy, iz) in the Nx x Ny x Nz node box.
__host__ __device__ __forceinline__ int64_t row_offset(int ix, int iy, int iz, int Nx, int Ny,
                                                       int Nz)
{
  const int64_t Sx = 3 * (int64_t)Nx - 2, Sy = 3 * (int64_t)Ny - 2;
  return pre_count(iz, Nz) * Sy * Sx + (int64_t)nbr(iz, Nz) * pre_count(iy, Ny) * Sx +
         (int64_t)nbr(iz, Nz) * nbr(iy, Ny) * pre_count(ix, Nx);
}

// Offset of row r (r == Nx*Ny*Nz gives the total nonzero count).
__host__ __device__ __forceinline__ int64_t row_offset_of(int64_t r, int Nx, int Ny, int Nz)
{
  const int64_t NxNy = (int64_t)Nx * Ny;
  if (r >= NxNy * Nz)
    return (3 * (int64_t)Nx - 2) * (3 * (int64_t)Ny - 2) * (3 * (int64_t)Nz - 2);
  return row_offset((int)(r % Nx), (int)((r / Nx) % Ny), (int)(r / NxNy), Nx, Ny, Nz);
}

// 32-bit variant for rows < 2^31 (every box the library accepts).
__host__ __device__ __forceinline__ int64_t row_offset_of32(int r, int Nx, int Ny, int Nz, int NxNy)
{
  if (r >= NxNy * Nz)
    return (3 * (int64_t)Nx - 2) * (3 * (int64_t)Ny - 2) * (3 * (int64_t)Nz - 2);
  const int iz = r / NxNy;
  const int rem = r - iz * NxNy;
  const int iy = rem / Nx;
  return row_offset(rem - iy * Nx, iy, iz, Nx, Ny, Nz);
}

}  // namespace mfe
