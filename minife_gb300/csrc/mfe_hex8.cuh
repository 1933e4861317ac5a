// Hex8 element math on the device, in the reference's floating-point
// operation order (ref/fem/Hex8.hpp).  The translation unit that includes
// this header is compiled with -fmad=false, so every multiply and add is
// rounded separately exactly as in the reference's g++ build, and division is
// IEEE round-to-nearest; element matrices and source vectors are therefore
// bit-identical to the reference's.
#pragma once

#include <cstdint>

namespace mfe {

// 2x2x2 Gauss points from gauss_pts(2) (ref/fem/gauss_pts.hpp:41,50-53): the
// truncated constant 0.577350269, weights 1.0.
constexpr double kGaussPt = 0.577350269;

// Reference-element shape-function gradients at the 8 Gauss points
// (compute_gradient_values, ref/fem/Hex8_ElemData.hpp:37-61), laid out
// [gp][node][dim]; gp = ig*4 + jg*2 + kg with pt = (gpts[ig], gpts[jg],
// gpts[kg]).  Filled once by the host (same expression order as
// Hex8::gradients, Hex8.hpp:68-113; products of constants, no adds to fuse).
struct Hex8Tables {
  double grad[8][8][3];
  double psi[8][8];  // shape_fns at each Gauss point (Hex8.hpp:44-65)
};

// Element node coordinates (get_elem_nodes_and_coords,
// ref/src/Hex8_box_utils.hpp:101-159 with get_coords, box_utils.hpp:64-82):
// node 0 at (ex/nx, ey/ny, ez/nz), the others at + h = 1/n per dimension.
struct ElemCorner {
  double x0, x1, y0, y1, z0, z1;
};

__device__ __forceinline__ ElemCorner elem_corner(int ex, int ey, int ez, int nx, int ny, int nz)
{
  ElemCorner c;
  // xdiv = Nx - 1 = nx (nx >= 1 for every assembled box)
  c.x0 = (1.0 * (double)ex) / (double)nx;
  c.y0 = 1.0 * (double)ey / (double)ny;
  c.z0 = (1.0 * (double)ez) / (double)nz;
  c.x1 = c.x0 + 1.0 / nx;
  c.y1 = c.y0 + 1.0 / ny;
  c.z1 = c.z0 + 1.0 / nz;
  return c;
}

// Coordinates of local node i (get_hex8_node_coords_3d order).
__device__ __forceinline__ void node_xyz(const ElemCorner& c, int i, double& x, double& y,
                                         double& z)
{
  const bool hx = (i == 1 || i == 2 || i == 5 || i == 6);
  const bool hy = (i == 2 || i == 3 || i == 6 || i == 7);
  const bool hz = (i >= 4);
  x = hx ? c.x1 : c.x0;
  y = hy ? c.y1 : c.y0;
  z = hz ? c.z1 : c.z0;
}

// Jacobian at one Gauss point (Hex8.hpp:198-236): J += grad * coord in node
// order 0..7.
__device__ __forceinline__ void jacobian(const ElemCorner& c, const double (*g)[3],
                                         double J[9])
{
  double J00 = 0, J01 = 0, J02 = 0, J10 = 0, J11 = 0, J12 = 0, J20 = 0, J21 = 0, J22 = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    double x, y, z;
    node_xyz(c, i, x, y, z);
    const double g0 = g[i][0], g1 = g[i][1], g2 = g[i][2];
    J00 += g0 * x; J01 += g0 * y; J02 += g0 * z;
    J10 += g1 * x; J11 += g1 * y; J12 += g1 * z;
    J20 += g2 * x; J21 += g2 * y; J22 += g2 * z;
  }
  J[0] = J00; J[1] = J01; J[2] = J02; J[3] = J10; J[4] = J11; J[5] = J12;
  J[6] = J20; J[7] = J21; J[8] = J22;
}

// diffusionMatrix_symm (Hex8.hpp:260-361) with conductivity k, and
// sourceVector (Hex8.hpp:364-410).  em: 36 upper-triangle entries, row-major;
// ev: 8 entries.  Both loops walk the Gauss points in the same order and
// compute the same Jacobian, so they share it.  jf(gp, J) provides the
// Jacobian at Gauss point gp (jacobian() from the corner coordinates, or the
// same values from per-axis tables, jacobian_column()).
template <typename JF>
__device__ __forceinline__ void element_matrix_vector_j(const Hex8Tables& T, JF jf, double k,
                                                        double em[36], double ev[8])
{
#pragma unroll
  for (int i = 0; i < 36; ++i) em[i] = 0.0;
#pragma unroll
  for (int i = 0; i < 8; ++i) ev[i] = 0.0;

#pragma unroll 1
  for (int gp = 0; gp < 8; ++gp) {
    const double (*g)[3] = T.grad[gp];
    double J[9];
    jf(gp, J);
    const double J00 = J[0], J01 = J[1], J02 = J[2], J10 = J[3], J11 = J[4], J12 = J[5],
                 J20 = J[6], J21 = J[7], J22 = J[8];
    const double term0 = J22 * J11 - J21 * J12;
    const double term1 = J22 * J01 - J21 * J02;
    const double term2 = J12 * J01 - J11 * J02;
    const double detJ = J00 * term0 - J10 * term1 + J20 * term2;
    const double inv_detJ = 1.0 / detJ;
    double iJ[9];
    iJ[0] = term0 * inv_detJ;
    iJ[1] = -term1 * inv_detJ;
    iJ[2] = term2 * inv_detJ;
    iJ[3] = -(J22 * J10 - J20 * J12) * inv_detJ;
    iJ[4] = (J22 * J00 - J20 * J02) * inv_detJ;
    iJ[5] = -(J12 * J00 - J10 * J02) * inv_detJ;
    iJ[6] = (J21 * J10 - J20 * J11) * inv_detJ;
    iJ[7] = -(J21 * J00 - J20 * J01) * inv_detJ;
    iJ[8] = (J11 * J00 - J10 * J01) * inv_detJ;

    // weights are 1.0: wi_wj_wk = 1*1*1 (Hex8.hpp:293-299)
    const double k_detJ_w = k * detJ * 1.0;
    double dx[8], dy[8], dz[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const double g0 = g[i][0], g1 = g[i][1], g2 = g[i][2];
      dx[i] = g0 * iJ[0] + g1 * iJ[1] + g2 * iJ[2];
      dy[i] = g0 * iJ[3] + g1 * iJ[4] + g2 * iJ[5];
      dz[i] = g0 * iJ[6] + g1 * iJ[7] + g2 * iJ[8];
    }
    int off = 0;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      em[off] += k_detJ_w * ((dx[m] * dx[m]) + (dy[m] * dy[m]) + (dz[m] * dz[m]));
      ++off;
#pragma unroll
      for (int n = m + 1; n < 8; ++n) {
        em[off] += k_detJ_w * ((dx[m] * dx[n]) + (dy[m] * dy[n]) + (dz[m] * dz[n]));
        ++off;
      }
    }
    // sourceVector: term = Q*detJ*wi*wj*wk with Q = 1 (Hex8.hpp:402)
    const double term = 1.0 * detJ * 1.0 * 1.0 * 1.0;
#pragma unroll
    for (int i = 0; i < 8; ++i) ev[i] += T.psi[gp][i] * term;
  }
}

__device__ __forceinline__ void element_matrix_vector(const Hex8Tables& T, const ElemCorner& c,
                                                      double k, double em[36], double ev[8])
{
  element_matrix_vector_j(T, [&](int gp, double J[9]) { jacobian(c, T.grad[gp], J); }, k, em, ev);
}

// The Jacobian's column for physical axis x (entries J[a][0], a = 0..2) sums
// grad[gp][i][a] * x_i over the element's 8 nodes, whose x is x0 or x1: it
// depends on the element's x pair only, and likewise for y and z.  Computed
// with jacobian()'s operations in its order (node order, from 0), the column
// of an element index along an axis is therefore exact for every element of
// that index.  axis: 0 x, 1 y, 2 z; (c0, c1) the index's coordinate pair.
__device__ __forceinline__ void jacobian_column(const Hex8Tables& T, int axis, double c0, double c1,
                                                int gp, double col[3])
{
  double s0 = 0, s1 = 0, s2 = 0;
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const bool hi = axis == 0 ? (i == 1 || i == 2 || i == 5 || i == 6)
                              : (axis == 1 ? (i == 2 || i == 3 || i == 6 || i == 7) : (i >= 4));
    const double v = hi ? c1 : c0;
    s0 += T.grad[gp][i][0] * v;
    s1 += T.grad[gp][i][1] * v;
    s2 += T.grad[gp][i][2] * v;
  }
  col[0] = s0;
  col[1] = s1;
  col[2] = s2;
}

// Index of (a, b) in the 36-entry upper triangle (a, b in 0..7).
__host__ __device__ constexpr int sym_index(int a, int b)
{
  return a <= b ? a * 8 - (a * (a - 1)) / 2 + (b - a) : b * 8 - (b * (b - 1)) / 2 + (a - b);
}

// Local node index (exodus order, Hex8_box_utils.hpp:49-56) of the corner
// at offset (ox, oy, oz) in {0,1}^3 from the element's node 0.
__host__ __device__ constexpr int local_node(int ox, int oy, int oz)
{
  return oz * 4 + (oy ? (ox ? 2 : 3) : (ox ? 1 : 0));
}

}  // namespace mfe
