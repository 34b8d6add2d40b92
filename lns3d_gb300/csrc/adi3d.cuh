// Kernels of the linearised single-Fourier-mode implicit ADI step
// (src/impdrv3d.f90): the fourth-order stencils with their boundary
// closures (src/cgrad.f90, src/cgrad2.f90), the frozen linear operators
// (src/genmtrx.f90, linear = 1), the time step (src/temporal.f90), the LHS
// of both sweeps (src/lhs1f3d.f90, src/lhs2f3d.f90, src/lhsbt2f3d.f90,
// src/lhsbc1f3d.f90, src/lhsbc2f3d.f90), the RHS with its boundary rows and
// residual (src/lrhs3d.f90, rbe3D, src/rhsbc3d.f90, src/resstat3d.f90) and
// the update with the boundary values (src/itrbc3d.f90).
//
// All fields keep the reference layout: v(5,nx,ny) complex (interleaved),
// vm(5,nx,ny), Ah(5,5,nx,ny), Vh(6,nx,ny), metrics (nx,ny).  One thread
// owns one grid point; a point's neighbours are read through L1.
#pragma once
#include "scalar.cuh"

namespace lns {
namespace a3 {

// src/stencil.f90:10-94
constexpr double ga1 = 8.333333333333333333333E-02, ga2 = -6.666666666666666666667E-01,
                 ga3 = 6.666666666666666666667E-01, ga4 = -8.333333333333333333333E-02;
constexpr double gc1 = -2.083333333333333333333E+00, gc2 = 4.000000000000000000000E+00,
                 gc3 = -3.000000000000000000000E+00, gc4 = 1.333333333333333333333E+00,
                 gc5 = -2.500000000000000000000E-01;
constexpr double gb1 = -2.500000000000000000000E-01, gb2 = -8.333333333333333333333E-01,
                 gb3 = 1.500000000000000000000E+00, gb4 = -5.000000000000000000000E-01,
                 gb5 = 8.333333333333333333333E-02;
constexpr double da1 = -8.333333333333333333333E-02, da2 = 1.333333333333333333333E+00,
                 da3 = -2.500000000000000000000E+00, da4 = 1.333333333333333333333E+00,
                 da5 = -8.333333333333333333333E-02;
constexpr double db1 = 9.166666666666666666667E-01, db2 = -1.666666666666666666667E+00,
                 db3 = 5.000000000000000000000E-01, db4 = 3.333333333333333333333E-01,
                 db5 = -8.333333333333333333333E-02;
constexpr double dd1 = 2.916666666666666666667E+00, dd2 = -8.666666666666666666667E+00,
                 dd3 = 9.500000000000000000000E+00, dd4 = -4.666666666666666666667E+00,
                 dd5 = 9.166666666666666666667E-01;
constexpr double pt5 = 0.5, pt66 = 6.6666666666666666666e-1, two = 2.0, four = 4.0;

struct Grid {
  int nx, ny;
  double dxi, deta;
  double Ma, Re, Pr, gamma, gamma1, omega, kz, alfa;
  int xper, yper, navier, wall, wallt, top;
  double gx[6], gy[6], dx2[7], dy2[7];   // interior first / second derivative stencils (src/cgrad*.f90)
  double dxinv, dyinv, dxsinv, dysinv;
};

__device__ __forceinline__ long long pix(const Grid& g, int i, int j) {
  return (long long)(i - 1) + (long long)g.nx * (j - 1);
}

// First derivative along a line of n points at point i (1-based), from the
// values u(k); periodic lines have period n-1 (point n repeats point 1).
template <class U>
__device__ __forceinline__ double d1_at(int i, int n, int periodic, const double* c, double dinv, U u) {
  if (periodic) {
    if (i == n) i = 1;
    auto w = [&](int k) { return k < 1 ? k + n - 1 : (k > n - 1 ? k - (n - 1) : k); };
    return c[0] * u(w(i - 3)) + c[1] * u(w(i - 2)) + c[2] * u(w(i - 1)) + c[3] * u(w(i + 1)) + c[4] * u(w(i + 2)) +
           c[5] * u(w(i + 3));
  }
  if (i == 1) return (gc1 * u(1) + gc2 * u(2) + gc3 * u(3) + gc4 * u(4) + gc5 * u(5)) * dinv;
  if (i == 2) return (gb1 * u(1) + gb2 * u(2) + gb3 * u(3) + gb4 * u(4) + gb5 * u(5)) * dinv;
  if (i == 3) return (ga1 * u(1) + ga2 * u(2) + ga3 * u(4) + ga4 * u(5)) * dinv;
  if (i == n - 2) return (ga1 * u(n - 4) + ga2 * u(n - 3) + ga3 * u(n - 1) + ga4 * u(n)) * dinv;
  if (i == n - 1) return -((gb1 * u(n) + gb2 * u(n - 1) + gb3 * u(n - 2) + gb4 * u(n - 3) + gb5 * u(n - 4)) * dinv);
  if (i == n) return -((gc1 * u(n) + gc2 * u(n - 1) + gc3 * u(n - 2) + gc4 * u(n - 3) + gc5 * u(n - 4)) * dinv);
  return c[0] * u(i - 3) + c[1] * u(i - 2) + c[2] * u(i - 1) + c[3] * u(i + 1) + c[4] * u(i + 2) + c[5] * u(i + 3);
}

template <class U>
__device__ __forceinline__ double d2_at(int i, int n, int periodic, const double* c, double dsinv, U u) {
  if (periodic) {
    if (i == n) i = 1;
    auto w = [&](int k) { return k < 1 ? k + n - 1 : (k > n - 1 ? k - (n - 1) : k); };
    return c[0] * u(w(i - 3)) + c[1] * u(w(i - 2)) + c[2] * u(w(i - 1)) + c[3] * u(i) + c[4] * u(w(i + 1)) +
           c[5] * u(w(i + 2)) + c[6] * u(w(i + 3));
  }
  if (i == 1) return (dd1 * u(1) + dd2 * u(2) + dd3 * u(3) + dd4 * u(4) + dd5 * u(5)) * dsinv;
  if (i == 2) return (db1 * u(1) + db2 * u(2) + db3 * u(3) + db4 * u(4) + db5 * u(5)) * dsinv;
  if (i == 3) return (da1 * u(1) + da2 * u(2) + da3 * u(3) + da4 * u(4) + da5 * u(5)) * dsinv;
  if (i == n - 2) return (da1 * u(n - 4) + da2 * u(n - 3) + da3 * u(n - 2) + da4 * u(n - 1) + da5 * u(n)) * dsinv;
  if (i == n - 1) return (db1 * u(n) + db2 * u(n - 1) + db3 * u(n - 2) + db4 * u(n - 3) + db5 * u(n - 4)) * dsinv;
  if (i == n) return (dd1 * u(n) + dd2 * u(n - 1) + dd3 * u(n - 2) + dd4 * u(n - 3) + dd5 * u(n - 4)) * dsinv;
  return c[0] * u(i - 3) + c[1] * u(i - 2) + c[2] * u(i - 1) + c[3] * u(i) + c[4] * u(i + 1) + c[5] * u(i + 2) +
         c[6] * u(i + 3);
}

}  // namespace a3
}  // namespace lns
