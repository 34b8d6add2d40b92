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

// The scalar coefficients of one LHS launch (direction and alfa fixed),
// formed on the host with the reference's expressions (src/lhs1f3d.f90:40-52,
// src/lhsf.f90:25-40, src/lhs.f90:25-33): FP64 division is slow on this part
// and correctly rounded on both sides, so no thread divides.
struct LhsCoef {
  double ak[5], bk[5];  // fourth-order band: alfa g_k / h, alfa d_k / h^2
  double ak2[3], bk2[3];  // second-order band: -alfa/2h, alfa 0, alfa/2h; alfa/h^2, -2 alfa/h^2, alfa/h^2
  double hinv, hsinv;   // 1/h, 1/h^2 (boundary rows)
};
inline LhsCoef lhs_coef(double alfa, double h) {
  LhsCoef c;
  const double gi[5] = {ga1, ga2, 0.0, ga3, ga4}, di[5] = {da1, da2, da3, da4, da5};
  for (int k = 0; k < 5; ++k) c.ak[k] = alfa * gi[k] / h, c.bk[k] = alfa * di[k] / (h * h);
  c.ak2[0] = -alfa * 0.5 / h, c.ak2[1] = alfa * 0.0, c.ak2[2] = alfa * 0.5 / h;
  c.bk2[0] = alfa / (h * h), c.bk2[1] = -alfa * 2.0 / (h * h), c.bk2[2] = alfa / (h * h);
  c.hinv = 1.0 / h, c.hsinv = 1.0 / (h * h);
  return c;
}

// Entry t (0..4) of a five-coefficient stencil, as register selects: a
// local array indexed by a thread-dependent t would live in local memory.
__host__ __device__ __forceinline__ double pick5(int t, double a0, double a1, double a2, double a3, double a4) {
  return t == 0 ? a0 : t == 1 ? a1 : t == 2 ? a2 : t == 3 ? a3 : a4;
}

struct Grid {
  int nx, ny;
  double dxi, deta;
  double Ma, Re, Pr, gamma, gamma1, omega, kz, alfa;
  int xper, yper, navier, wall, wallt, top;
  int left = -1, right = -1;             // xi boundaries when xper = 0 (7: symmetry plane)
  int nbl = 0;                           // the linear 2D nonreflecting planes act on rows j > nbl
  double gx[6], gy[6], dx2[7], dy2[7];   // interior first / second derivative stencils (src/cgrad*.f90)
  double dxinv, dyinv, dxsinv, dysinv;
};

// The left plane code of the linear 2D step's symmetry plane (its left 7):
// the mirrored stencils and symmetric xi LHS rows of left 7 (src/grad.f90:155
// with lsym from src/input.f90:235, src/lhsbt1f.f90:30-32), and besides v = 0
// and r = 0 for the second velocity component on column 1
// (src/itrbc.f90:525-527, src/rhsbc.f90:229-231).  Only the linear 2D
// context sets it.
constexpr int kLinSymLeft = 17;
// The plane codes of the linear 2D step's nonreflecting planes (its left 1
// and right 1, src/itrbc.f90:318-346, 542-566, src/rhsbc.f90:193-201,
// 242-250, src/lhsbc1f.f90:117-139, 192-221, src/lhsbc2f.f90:133-144,
// 173-184): on rows j > nbl, the density row ties rho to the outgoing
// characteristic, rho = (gamma Ma^2 rho_m c_m u - rho_m T) / T_m; the other
// rows keep the one-sided stencils and closure rows.  The per-row mean-flow
// factors are kept in tleft (column 1) and tright (column nx) as
// (gamma Ma rho_m sqrt(T_m), rho_m, T_m, gamma Ma^2 rho_m c_m).  Only the
// linear 2D context sets them.
constexpr int kLinNrLeft = 11, kLinNrRight = 21;

// symmetry planes of the xi lines (left / right 7), the d1_at / d2_at sym bits
__host__ __device__ __forceinline__ int xsym(const Grid& g) {
  return g.xper ? 0 : (g.left == 7 || g.left == kLinSymLeft ? 1 : 0) | (g.right == 7 ? 2 : 0);
}

// true when every interior stencil of g has zero outermost coefficients
inline bool narrow_stencils(const Grid& g) {
  return g.gx[0] == 0.0 && g.gx[5] == 0.0 && g.gy[0] == 0.0 && g.gy[5] == 0.0 && g.dx2[0] == 0.0 &&
         g.dx2[6] == 0.0 && g.dy2[0] == 0.0 && g.dy2[6] == 0.0;
}

// Frozen operators on the device, structure-of-arrays: element (a,b)
// (0-based) of a 5x5 operator at point p is at [(a + 5 b) * np + p], entry k
// of a 6-vector at [k * np + p].
struct Ops {
  double *Ah, *Bh, *Dh, *Dhi, *V11, *V12, *V22, *AB, *dtl;
  long long np;
  // the sponge coefficient (nx,ny): spg, or spg + spg2 for the double
  // sponge; null without a sponge
  const double* spg = nullptr;
  // the target sponges: ispg 2, 3 r += spg_a v + spg_b (v - vt) (spg_a = spg,
  // spg_b = spg2); ispg 4 r += spg_b (v - vt) (spg_b = spg + spg2); vt is
  // the complex target (5,nx,ny) as interleaved doubles
  const double* spg_a = nullptr;
  const double* spg_b = nullptr;
  const double* vt = nullptr;
  // the forced top boundary (top = 1): its wave at row ny, complex (5,nx)
  const double* ttop = nullptr;
  // the forced left boundary (left = 1, xper = 0): its wave at column 1, complex (5,ny)
  const double* tleft = nullptr;
  // the eigenfunction outflow (right = 4, xper = 0): its values at column nx, complex (5,ny)
  const double* tright = nullptr;
  // the bump wall (wall = 3): u1w, u2w, u3w, tw, twp, complex (5,nx)
  const double* bump = nullptr;
  // explicit smoother / implicit damping: eps_e buff(nx,ny); null when eps_e = 0
  const double* buff = nullptr;
  double eps_e = 0.0;
};

struct Metrics {
  const double *m1, *m2, *n1, *n2, *m11, *m12, *m22, *n11, *n12, *n22;
};

__device__ __forceinline__ long long pix(const Grid& g, int i, int j) {
  return (long long)(i - 1) + (long long)g.nx * (j - 1);
}

// First derivative along a line of n points at point i (1-based), from the
// values u(k); periodic lines have period n-1 (point n repeats point 1).
// sym: symmetry planes of a non-periodic line (bit 0 at point 1, bit 1 at
// point n, the reference's lsym / rsym): the three points next to such a
// plane take the interior stencil over the mirrored values u(2 - k),
// u(2n - k), times sgn (-1 for the component that changes sign,
// src/cgrad.f90:193-266, src/cgrad2.f90:232-307).
// NARROW: the interior stencil's outermost coefficients (offsets +-3) are zero,
// as for the fourth-order scheme (optx, opty = -1); their terms are skipped,
// and the sum is an explicit left-to-right chain of fused multiply-adds so
// that every kernel using it rounds the same way.
template <bool NARROW = false, class U>
__device__ __forceinline__ double d1_at(int i, int n, int periodic, const double* c, double dinv, U u, int sym = 0,
                                        double sgn = 1.0) {
  if (!periodic && (((sym & 1) && i <= 3) || ((sym & 2) && i >= n - 2))) {
    auto w = [&](int k) { return k < 1 ? sgn * u(2 - k) : (k > n ? sgn * u(2 * n - k) : u(k)); };
    if constexpr (NARROW) return fma(c[4], w(i + 2), fma(c[3], w(i + 1), fma(c[2], w(i - 1), c[1] * w(i - 2))));
    return c[0] * w(i - 3) + c[1] * w(i - 2) + c[2] * w(i - 1) + c[3] * w(i + 1) + c[4] * w(i + 2) + c[5] * w(i + 3);
  }
  if (periodic) {
    if (i == n) i = 1;
    auto w = [&](int k) { return k < 1 ? k + n - 1 : (k > n - 1 ? k - (n - 1) : k); };
    if constexpr (NARROW) return fma(c[4], u(w(i + 2)), fma(c[3], u(w(i + 1)), fma(c[2], u(w(i - 1)), c[1] * u(w(i - 2)))));
    return c[0] * u(w(i - 3)) + c[1] * u(w(i - 2)) + c[2] * u(w(i - 1)) + c[3] * u(w(i + 1)) + c[4] * u(w(i + 2)) +
           c[5] * u(w(i + 3));
  }
  if (i == 1) return (gc1 * u(1) + gc2 * u(2) + gc3 * u(3) + gc4 * u(4) + gc5 * u(5)) * dinv;
  if (i == 2) return (gb1 * u(1) + gb2 * u(2) + gb3 * u(3) + gb4 * u(4) + gb5 * u(5)) * dinv;
  if (i == 3) return (ga1 * u(1) + ga2 * u(2) + ga3 * u(4) + ga4 * u(5)) * dinv;
  if (i == n - 2) return (ga1 * u(n - 4) + ga2 * u(n - 3) + ga3 * u(n - 1) + ga4 * u(n)) * dinv;
  if (i == n - 1) return -((gb1 * u(n) + gb2 * u(n - 1) + gb3 * u(n - 2) + gb4 * u(n - 3) + gb5 * u(n - 4)) * dinv);
  if (i == n) return -((gc1 * u(n) + gc2 * u(n - 1) + gc3 * u(n - 2) + gc4 * u(n - 3) + gc5 * u(n - 4)) * dinv);
  if constexpr (NARROW) return fma(c[4], u(i + 2), fma(c[3], u(i + 1), fma(c[2], u(i - 1), c[1] * u(i - 2))));
  return c[0] * u(i - 3) + c[1] * u(i - 2) + c[2] * u(i - 1) + c[3] * u(i + 1) + c[4] * u(i + 2) + c[5] * u(i + 3);
}

template <bool NARROW = false, class U>
__device__ __forceinline__ double d2_at(int i, int n, int periodic, const double* c, double dsinv, U u, int sym = 0,
                                        double sgn = 1.0) {
  if (!periodic && (((sym & 1) && i <= 3) || ((sym & 2) && i >= n - 2))) {
    auto w = [&](int k) { return k < 1 ? sgn * u(2 - k) : (k > n ? sgn * u(2 * n - k) : u(k)); };
    if constexpr (NARROW)
      return fma(c[5], w(i + 2), fma(c[4], w(i + 1), fma(c[3], w(i), fma(c[2], w(i - 1), c[1] * w(i - 2)))));
    return c[0] * w(i - 3) + c[1] * w(i - 2) + c[2] * w(i - 1) + c[3] * w(i) + c[4] * w(i + 1) + c[5] * w(i + 2) +
           c[6] * w(i + 3);
  }
  if (periodic) {
    if (i == n) i = 1;
    auto w = [&](int k) { return k < 1 ? k + n - 1 : (k > n - 1 ? k - (n - 1) : k); };
    if constexpr (NARROW)
      return fma(c[5], u(w(i + 2)), fma(c[4], u(w(i + 1)), fma(c[3], u(i), fma(c[2], u(w(i - 1)), c[1] * u(w(i - 2))))));
    return c[0] * u(w(i - 3)) + c[1] * u(w(i - 2)) + c[2] * u(w(i - 1)) + c[3] * u(i) + c[4] * u(w(i + 1)) +
           c[5] * u(w(i + 2)) + c[6] * u(w(i + 3));
  }
  if (i == 1) return (dd1 * u(1) + dd2 * u(2) + dd3 * u(3) + dd4 * u(4) + dd5 * u(5)) * dsinv;
  if (i == 2) return (db1 * u(1) + db2 * u(2) + db3 * u(3) + db4 * u(4) + db5 * u(5)) * dsinv;
  if (i == 3) return (da1 * u(1) + da2 * u(2) + da3 * u(3) + da4 * u(4) + da5 * u(5)) * dsinv;
  if (i == n - 2) return (da1 * u(n - 4) + da2 * u(n - 3) + da3 * u(n - 2) + da4 * u(n - 1) + da5 * u(n)) * dsinv;
  if (i == n - 1) return (db1 * u(n) + db2 * u(n - 1) + db3 * u(n - 2) + db4 * u(n - 3) + db5 * u(n - 4)) * dsinv;
  if (i == n) return (dd1 * u(n) + dd2 * u(n - 1) + dd3 * u(n - 2) + dd4 * u(n - 3) + dd5 * u(n - 4)) * dsinv;
  if constexpr (NARROW) return fma(c[5], u(i + 2), fma(c[4], u(i + 1), fma(c[3], u(i), fma(c[2], u(i - 1), c[1] * u(i - 2)))));
  return c[0] * u(i - 3) + c[1] * u(i - 2) + c[2] * u(i - 1) + c[3] * u(i) + c[4] * u(i + 1) + c[5] * u(i + 2) +
         c[6] * u(i + 3);
}


// Kernels shared by the 3D and 2D steps (internal linkage: each translation
// unit that launches them holds its own copy).

// -------------------------------------------------------------- time step
// src/temporal.f90:40-95: acoustic CFL per point of the field vm (the mean
// flow, or the state of a nonlinear step); block maxima in part[]
static __global__ void cfl_kernel(Grid g, const double* __restrict__ vm, Metrics mt, double* dtl, double* part) {
  __shared__ double red[256];
  const long long np = (long long)g.nx * g.ny;
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  double c = -1.0;
  if (p < np) {
    const double m1 = mt.m1[p], m2 = mt.m2[p], n1 = mt.n1[p], n2 = mt.n2[p];
    double volinv = 1.0 / (m1 * n2 - m2 * n1);
    const double sxj = n2 * g.dxi * volinv, syj = -m2 * g.dxi * volinv;
    const double sxi = -n1 * g.deta * volinv, syi = m1 * g.deta * volinv;
    volinv = 1.0 / (g.dxi * g.deta * volinv);
    const double acoustic =
        sqrt(sxi * sxi + two * sxi * syi + syi * syi + sxj * sxj + two * sxj * syj + syj * syj) / g.Ma;
    const double u1 = vm[1 + 5 * p], u2 = vm[2 + 5 * p], t = sqrt(vm[4 + 5 * p]);
    c = (fabs(u1 * sxi + u2 * syi) + fabs(u1 * sxj + u2 * syj) + t * acoustic) * volinv;
    dtl[p] = c;
  }
  red[threadIdx.x] = c;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + s]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// maximum of the block maxima, then the local or global time step
static __global__ void dtl_kernel(long long np, int nparts, const double* part, double* dtl, double cflmax, double dtmax,
                           int loctime, double* cfl_out) {
  __shared__ double cfla;
  if (threadIdx.x == 0) {
    double m = -1.0;
    for (int k = 0; k < nparts; ++k) m = fmax(m, part[k]);
    cfla = m;
  }
  __syncthreads();
  const double cfl = cfla;
  const bool fixed = cfl * dtmax <= cflmax;
  const double delt = fixed ? dtmax : cflmax / cfl;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < np; p += (long long)gridDim.x * blockDim.x)
    dtl[p] = fixed ? dtmax : (loctime == 0 ? delt : cflmax / dtl[p]);
  if (blockIdx.x == 0 && threadIdx.x == 0) *cfl_out = cfl * delt;
}

// totres = sqrt(sum / (nx ny)) in a fixed summation order (src/resstat3d.f90:37-60)
static __global__ void resid_kernel(int nparts, const double* part, long long npts, double* out) {
  __shared__ double red[256];
  double s = 0.0;
  for (int k = threadIdx.x; k < nparts; k += blockDim.x) s += part[k];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *out = sqrt(red[0] / (double)npts);
  }
}

// v += r over every entry (src/impdrv3d.f90:339-347, src/impdrv.f90:381-389)
template <typename VT, typename RT>
__global__ void add_kernel(long long n, VT* __restrict__ v, const RT* __restrict__ r) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= n) return;
  v[e] = add(v[e], to_hi(r[e]));
}

}  // namespace a3
}  // namespace lns
