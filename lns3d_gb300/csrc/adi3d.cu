// The linearised single-Fourier-mode implicit ADI step on the GPU
// (src/impdrv3d.f90:130-356 with impl = 1, iLHS = 1) and its C ABI
// (lns_ctx3d_*, include/lns3d_gb300.h).
//
// A context owns everything the step needs on the device: the frozen
// operators (built once from the mean flow by genmtrx_kernel, or uploaded),
// the local time step, the two factored LHS (factored once, at the first
// step, as the reference does), and the disturbance.  A step is
//   c1v = d v/d xi                                     grad1_kernel
//   r = vold - v - dtl L(v), boundary rows, residual    rhs_kernel
//   xi sweep, eta sweep (stored factors)                penta_solve_kernel
//   v += r, boundary values                             add_kernel, bc_kernel
// In the mixed-precision mode the factors and the sweeps are FP32 and the
// RHS, residual and update stay FP64.
#include <cuda_runtime.h>

#include <algorithm>
#include <complex>
#include <chrono>
#include <cmath>
#include <deque>
#include <map>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/lns3d_gb300.h"
#include "adi3d.cuh"
#include "launch.cuh"
#include "penta_chain.cuh"

namespace lns {
namespace a3 {

__device__ __forceinline__ double& opel(double* A, const Ops& o, int a, int b, long long p) {
  return A[(long long)(a + 5 * b) * o.np + p];
}

// ------------------------------------------------------------------ genmtrx
// src/genmtrx.f90 with linear = 1, general = true, mattyp = 0, idamp = 0,
// complex_analysis = true; one thread per point.
__global__ void genmtrx_kernel(Grid g, const double* __restrict__ vm, Metrics mt, Ops o) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y + 1;
  if (i > g.nx) return;
  const long long p = pix(g, i, j);
  auto V = [&](int k, int ii, int jj) { return vm[k + 5 * pix(g, ii, jj)]; };
  double g1v[5], g2v[5], g11v[5], g12v[5], g22v[5];
  for (int k = 0; k < 5; ++k) {
    g1v[k] = d1_at(i, g.nx, g.xper, g.gx, g.dxinv, [&](int ii) { return V(k, ii, j); });
    g2v[k] = d1_at(j, g.ny, g.yper, g.gy, g.dyinv, [&](int jj) { return V(k, i, jj); });
    g11v[k] = d2_at(i, g.nx, g.xper, g.dx2, g.dxsinv, [&](int ii) { return V(k, ii, j); });
    g22v[k] = d2_at(j, g.ny, g.yper, g.dy2, g.dysinv, [&](int jj) { return V(k, i, jj); });
    g12v[k] = d1_at(j, g.ny, g.yper, g.gy, g.dyinv, [&](int jj) {
      return d1_at(i, g.nx, g.xper, g.gx, g.dxinv, [&](int ii) { return V(k, ii, jj); });
    });
  }
  if (g.navier && !g.yper && (g.wallt == 1 || g.wallt == 2) && j == 1) g2v[4] = 0.0;  // src/gradbc.f90
  const double m1 = mt.m1[p], m2 = mt.m2[p], n1 = mt.n1[p], n2 = mt.n2[p];
  const double m11 = mt.m11[p], m12 = mt.m12[p], m22 = mt.m22[p], n11 = mt.n11[p], n12 = mt.n12[p], n22 = mt.n22[p];
  const double m1m1 = m1 * m1, m1m2 = m1 * m2, m2m2 = m2 * m2, n1n1 = n1 * n1, n1n2 = n1 * n2, n2n2 = n2 * n2;
  const double m1n1 = m1 * n1, m1n2 = m1 * n2, m2n1 = m2 * n1, m2n2 = m2 * n2;
  double g1vl[5], g2vl[5], g11vl[5], g12vl[5], g22vl[5];
  for (int k = 0; k < 5; ++k) {  // src/genmtrx.f90:116-136
    g11vl[k] = g11v[k] * m1m1 + two * g12v[k] * m1n1 + g22v[k] * n1n1 + g1v[k] * m11 + g2v[k] * n11;
    g12vl[k] = g11v[k] * m1m2 + g12v[k] * (m1n2 + m2n1) + g22v[k] * n1n2 + g1v[k] * m12 + g2v[k] * n12;
    g22vl[k] = g11v[k] * m2m2 + two * g12v[k] * m2n2 + g22v[k] * n2n2 + g1v[k] * m22 + g2v[k] * n22;
    g1vl[k] = g1v[k] * m1 + g2v[k] * n1;
    g2vl[k] = g1v[k] * m2 + g2v[k] * n2;
  }
  const double rho = V(0, i, j), u1 = V(1, i, j), u2 = V(2, i, j), u3 = V(3, i, j), t = V(4, i, j);
  const double rhoinv = 1.0 / rho;
  const double grho[3] = {g1vl[0], g2vl[0], 0.0};
  const double gu[3][3] = {{g1vl[1], g2vl[1], 0.0}, {g1vl[2], g2vl[2], 0.0}, {g1vl[3], g2vl[3], 0.0}};
  const double gt[3] = {g1vl[4], g2vl[4], 0.0};
  const double g1divu = g11vl[1] + g12vl[2], g2divu = g12vl[1] + g22vl[2], g3divu = 0.0;
  const double S1jj = pt5 * (g11vl[1] + g11vl[1] + g22vl[1] + g12vl[2]);
  const double S2jj = pt5 * (g11vl[2] + g12vl[1] + g22vl[2] + g22vl[2]);
  const double S3jj = pt5 * (g11vl[3] + g22vl[3]);
  const double Lapt = g11vl[4] + g22vl[4];
  const double divu = gu[0][0] + gu[1][1] + gu[2][2];
  double S[3][3] = {{gu[0][0], pt5 * (gu[0][1] + gu[1][0]), pt5 * gu[2][0]},
                    {pt5 * (gu[1][0] + gu[0][1]), gu[1][1], pt5 * gu[2][1]},
                    {pt5 * gu[2][0], pt5 * gu[2][1], 0.0}};
  // getmat, src/getmat.f90:11-20 (mattyp 0)
  const double mu = 1.0, dmu = 0.0, d2mu = 0.0, con = mu, dcon = dmu, d2con = d2mu;
  const double lm = -pt66 * mu, dlm = -pt66 * dmu, d2lm = -pt66 * d2mu;
  const double g1mu = dmu * gt[0], g2mu = dmu * gt[1], g3mu = dmu * gt[2];
  const double g1dmu = d2mu * gt[0], g2dmu = d2mu * gt[1], g3dmu = d2mu * gt[2];
  const double g1con = dcon * gt[0], g2con = dcon * gt[1], g3con = dcon * gt[2];
  const double g1dcon = d2con * gt[0], g2dcon = d2con * gt[1], g3dcon = d2con * gt[2];
  const double g1lm = dlm * gt[0], g2lm = dlm * gt[1], g3lm = dlm * gt[2];
  const double g1dlm = d2lm * gt[0], g2dlm = d2lm * gt[1], g3dlm = d2lm * gt[2];
  const double gamma = g.gamma, gamma1 = g.gamma1, Ma2 = g.Ma * g.Ma, Re = g.Re, Pr = g.Pr, kzl = g.kz;
  double A[5][5] = {}, B[5][5] = {}, C[5][5] = {}, D[5][5] = {}, Vij[4];
  double fact1 = rhoinv / Re, fact2;
  const double gmsinv = 1.0 / (gamma * Ma2);
  // A, src/genmtrx.f90:463-507
  A[0][0] = u1; A[0][1] = rho;
  A[1][0] = rhoinv * t * gmsinv;
  A[1][1] = u1 - fact1 * g1lm - fact1 * two * g1mu;
  A[1][2] = -(fact1 * g2mu);
  A[1][3] = -(fact1 * g3mu);
  A[1][4] = gmsinv - fact1 * dlm * divu - fact1 * dmu * two * S[0][0];
  A[2][1] = -(fact1 * g2lm);
  A[2][2] = u1 - fact1 * g1mu;
  A[2][4] = -(fact1 * dmu * two * S[1][0]);
  A[3][1] = -(fact1 * g3lm);
  A[3][3] = u1 - fact1 * g1mu;
  A[3][4] = -(fact1 * dmu * two * S[2][0]);
  // B, src/genmtrx.f90:530-574
  B[0][0] = u2; B[0][2] = rho;
  B[1][1] = u2 - fact1 * g2mu;
  B[1][2] = -(fact1 * g1lm);
  B[1][4] = -(fact1 * dmu * two * S[0][1]);
  B[2][0] = rhoinv * t * gmsinv;
  B[2][1] = -(fact1 * g1mu);
  B[2][2] = u2 - fact1 * g2lm - fact1 * two * g2mu;
  B[2][3] = -(fact1 * g3mu);
  B[2][4] = gmsinv - fact1 * dlm * divu - fact1 * dmu * two * S[1][1];
  B[3][2] = -(fact1 * g3lm);
  B[3][3] = u2 - fact1 * g2mu;
  B[3][4] = -(fact1 * dmu * two * S[2][1]);
  // C, src/genmtrx.f90:929-973
  C[0][0] = u3; C[0][3] = rho;
  C[1][1] = u3 - fact1 * g3mu;
  C[1][3] = -(fact1 * g1lm);
  C[1][4] = -(fact1 * dmu * two * S[0][2]);
  C[2][2] = u3 - fact1 * g3mu;
  C[2][3] = -(fact1 * g2lm);
  C[2][4] = -(fact1 * dmu * two * S[1][2]);
  C[3][0] = rhoinv * t * gmsinv;
  C[3][1] = -(fact1 * g1mu);
  C[3][2] = -(fact1 * g2mu);
  C[3][3] = u3 - fact1 * g3lm - fact1 * two * g3mu;
  C[3][4] = gmsinv - fact1 * dlm * divu - fact1 * dmu * two * S[2][2];
  // D, src/genmtrx.f90:708-780 (linear = 1)
  D[0][0] = divu; D[0][1] = grho[0]; D[0][2] = grho[1]; D[0][3] = grho[2];
  D[1][0] = rhoinv * (u1 * gu[0][0] + u2 * gu[0][1] + u3 * gu[0][2] + gmsinv * gt[0]);
  D[1][1] = gu[0][0]; D[1][2] = gu[0][1]; D[1][3] = gu[0][2];
  D[1][4] = rhoinv * gmsinv * grho[0] - fact1 * (g1dlm * divu + dlm * g1divu) -
            fact1 * two * (g1dmu * S[0][0] + g2dmu * S[0][1] + g3dmu * S[0][2] + dmu * S1jj);
  D[2][0] = rhoinv * (u1 * gu[1][0] + u2 * gu[1][1] + u3 * gu[1][2] + gmsinv * gt[1]);
  D[2][1] = gu[1][0]; D[2][2] = gu[1][1]; D[2][3] = gu[1][2];
  D[2][4] = rhoinv * gmsinv * grho[1] - fact1 * (g2dlm * divu + dlm * g2divu) -
            fact1 * two * (g1dmu * S[1][0] + g2dmu * S[1][1] + g3dmu * S[1][2] + dmu * S2jj);
  D[3][0] = rhoinv * (u1 * gu[2][0] + u2 * gu[2][1] + u3 * gu[2][2] + gmsinv * gt[2]);
  D[3][1] = gu[2][0]; D[3][2] = gu[2][1]; D[3][3] = gu[2][2];
  D[3][4] = rhoinv * gmsinv * grho[2] - fact1 * (g3dlm * divu + dlm * g3divu) -
            fact1 * two * (g1dmu * S[2][0] + g2dmu * S[2][1] + g3dmu * S[2][2] + dmu * S3jj);
  fact1 = gamma * rhoinv / (Pr * Re);
  fact2 = gamma * gamma1 * Ma2 * rhoinv / Re;
  A[4][1] = gamma1 * t - fact2 * two * lm * divu - four * fact2 * mu * S[0][0];
  A[4][2] = -(four * fact2 * mu * S[1][0]);
  A[4][3] = -(four * fact2 * mu * S[2][0]);
  A[4][4] = u1 - fact1 * (g1con + dcon * gt[0]);
  B[4][1] = -(four * fact2 * mu * S[0][1]);
  B[4][2] = gamma1 * t - fact2 * two * lm * divu - four * fact2 * mu * S[1][1];
  B[4][3] = -(four * fact2 * mu * S[2][1]);
  B[4][4] = u2 - fact1 * (g2con + dcon * gt[1]);
  C[4][1] = -(four * fact2 * mu * S[0][2]);
  C[4][2] = -(four * fact2 * mu * S[1][2]);
  C[4][3] = gamma1 * t - fact2 * two * lm * divu - four * fact2 * mu * S[2][2];
  C[4][4] = u3 - fact1 * (g3con + dcon * gt[2]);
  D[4][0] = rhoinv * (u1 * gt[0] + u2 * gt[1] + u3 * gt[2] + gamma1 * t * divu);
  D[4][1] = gt[0]; D[4][2] = gt[1]; D[4][3] = gt[2];
  {
    const double ssq = S[0][0] * S[0][0] + S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][0] * S[1][0] +
                       S[1][1] * S[1][1] + S[1][2] * S[1][2] + S[2][0] * S[2][0] + S[2][1] * S[2][1] +
                       S[2][2] * S[2][2];
    D[4][4] = -(gamma1 * rhoinv * (u1 * grho[0] + u2 * grho[1] + u3 * grho[2]));
    D[4][4] = D[4][4] - fact1 * (g1dcon * gt[0] + g2dcon * gt[1] + g3dcon * gt[2] + dcon * Lapt) -
              fact2 * dlm * (divu * divu) - two * fact2 * dmu * ssq;
  }
  // Vij, src/genmtrx.f90:590-600
  fact1 = 1.0 / Re;
  fact2 = gamma / (Pr * Re);
  Vij[0] = fact1 * rhoinv * (lm + two * mu);
  Vij[1] = fact1 * rhoinv * mu;
  Vij[2] = fact2 * rhoinv * con;
  Vij[3] = fact1 * rhoinv * (lm + mu);
  // \hat{A}, \hat{B}, src/genmtrx.f90:608-694
  for (int pass = 0; pass < 2; ++pass) {
    double* H = pass == 0 ? o.Ah : o.Bh;
    const double e1 = pass == 0 ? m1 : n1, e2 = pass == 0 ? m2 : n2;
    const double e11 = pass == 0 ? m11 : n11, e12 = pass == 0 ? m12 : n12, e22 = pass == 0 ? m22 : n22;
    double h[5][5];
    h[0][0] = A[0][0] * e1 + B[0][0] * e2; h[0][1] = A[0][1] * e1; h[0][2] = B[0][2] * e2; h[0][3] = 0.0; h[0][4] = 0.0;
    h[1][0] = A[1][0] * e1;
    h[1][1] = A[1][1] * e1 + B[1][1] * e2 - Vij[0] * e11 - Vij[1] * e22;
    h[1][2] = A[1][2] * e1 + B[1][2] * e2 - Vij[3] * e12;
    h[1][3] = A[1][3] * e1;
    h[1][4] = A[1][4] * e1 + B[1][4] * e2;
    h[2][0] = B[2][0] * e2;
    h[2][1] = A[2][1] * e1 + B[2][1] * e2 - Vij[3] * e12;
    h[2][2] = A[2][2] * e1 + B[2][2] * e2 - Vij[1] * e11 - Vij[0] * e22;
    h[2][3] = B[2][3] * e2;
    h[2][4] = A[2][4] * e1 + B[2][4] * e2;
    h[3][0] = 0.0;
    h[3][1] = A[3][1] * e1;
    h[3][2] = B[3][2] * e2;
    h[3][3] = A[3][3] * e1 + B[3][3] * e2 - Vij[1] * e11 - Vij[1] * e22;
    h[3][4] = A[3][4] * e1 + B[3][4] * e2;
    for (int b = 0; b < 4; ++b) h[4][b] = A[4][b] * e1 + B[4][b] * e2;
    h[4][4] = A[4][4] * e1 + B[4][4] * e2 - Vij[2] * e11 - Vij[2] * e22;
    if (pass == 1 && !g.yper && g.wallt == 2 && j == 1)
      for (int a = 0; a < 5; ++a) h[a][4] = 0.0;
    for (int a = 0; a < 5; ++a)
      for (int b = 0; b < 5; ++b) opel(H, o, a, b, p) = h[a][b];
  }
  if (kzl != 0.0) {  // src/genmtrx.f90:843-848
    D[1][1] = D[1][1] + (kzl * kzl) * Vij[1];
    D[2][2] = D[2][2] + (kzl * kzl) * Vij[1];
    D[3][3] = D[3][3] + (kzl * kzl) * Vij[0];
    D[4][4] = D[4][4] + (kzl * kzl) * Vij[2];
  }
  for (int a = 0; a < 5; ++a)
    for (int b = 0; b < 5; ++b) {
      opel(o.Dh, o, a, b, p) = D[a][b];
      opel(o.Dhi, o, a, b, p) = kzl * C[a][b] - (a == b ? g.omega : 0.0);
    }
  // \hat{V}, src/genmtrx.f90:867-913; 3D terms :919-925
  const long long np = o.np;
  o.V11[0 * np + p] = Vij[0] * m1m1 + Vij[1] * m2m2;
  o.V11[1 * np + p] = Vij[1] * m1m1 + Vij[0] * m2m2;
  o.V11[2 * np + p] = Vij[1] * m1m1 + Vij[1] * m2m2;
  o.V11[3 * np + p] = Vij[2] * m1m1 + Vij[2] * m2m2;
  o.V11[4 * np + p] = Vij[3] * m1m2;
  o.V11[5 * np + p] = Vij[3] * m1m2;
  o.V12[0 * np + p] = two * (Vij[0] * m1n1 + Vij[1] * m2n2);
  o.V12[1 * np + p] = two * (Vij[1] * m1n1 + Vij[0] * m2n2);
  o.V12[2 * np + p] = two * (Vij[1] * m1n1 + Vij[1] * m2n2);
  o.V12[3 * np + p] = two * (Vij[2] * m1n1 + Vij[2] * m2n2);
  o.V12[4 * np + p] = Vij[3] * (m1n2 + m2n1);
  o.V12[5 * np + p] = Vij[3] * (m1n2 + m2n1);
  o.V22[0 * np + p] = Vij[0] * n1n1 + Vij[1] * n2n2;
  o.V22[1 * np + p] = Vij[1] * n1n1 + Vij[0] * n2n2;
  o.V22[2 * np + p] = Vij[1] * n1n1 + Vij[1] * n2n2;
  o.V22[3 * np + p] = Vij[2] * n1n1 + Vij[2] * n2n2;
  o.V22[4 * np + p] = Vij[3] * n1n2;
  o.V22[5 * np + p] = Vij[3] * n1n2;
  o.AB[0 * np + p] = kzl * Vij[3] * m1;
  o.AB[1 * np + p] = kzl * Vij[3] * m2;
  o.AB[2 * np + p] = kzl * Vij[3] * n1;
  o.AB[3 * np + p] = kzl * Vij[3] * n2;
  o.AB[4 * np + p] = 0.0;
  o.AB[5 * np + p] = 0.0;
}

// -------------------------------------------------------------------- LHS
// Entry (k, a, b) of the block row of point p (src/lhs1f3d.f90:53-122,
// src/lhs2f3d.f90), given the first (ak) and second (bk) derivative
// coefficient of slot k; `combined` selects the boundary-row form of
// src/lhsbt2f3d.f90:44-50 in which the diagonal slot is formed as
// dtl (a X + rcalcd alfa (Dh + i Dhi)).  The operations run in the order of
// the reference's loops.
__device__ __forceinline__ cd lhs_entry(const Grid& g, const Ops& o, int dir, long long p, int k, int a, int b,
                                        double ak, double bk, bool combined, int damp, double dampc = 0.0,
                                        long long pab = -1) {
  const long long np = o.np;
  const long long e = (long long)((a - 1) + 5 * (b - 1)) * np + p;
  const double x = (dir == 1 ? o.Ah : o.Bh)[e];
  const double d = o.dtl[p], alfa = g.alfa;
  const bool calcd = dir == 1;
  const double rcalcd = calcd ? 1.0 : 0.0;
  double re, im;
  if (combined && k == 3) {
    re = d * (ak * x + rcalcd * alfa * o.Dh[e]);
    im = d * (0.0 + rcalcd * alfa * o.Dhi[e]);
  } else {
    re = ak * d * x;
    im = 0.0;
  }
  // \hat{A}_i, \hat{B}_i: c_k = i a_k
  const double w = ak * d;
  const long long pa = pab < 0 ? p : pab;
  if ((a == 2 && b == 4) || (a == 4 && b == 2)) im = im - w * o.AB[(dir == 1 ? 0 : 2) * np + pa];
  if ((a == 3 && b == 4) || (a == 4 && b == 3)) im = im - w * o.AB[(dir == 1 ? 1 : 3) * np + pa];
  if (calcd && !combined && k == 3) {
    re = re + alfa * d * o.Dh[e];
    im = im + alfa * d * o.Dhi[e];
  }
  // viscous terms: V(0) (2,2), V(4) (2,3), V(5) (3,2), V(1) (3,3), V(2) (4,4), V(3) (5,5)
  int vk = -1;
  if (a == 2 && b == 2) vk = 0;
  else if (a == 2 && b == 3) vk = 4;
  else if (a == 3 && b == 2) vk = 5;
  else if (a == 3 && b == 3) vk = 1;
  else if (a == 4 && b == 4) vk = 2;
  else if (a == 5 && b == 5) vk = 3;
  if (vk >= 0) re = re - (bk * d) * (dir == 1 ? o.V11 : o.V22)[vk * np + p];
  if (k == 3 && a == b) re = re + 1.0;
  // implicit damping: damp 0 the band fb1..fb5 (src/lhs1f3d.f90:168-200,
  // src/lhs2f3d.f90:171-203), 2 the eta rows 2 and ny-1, (-1, 2, -1) in
  // slots 2..4 (src/lhsbt2f3d.f90:277-298, 431-452), 1 none (rows 1, ny)
  if (o.buff && a == b && damp != 1) {
    const double c = damp == 0   ? pick5(k - 1, 1.0, -4.0, 6.0, -4.0, 1.0)
                     : damp == 3 ? dampc
                                 : pick5(k - 1, 0.0, -1.0, 2.0, -1.0, 0.0);
    if (c != 0.0) re = re + g.alfa * d * o.eps_e * o.buff[p] * c;
  }
  // sponge of the eta LHS (src/lhs2f3d.f90:207-224, src/lhsbt2f3d.f90:147-167;
  // the xi LHS has calcd = true and no sponge)
  if (dir == 2 && o.spg && k == 3 && a == b) re = re + g.alfa * d * o.spg[p];
  return cd{re, im};
}

__device__ __forceinline__ void store_el(cd* m, long long q, cd v) { m[q] = v; }
__device__ __forceinline__ void store_el(cf* m, long long q, cd v) { m[q] = cf{(float)v.x, (float)v.y}; }

// The LHS of the xi (dir 1, src/lhs1f3d.f90 + src/lhsbc1f3d.f90) or eta
// sweep (dir 2, src/lhs2f3d.f90 + src/lhsbt2f3d.f90 + src/lhsbc2f3d.f90),
// mat(5,5,5,nx,ny).  One thread per entry, so consecutive threads store
// consecutive entries; T = cf rounds the FP64 entry to FP32.
template <typename T>
__global__ void lhs_kernel(Grid g, Ops o, int dir, LhsCoef lc, T* __restrict__ mat) {
  // 32-bit index arithmetic: creation bounds 125 nx ny below 2^31, and a
  // 64-bit division by the run-time nx would be a long software sequence
  const unsigned q32 = blockIdx.x * blockDim.x + threadIdx.x;
  if (q32 >= 125u * (unsigned)o.np) return;
  const unsigned p32 = q32 / 125u;
  const long long q = q32, p = p32;
  const int e = (int)(q32 - 125u * p32);
  const int k = e % 5 + 1, a = (e / 5) % 5 + 1, b = e / 25 + 1;
  const unsigned jm = p32 / (unsigned)g.nx;
  const int i = (int)(p32 - jm * (unsigned)g.nx) + 1, j = (int)jm + 1;
  const cd one{1.0, 0.0}, zero{0.0, 0.0};
  const cd ident = (k == 3 && a == b) ? one : zero;
  // the linear 2D nonreflecting planes' density rows (j > nbl): in the xi LHS
  // -rho + (gamma Ma rho_m sqrt(T_m) / T_m) u - (rho_m / T_m) T; right 1 writes
  // that row into column 1 as well (src/lhsbc1f.f90:194-198, after the left
  // plane, so it also replaces a zero-disturbance left plane's row there); in
  // the eta LHS the identity row; these follow the wall and top rows and the
  // other xi plane rows
  if (!g.xper && a == 1 && j > g.nbl &&
      ((i == 1 && (g.left == kLinNrLeft || (dir == 1 && g.right == kLinNrRight))) ||
       (i == g.nx && g.right == kLinNrRight))) {
    if (dir == 2) return store_el(mat, q, ident);
    const double* F = (i == 1 ? o.tleft : o.tright) + 4 * (j - 1);
    const double val = k != 3 ? 0.0 : b == 1 ? -1.0 : b == 2 ? F[0] / F[2] : b == 5 ? -F[1] / F[2] : 0.0;
    return store_el(mat, q, cd{val, 0.0});
  }
  // the xi boundaries of a non-periodic xi direction (src/lhsbc1f3d.f90:412-448,
  // src/lhsbc2f3d.f90:146-174); they follow the wall and top rows, so the
  // corners take them
  if (!g.xper && ((i == 1 && (g.left == 0 || g.left == 4 || g.left == 5)) ||
                   (i == g.nx && (g.right == 0 || g.right == 4 || g.right == 5))))
    return store_el(mat, q, ident);
  // the held right plane (right 8): -I in the xi LHS only (src/lhsbc1f3d.f90:439-446)
  if (!g.xper && dir == 1 && i == g.nx && g.right == 8) return store_el(mat, q, cd{-ident.x, -ident.y});
  // boundary conditions of the wall (j = 1) and top (j = ny) rows
  if (!g.yper && (g.top == 0 || g.top == 1) && j == g.ny) return store_el(mat, q, ident);
  if (!g.yper && g.navier && j == 1) {
    if (dir == 1) return store_el(mat, q, ident);  // src/lhsbc1f3d.f90:24-45
    // src/lhsbc2f3d.f90:24-66: continuity / temperature rows in slots 3,4,5,1,2
    const int tk = (k + 2) % 5;  // coefficient of slot k: slots 3,4,5,1,2 <-> 0..4
    if (a >= 2 && a <= 4) return store_el(mat, q, ident);
    if ((a == 1 && g.wall == 1) || (a == 5 && g.wallt == 1))
      return store_el(mat, q, b == a ? cd{-pick5(tk, gc1, gc2, gc3, gc4, gc5), 0.0} : zero);
    if (a == 1 && g.wall == 3)  // third-order extrapolation, src/lhsbc2f3d.f90:41-48
      return store_el(mat, q, b == 1 ? cd{pick5(tk, -1.0, 4.0, -6.0, 4.0, -1.0), 0.0} : zero);
    if (a == 5 && g.wallt == 0) return store_el(mat, q, ident);
  }
  const double h = dir == 1 ? g.dxi : g.deta, alfa = g.alfa;
  const int per = dir == 1 ? g.xper : g.yper;
  const int pos = dir == 1 ? i : j, n = dir == 1 ? g.nx : g.ny;
  double ak, bk;
  bool combined = false;
  const int sym = dir == 1 ? xsym(g) : 0;
  if (((sym & 1) && pos <= 2) || ((sym & 2) && pos >= n - 1)) {
    // symmetry plane (src/lhsbs1f3d.f90): the band stencil with the nodes
    // beyond the plane folded onto their mirror images, times -1 in the
    // columns of the component that changes sign (b = 3)
    const double sg = b == 3 ? -1.0 : 1.0;
    double fa = 0.0, fb = 0.0, fd = 0.0;  // first-derivative, second-derivative and damping stencils
    for (int o5 = 0; o5 < 5; ++o5) {
      int m = pos + o5 - 2;
      bool mir = false;
      if (m < 1) m = 2 - m, mir = true;
      if (m > n) m = 2 * n - m, mir = true;
      if (m - pos + 3 != k) continue;
      const double fbk = pick5(o5, 1.0, -4.0, 6.0, -4.0, 1.0);
      fa = fa + (mir ? sg * lc.ak[o5] : lc.ak[o5]);
      fb = fb + (mir ? sg * lc.bk[o5] : lc.bk[o5]);
      fd = fd + (mir ? sg * fbk : fbk);
    }
    // the reference declares this routine's ABhi dummy (6,ny,nx) for the
    // (6,nx,ny) actual, so it reads entry (k, i, j) at point (i-1) + ny (j-1)
    // (src/lhsbs1f3d.f90:17); creation requires ny <= nx, which keeps that
    // point inside the array
    const long long pab = (long long)(i - 1) + (long long)g.ny * (j - 1);
    store_el(mat, q, lhs_entry(g, o, dir, p, k, a, b, fa, fb, true, 3, fd, pab));
    return;
  }
  if (per || (pos > 2 && pos < n - 1)) {
    ak = lc.ak[k - 1];
    bk = lc.bk[k - 1];
  } else {
    // boundary rows j = 1, 2, ny-1, ny (src/lhsbt2f3d.f90:36-600): coefficient t of slot k
    const double hinv = lc.hinv, hsinv = lc.hsinv;
    auto g1 = [](int t) { return pick5(t, gc1, gc2, gc3, gc4, gc5); };
    auto d1 = [](int t) { return pick5(t, dd1, dd2, dd3, dd4, dd5); };
    auto g2 = [](int t) { return pick5(t, gb1, gb2, gb3, gb4, gb5); };
    auto d2 = [](int t) { return pick5(t, db1, db2, db3, db4, db5); };
    combined = true;
    if (pos == 1) {  // slots 3,4,5,1,2
      const int t = (k + 2) % 5;
      ak = alfa * g1(t) * hinv, bk = alfa * d1(t) * hsinv;
    } else if (pos == 2) {  // slots 2,3,4,5,1
      const int t = (k + 3) % 5;
      ak = alfa * g2(t) * hinv, bk = alfa * d2(t) * hsinv;
    } else if (pos == n - 1) {  // slots 4,3,2,1,5
      const int t = k == 5 ? 4 : 4 - k;
      ak = -(alfa * g2(t) * hinv), bk = alfa * d2(t) * hsinv;
    } else {  // slots 3,2,1,5,4
      const int t = k <= 3 ? 3 - k : 8 - k;
      ak = -(alfa * g1(t) * hinv), bk = alfa * d1(t) * hsinv;
    }
  }
  const int damp = !combined ? 0 : (pos == 2 || pos == n - 1) ? 2 : 1;
  store_el(mat, q, lhs_entry(g, o, dir, p, k, a, b, ak, bk, combined, damp));
}

// The inflow sponge's target (ispg 2, 3; src/lrhs3d.f90:242-280) at every
// point from the mean flow vm, the x coordinates and x0, wamp (ispg 3):
// c3 = [wamp(i)] exp(-a (x - x0)) exp(i kk x), cm = sqrt(T)/Ma,
// kk = omega/(cm + u), a = omega^2 d/(cm + u)^3, d = (4/3 + (gamma-1)/Pr)/(2 Re);
// t = (c3/(2 cm^2), c3/(2 rho cm), 0, 0, (gamma Ma^2 c3/2 - T c3/(2 cm^2))/rho)
// With row0 > 0 the kernel forms only row row0 (the forced top boundary's
// wave, src/itrbc3d.f90:166-196, wamp always applied) into vt(5,nx).
// With col0 > 0 it forms column col0 (the left boundary's wave,
// src/itrbc3d.f90:221-247, no wamp) into vt(5,ny).
__global__ void inflow_target_kernel(Grid g, int with_wamp, int row0, int col0, const double* __restrict__ vm,
                                     const double* __restrict__ xc, const double* __restrict__ wamp, double x0,
                                     cd* __restrict__ vt) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long nt = row0 > 0 ? (long long)g.nx : col0 > 0 ? (long long)g.ny : (long long)g.nx * g.ny;
  if (t >= nt) return;
  const long long p = row0 > 0 ? (long long)(row0 - 1) * g.nx + t : col0 > 0 ? t * g.nx + (col0 - 1) : t;
  const long long o = row0 > 0 || col0 > 0 ? t : p;  // output record
  const int i = (int)(p % g.nx) + 1;
  const double* m = vm + 5 * p;
  const double cm = sqrt(m[4]) / g.Ma, um = m[1];
  const double d = 0.5 * (1.3333333333333333333e+0 + g.gamma1 / g.Pr) / g.Re;
  const double cu = cm + um;
  const double kk = g.omega / cu;
  const double a = g.omega * g.omega * d / (cu * cu * cu);
  const double xl = xc[p];
  const double e = exp(-a * (xl - x0));
  const double w = with_wamp ? wamp[i - 1] * e : e;
  double sn, cs;
  sincos(kk * xl, &sn, &cs);
  const double c3r = w * cs, c3i = w * sn;
  const double cm2 = cm * cm, gm2 = g.gamma * (g.Ma * g.Ma);
  vt[5 * o + 0] = cd{0.5 * c3r / cm2, 0.5 * c3i / cm2};
  vt[5 * o + 1] = cd{c3r * 0.5 / (m[0] * cm), c3i * 0.5 / (m[0] * cm)};
  vt[5 * o + 2] = cd{0.0, 0.0};
  vt[5 * o + 3] = cd{0.0, 0.0};
  vt[5 * o + 4] = cd{(gm2 * c3r * 0.5 - m[4] * 0.5 * c3r / cm2) / m[0], (gm2 * c3i * 0.5 - m[4] * 0.5 * c3i / cm2) / m[0]};
}

// The acoustic wave of a xi plane (left 5 at column 1, right 5 at column
// nx; src/itrbc3d.f90:322-340, 382-405, src/rhsbc3d.f90:248-268, 286-308):
// from the mean flow at (col, j), c3 = exp(i kk x) with kk = omega/(cm + u),
// cm = sqrt(T)/Ma, and t = (c3/(2 cm^2), c3/(2 rho cm), 0, 0,
// (gamma Ma^2 c3/2 - T c3/(2 cm^2))/rho).  The reference takes x as x(j,col)
// of the (nx,ny) array, point (j-1) + nx (col-1), not (col, j): kept, as a
// drop-in must (creation requires ny >= nx for right 5, which keeps that
// point inside the array).
__global__ void plane5_target_kernel(Grid g, int col, const double* __restrict__ vm, const double* __restrict__ xc,
                                     cd* __restrict__ vt) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > g.ny) return;
  const double* m = vm + 5 * pix(g, col, j);
  const double cm = sqrt(m[4]) / g.Ma, um = m[1];
  const double kk = g.omega / (cm + um);
  const double xl = xc[(long long)(j - 1) + (long long)g.nx * (col - 1)];
  double sn, cs;
  sincos(kk * xl, &sn, &cs);
  const double cm2 = cm * cm, gm2 = g.gamma * (g.Ma * g.Ma);
  cd* o = vt + 5 * (j - 1);
  o[0] = cd{0.5 * cs / cm2, 0.5 * sn / cm2};
  o[1] = cd{cs * 0.5 / (m[0] * cm), sn * 0.5 / (m[0] * cm)};
  o[2] = cd{0.0, 0.0};
  o[3] = cd{0.0, 0.0};
  o[4] = cd{(gm2 * cs * 0.5 - m[4] * 0.5 * cs / cm2) / m[0], (gm2 * sn * 0.5 - m[4] * 0.5 * sn / cm2) / m[0]};
}

// The mean-flow factors of the linear 2D nonreflecting plane at column col
// (kLinNrLeft / kLinNrRight), each formed as the reference's expressions
// are: gamma Ma rho_m sqrt(T_m) (src/rhsbc.f90:195-197, src/lhsbc1f.f90:121),
// rho_m, T_m, and gamma Ma^2 rho_m c_m with c_m = sqrt(T_m) / Ma on the left
// and (1 / Ma) sqrt(T_m) on the right (src/itrbc.f90:322, 546, 340, 559).
__global__ void nr_coef_kernel(Grid g, int col, const double* __restrict__ vm, double* __restrict__ f) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x + 1;
  if (j > g.ny) return;
  const double* m = vm + 5 * pix(g, col, j);
  const double rho = m[0], t = m[4];
  const double cm = col == 1 ? sqrt(t) / g.Ma : 1.0 / g.Ma * sqrt(t);
  double* o = f + 4 * (j - 1);
  o[0] = g.gamma * g.Ma * rho * sqrt(t);
  o[1] = rho;
  o[2] = t;
  o[3] = g.gamma * (g.Ma * g.Ma) * rho * cm;
}

// -------------------------------------------------------------------- RHS
// c1v = d v / d xi (complex); (bx, by) is the block within the problem
__device__ __forceinline__ void grad1_body(const Grid& g, const cd* __restrict__ v, cd* __restrict__ c1v, int bx,
                                           int by) {
  const int i = bx * blockDim.x + threadIdx.x + 1;
  const int j = by + 1;
  if (i > g.nx) return;
  const long long p = pix(g, i, j);
  const int sym = xsym(g);
  for (int k = 0; k < 5; ++k) {
    const double sg = k == 2 ? -1.0 : 1.0;  // v changes sign across a symmetry plane
    const double re =
        d1_at(i, g.nx, g.xper, g.gx, g.dxinv, [&](int ii) { return v[k + 5 * pix(g, ii, j)].x; }, sym, sg);
    const double im =
        d1_at(i, g.nx, g.xper, g.gx, g.dxinv, [&](int ii) { return v[k + 5 * pix(g, ii, j)].y; }, sym, sg);
    c1v[k + 5 * p] = cd{re, im};
  }
}

__global__ void grad1_kernel(Grid g, const cd* __restrict__ v, cd* __restrict__ c1v) {
  grad1_body(g, v, c1v, blockIdx.x, blockIdx.y);
}

// r = vold - vs - dtl L(v) (src/lrhs3d.f90:33-218, rbe3D), or with v2old
// the two-step backward r = 4/3 vold - 1/3 v2old - vs - 2/3 dtl L(v)
// (rtb3D, src/impdrv3d.f90:471-501), then the boundary rows of the state vs
// (src/rhsbc3d.f90), written as FP64 (r64) and/or FP32 (r32); the block sums
// of |r|^2 / dtl^2 (src/resstat3d.f90:37-46) go to part[bx + nbx by].  v is
// the field the operator is applied to: the state, or (v + vold)/2 for the
// midpoint rule.
template <bool NARROW>
__device__ __forceinline__ void rhs_body(const Grid& g, const Ops& o, const cd* __restrict__ v,
                                         const cd* __restrict__ vs, const cd* __restrict__ vold,
                                         const cd* __restrict__ v2old, const cd* __restrict__ c1v, cd* r64, cf* r32,
                                         double* part, int bx, int by, int nbx) {
  __shared__ double red[128];
  const int i = bx * blockDim.x + threadIdx.x + 1;
  const int j = by + 1;
  double resnod = 0.0;
  if (i <= g.nx) {
    const long long p = pix(g, i, j), np = o.np;
    auto OP = [&](const double* A, int a, int b) { return A[(long long)(a + 5 * b) * np + p]; };
    auto VH = [&](const double* A, int k) { return A[(long long)k * np + p]; };
    // i z = (-Im z, Re z); r -= i s  <=>  r += (Im s, -Re s)
    auto subi = [](cd& rr, double sx, double sy) { rr = cd{rr.x + sy, rr.y - sx}; };
    const double a1 = VH(o.AB, 0), a2 = VH(o.AB, 1), a3 = VH(o.AB, 2), a4 = VH(o.AB, 3);
    const double* Vs[3] = {o.V11, o.V12, o.V22};
    cd r[5];
    #pragma unroll
    for (int m = 0; m < 5; ++m) r[m] = cd{0.0, 0.0};
    // One input component b at a time: its derivatives, then its terms in
    // every output row, so that only r and one component's derivatives are
    // live.
    #pragma unroll 1
    for (int b = 0; b < 5; ++b) {
      auto VX = [&](int ii) -> const cd& { return v[b + 5 * pix(g, ii, j)]; };
      auto VY = [&](int jj) -> const cd& { return v[b + 5 * pix(g, i, jj)]; };
      auto CY = [&](int jj) -> const cd& { return c1v[b + 5 * pix(g, i, jj)]; };
      const cd vb = v[b + 5 * p], c1b = c1v[b + 5 * p];
      cd c2b{d1_at<NARROW>(j, g.ny, g.yper, g.gy, g.dyinv, [&](int jj) { return VY(jj).x; }),
             d1_at<NARROW>(j, g.ny, g.yper, g.gy, g.dyinv, [&](int jj) { return VY(jj).y; })};
      if (b == 4 && g.navier && (g.wallt == 1 || g.wallt == 2) && j == 1) c2b = cd{0.0, 0.0};  // src/cgradbc.f90
      #pragma unroll
      for (int m = 0; m < 5; ++m) {
        const double A = OP(o.Ah, m, b), B = OP(o.Bh, m, b), D = OP(o.Dh, m, b), Di = OP(o.Dhi, m, b);
        r[m].x += A * c1b.x + B * c2b.x + D * vb.x - Di * vb.y;
        r[m].y += A * c1b.y + B * c2b.y + D * vb.y + Di * vb.x;
      }
      if (b == 0) continue;
      const int sym = xsym(g);
      const double sg = b == 2 ? -1.0 : 1.0;
      const cd c11b{d2_at<NARROW>(i, g.nx, g.xper, g.dx2, g.dxsinv, [&](int ii) { return VX(ii).x; }, sym, sg),
                    d2_at<NARROW>(i, g.nx, g.xper, g.dx2, g.dxsinv, [&](int ii) { return VX(ii).y; }, sym, sg)};
      const cd c22b{d2_at<NARROW>(j, g.ny, g.yper, g.dy2, g.dysinv, [&](int jj) { return VY(jj).x; }),
                    d2_at<NARROW>(j, g.ny, g.yper, g.dy2, g.dysinv, [&](int jj) { return VY(jj).y; })};
      const cd c12b{d1_at<NARROW>(j, g.ny, g.yper, g.gy, g.dyinv, [&](int jj) { return CY(jj).x; }),
                    d1_at<NARROW>(j, g.ny, g.yper, g.gy, g.dyinv, [&](int jj) { return CY(jj).y; })};
      const cd Cs[3] = {c11b, c12b, c22b};
      // viscous terms (entries of Vh11, Vh12, Vh22) and the 3D terms of ABhi
      #pragma unroll
      for (int s3 = 0; s3 < 3; ++s3) {
        auto sub = [&](int m, int k) { const double c = VH(Vs[s3], k); r[m] = cd{r[m].x - c * Cs[s3].x, r[m].y - c * Cs[s3].y}; };
        if (b == 1) { sub(1, 0); sub(2, 5); }
        if (b == 2) { sub(1, 4); sub(2, 1); }
        if (b == 3) sub(3, 2);
        if (b == 4) sub(4, 3);
      }
      if (b == 1) subi(r[3], a1 * c1b.x + a3 * c2b.x, a1 * c1b.y + a3 * c2b.y);
      if (b == 2) subi(r[3], a2 * c1b.x + a4 * c2b.x, a2 * c1b.y + a4 * c2b.y);
      if (b == 3) {
        subi(r[1], a1 * c1b.x + a3 * c2b.x, a1 * c1b.y + a3 * c2b.y);
        subi(r[2], a2 * c1b.x + a4 * c2b.x, a2 * c1b.y + a4 * c2b.y);
      }
    }
    // sponge, src/lrhs3d.f90:222-280 and src/sponge.f90:596-604: r = r +
    // spg v, or the target sponges, on the operator's field
    if (o.spg_b) {
      const double sa = o.spg_a ? o.spg_a[p] : 0.0, sb = o.spg_b[p];
      const cd* T = reinterpret_cast<const cd*>(o.vt) + 5 * p;
      #pragma unroll
      for (int m = 0; m < 5; ++m) {
        const cd vm = v[m + 5 * p], tm = T[m];
        if (o.spg_a) r[m] = cd{r[m].x + sa * vm.x, r[m].y + sa * vm.y};
        r[m] = cd{r[m].x + sb * (vm.x - tm.x), r[m].y + sb * (vm.y - tm.y)};
      }
    } else if (o.spg) {
      const double sp = o.spg[p];
      #pragma unroll
      for (int m = 0; m < 5; ++m) {
        const cd vm = v[m + 5 * p];
        r[m] = cd{r[m].x + sp * vm.x, r[m].y + sp * vm.y};
      }
    }
    // smoother3D (src/smoother3d.f90), the eta pass then the xi pass:
    // rows/columns 2 and n-1 second order, 3 and n-2 fourth order, the rest
    // sixth order; no periodic wrap.  Beside a symmetry plane the xi pass
    // takes the sixth-order stencil at points 1..3 (n-2..n) over the
    // mirrored values, v with its sign changed (src/smoother3d.f90:89-250).
    if (o.buff) {
      const double eb = o.eps_e * o.buff[p];
      const double fa[7] = {-1.666666666666667E-01, 2.0, -6.5, 9.333333333333333, -6.5, 2.0, -1.666666666666667E-01};
      #pragma unroll 1
      for (int pass = 0; pass < 2; ++pass) {
        const int c = pass == 0 ? j : i, n = pass == 0 ? g.ny : g.nx;
        const int sx_ = pass == 1 ? xsym(g) : 0;
        const bool mirror = ((sx_ & 1) && c <= 3) || ((sx_ & 2) && c >= n - 2);
        if (!mirror && (c < 2 || c > n - 1)) continue;
        const long long st = pass == 0 ? 5LL * g.nx : 5LL;
        #pragma unroll
        for (int m = 0; m < 5; ++m) {
          const cd* V = v + m + 5 * p;
          auto S = [&](int dd) -> const cd& { return V[dd * st]; };
          double sx, sy;
          if (mirror) {
            const double sg = m == 2 ? -1.0 : 1.0;
            auto M = [&](int dd) -> cd {
              int kk = c + dd;
              double f = 1.0;
              if (kk < 1) kk = 2 - kk, f = sg;
              else if (kk > n) kk = 2 * n - kk, f = sg;
              const cd& x = V[(kk - c) * st];
              return cd{f * x.x, f * x.y};
            };
            sx = fa[0] * M(-3).x + fa[1] * M(-2).x + fa[2] * M(-1).x + fa[3] * M(0).x + fa[4] * M(1).x +
                 fa[5] * M(2).x + fa[6] * M(3).x;
            sy = fa[0] * M(-3).y + fa[1] * M(-2).y + fa[2] * M(-1).y + fa[3] * M(0).y + fa[4] * M(1).y +
                 fa[5] * M(2).y + fa[6] * M(3).y;
          } else if (c == 2 || c == n - 1) {
            sx = -1.0 * S(-1).x + 2.0 * S(0).x - 1.0 * S(1).x;
            sy = -1.0 * S(-1).y + 2.0 * S(0).y - 1.0 * S(1).y;
          } else if (c == 3 || c == n - 2) {
            sx = S(-2).x - 4.0 * S(-1).x + 6.0 * S(0).x - 4.0 * S(1).x + 1.0 * S(2).x;
            sy = S(-2).y - 4.0 * S(-1).y + 6.0 * S(0).y - 4.0 * S(1).y + 1.0 * S(2).y;
          } else {
            sx = fa[0] * S(-3).x + fa[1] * S(-2).x + fa[2] * S(-1).x + fa[3] * S(0).x + fa[4] * S(1).x +
                 fa[5] * S(2).x + fa[6] * S(3).x;
            sy = fa[0] * S(-3).y + fa[1] * S(-2).y + fa[2] * S(-1).y + fa[3] * S(0).y + fa[4] * S(1).y +
                 fa[5] * S(2).y + fa[6] * S(3).y;
          }
          r[m] = cd{r[m].x + eb * sx, r[m].y + eb * sy};
        }
      }
    }
    // rbe3D
    const double dtl = o.dtl[p];
    if (v2old) {
      const double onept33 = 1.3333333333333333333e+0, pt33 = 3.3333333333333333333e-1,
                   pt66 = 6.6666666666666666666e-1;  // src/global.f90:13-18
      #pragma unroll
      for (int m = 0; m < 5; ++m) {
        const cd vo = vold[m + 5 * p], v2 = v2old[m + 5 * p], vm = vs[m + 5 * p];
        r[m] = cd{onept33 * vo.x - pt33 * v2.x - vm.x - pt66 * dtl * r[m].x,
                  onept33 * vo.y - pt33 * v2.y - vm.y - pt66 * dtl * r[m].y};
      }
    } else {
      #pragma unroll
      for (int m = 0; m < 5; ++m) {
        const cd vo = vold[m + 5 * p], vm = vs[m + 5 * p];
        r[m] = cd{vo.x - vm.x - dtl * r[m].x, vo.y - vm.y - dtl * r[m].y};
      }
    }
    // boundary rows, src/rhsbc3d.f90:34-170
    if (!g.yper) {
      if (g.navier && j == 1) {
        auto W = [&](int k, int jj) -> const cd& { return vs[k + 5 * pix(g, i, jj)]; };
        // the bump wall (wall 3, src/rhsbc3d.f90:45-104): u1w..u3w, tw, twp
        const cd* BW = g.wall == 3 ? reinterpret_cast<const cd*>(o.bump) + 5 * (i - 1) : nullptr;
        for (int m = 1; m <= 3; ++m) {
          const cd u = BW ? BW[m - 1] : cd{0.0, 0.0};
          r[m] = cd{-(W(m, 1).x - u.x), -(W(m, 1).y - u.y)};
        }
        if (g.wall == 1)
          r[0] = cd{gc1 * W(0, 1).x + gc2 * W(0, 2).x + gc3 * W(0, 3).x + gc4 * W(0, 4).x + gc5 * W(0, 5).x,
                    gc1 * W(0, 1).y + gc2 * W(0, 2).y + gc3 * W(0, 3).y + gc4 * W(0, 4).y + gc5 * W(0, 5).y};
        if (g.wall == 2)
          r[0] = cd{W(0, 1).x - two * W(0, 2).x + W(0, 3).x, W(0, 1).y - two * W(0, 2).y + W(0, 3).y};
        if (g.wall == 3)
          r[0] = cd{W(0, 1).x - (4.0 * W(0, 2).x - 6.0 * W(0, 3).x + 4.0 * W(0, 4).x - W(0, 5).x),
                    W(0, 1).y - (4.0 * W(0, 2).y - 6.0 * W(0, 3).y + 4.0 * W(0, 4).y - W(0, 5).y)};
        if (g.wallt == 0) r[4] = BW ? cd{-(W(4, 1).x - BW[3].x), -(W(4, 1).y - BW[3].y)} : cd{0.0, 0.0};
        if (g.wallt == 1) {
          r[4] = cd{gc1 * W(4, 1).x + gc2 * W(4, 2).x + gc3 * W(4, 3).x + gc4 * W(4, 4).x + gc5 * W(4, 5).x,
                    gc1 * W(4, 1).y + gc2 * W(4, 2).y + gc3 * W(4, 3).y + gc4 * W(4, 4).y + gc5 * W(4, 5).y};
          if (BW) r[4] = cd{r[4].x - BW[4].x, r[4].y - BW[4].y};
        }
      }
      if (g.top == 0 && j == g.ny)
        #pragma unroll
        for (int m = 0; m < 5; ++m) r[m] = cd{0.0, 0.0};
      if (g.top == 1 && j == g.ny) {  // src/rhsbc3d.f90:129-160: r = -(v - t)
        const cd* T = reinterpret_cast<const cd*>(o.ttop) + 5 * (i - 1);
        #pragma unroll
        for (int m = 0; m < 5; ++m) {
          const cd w = vs[m + 5 * p];
          r[m] = cd{-(w.x - T[m].x), -(w.y - T[m].y)};
        }
      }
    } else if (j == g.ny) {
      #pragma unroll
      for (int m = 0; m < 5; ++m) r[m] = cd{0.0, 0.0};
    }
    // the xi boundaries (src/rhsbc3d.f90:167-324), after the wall and top rows
    if (!g.xper && ((i == 1 && g.left == 0) || (i == g.nx && (g.right == 0 || g.right == 4 || g.right == 8))))
      #pragma unroll
      for (int m = 0; m < 5; ++m) r[m] = cd{0.0, 0.0};
    // the incoming wave (left 1, src/rhsbc3d.f90:178-206), the eigenfunction
    // inflow (left 4, :207-243), the acoustic planes (left 5, :248-268; right
    // 5, :286-308): r = -(v - t)
    if (!g.xper && i == g.nx && g.right == 5) {
      const cd* T = reinterpret_cast<const cd*>(o.tright) + 5 * (j - 1);
      #pragma unroll
      for (int m = 0; m < 5; ++m) {
        const cd w = vs[m + 5 * p];
        r[m] = cd{-(w.x - T[m].x), -(w.y - T[m].y)};
      }
    }
    if (!g.xper && i == 1 && (g.left == 1 || g.left == 4 || g.left == 5)) {
      const cd* T = reinterpret_cast<const cd*>(o.tleft) + 5 * (j - 1);
      #pragma unroll
      for (int m = 0; m < 5; ++m) {
        const cd w = vs[m + 5 * p];
        r[m] = cd{-(w.x - T[m].x), -(w.y - T[m].y)};
      }
    }
    if (!g.xper && i == 1 && g.left == kLinSymLeft) r[2] = cd{0.0, 0.0};
    // the linear 2D nonreflecting planes: r(1) = rho - (gamma Ma rho_m sqrt(T_m) u - rho_m T) / T_m
    if (!g.xper && j > g.nbl && ((i == 1 && g.left == kLinNrLeft) || (i == g.nx && g.right == kLinNrRight))) {
      const double* F = (i == 1 ? o.tleft : o.tright) + 4 * (j - 1);
      const cd w1 = vs[0 + 5 * p], w2 = vs[1 + 5 * p], w5 = vs[4 + 5 * p];
      r[0] = cd{w1.x - (F[0] * w2.x - F[1] * w5.x) / F[2], w1.y - (F[0] * w2.y - F[1] * w5.y) / F[2]};
    }
    if (g.xper && i == g.nx)
      #pragma unroll
      for (int m = 0; m < 5; ++m) r[m] = cd{0.0, 0.0};
    #pragma unroll
    for (int m = 0; m < 5; ++m) {
      if (r64) r64[m + 5 * p] = r[m];
      if (r32) r32[m + 5 * p] = cf{(float)r[m].x, (float)r[m].y};
      resnod += r[m].x * r[m].x + r[m].y * r[m].y;
    }
    resnod = resnod / (dtl * dtl);
  }
  red[threadIdx.x] = resnod;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[bx + nbx * by] = red[0];
}
template <bool NARROW>
__global__ void __launch_bounds__(128, 4) rhs_kernel(Grid g, Ops o, const cd* __restrict__ v,
                                                  const cd* __restrict__ vs, const cd* __restrict__ vold,
                                                  const cd* __restrict__ v2old, const cd* __restrict__ c1v,
                                                  cd* r64, cf* r32, double* part) {
  rhs_body<NARROW>(g, o, v, vs, vold, v2old, c1v, r64, r32, part, blockIdx.x, blockIdx.y, gridDim.x);
}

// ----------------------------------------------------------------- update
// The boundary values of src/itrbc3d.f90:35-205: threads 0..ncol-1 own a
// column i (wall row j = 1 from rows 2..5, top row j = ny); with a periodic
// x direction the remaining threads copy the interior rows of column 1 to
// column nx, and the thread of column 1 copies its boundary rows.
__device__ __forceinline__ void bc_body(const Grid& g, cd* __restrict__ v, const double* __restrict__ ttop,
                                        const double* __restrict__ bump, const double* __restrict__ tleft,
                                        const double* __restrict__ tright, int bx) {
  const int t = bx * blockDim.x + threadIdx.x;
  const int ncol = g.xper ? g.nx - 1 : g.nx;
  if (t < ncol) {
    const int i = t + 1;
    auto W = [&](int k, int jj) -> cd& { return v[k + 5 * pix(g, i, jj)]; };
    if (!g.yper) {
      if (g.navier) {
        // the bump wall (wall 3, src/itrbc3d.f90:46-121): u1w..u3w, tw, twp
        const cd* BW = g.wall == 3 ? reinterpret_cast<const cd*>(bump) + 5 * (i - 1) : nullptr;
        for (int m = 1; m <= 3; ++m) W(m, 1) = BW ? BW[m - 1] : cd{0.0, 0.0};
        if (g.wall == 1)
          W(0, 1) = cd{-(gc2 * W(0, 2).x + gc3 * W(0, 3).x + gc4 * W(0, 4).x + gc5 * W(0, 5).x) / gc1,
                       -(gc2 * W(0, 2).y + gc3 * W(0, 3).y + gc4 * W(0, 4).y + gc5 * W(0, 5).y) / gc1};
        if (g.wall == 2) W(0, 1) = cd{two * W(0, 2).x - W(0, 3).x, two * W(0, 2).y - W(0, 3).y};
        if (g.wall == 3)
          W(0, 1) = cd{4.0 * W(0, 2).x - 6.0 * W(0, 3).x + 4.0 * W(0, 4).x - W(0, 5).x,
                       4.0 * W(0, 2).y - 6.0 * W(0, 3).y + 4.0 * W(0, 4).y - W(0, 5).y};
        if (g.wallt == 0) W(4, 1) = BW ? BW[3] : cd{0.0, 0.0};
        if (g.wallt == 1) {
          if (BW)
            W(4, 1) = cd{(BW[4].x - (gc2 * W(4, 2).x + gc3 * W(4, 3).x + gc4 * W(4, 4).x + gc5 * W(4, 5).x)) / gc1,
                         (BW[4].y - (gc2 * W(4, 2).y + gc3 * W(4, 3).y + gc4 * W(4, 4).y + gc5 * W(4, 5).y)) / gc1};
          else
            W(4, 1) = cd{-(gc2 * W(4, 2).x + gc3 * W(4, 3).x + gc4 * W(4, 4).x + gc5 * W(4, 5).x) / gc1,
                         -(gc2 * W(4, 2).y + gc3 * W(4, 3).y + gc4 * W(4, 4).y + gc5 * W(4, 5).y) / gc1};
        }
      }
      if (g.top == 0)
        for (int m = 0; m < 5; ++m) W(m, g.ny) = cd{0.0, 0.0};
      if (g.top == 1)  // src/itrbc3d.f90:145-196: the incoming wave
        for (int m = 0; m < 5; ++m) W(m, g.ny) = reinterpret_cast<const cd*>(ttop)[m + 5 * (i - 1)];
    } else {
      for (int m = 0; m < 5; ++m) W(m, g.ny) = W(m, 1);
    }
    if (g.xper && i == 1)
      for (int m = 0; m < 5; ++m) {
        v[m + 5 * pix(g, g.nx, 1)] = W(m, 1);
        v[m + 5 * pix(g, g.nx, g.ny)] = W(m, g.ny);
      }
    // the xi boundaries (src/itrbc3d.f90:203-414), after the wall and top rows
    if (!g.xper && ((i == 1 && g.left == 0) || (i == g.nx && g.right == 0)))
      for (int jj = 1; jj <= g.ny; ++jj)
        for (int m = 0; m < 5; ++m) W(m, jj) = cd{0.0, 0.0};
    // the incoming wave (left 1) and the eigenfunction inflow (left 4,
    // src/itrbc3d.f90:247-320) hold column 1 at t; the eigenfunction outflow
    // (right 4, :357-381) holds column nx at its profile times exp(i lalpha x)
    if (!g.xper && i == 1 && (g.left == 1 || g.left == 4 || g.left == 5))
      for (int jj = 1; jj <= g.ny; ++jj)
        for (int m = 0; m < 5; ++m) W(m, jj) = reinterpret_cast<const cd*>(tleft)[m + 5 * (jj - 1)];
    if (!g.xper && i == g.nx && (g.right == 4 || g.right == 5))
      for (int jj = 1; jj <= g.ny; ++jj)
        for (int m = 0; m < 5; ++m) W(m, jj) = reinterpret_cast<const cd*>(tright)[m + 5 * (jj - 1)];
    if (!g.xper && i == 1 && g.left == kLinSymLeft)
      for (int jj = 1; jj <= g.ny; ++jj) W(2, jj) = cd{0.0, 0.0};
    // the linear 2D nonreflecting planes: rho = (gamma Ma^2 rho_m c_m u - rho_m T) / T_m on rows j > nbl
    if (!g.xper && ((i == 1 && g.left == kLinNrLeft) || (i == g.nx && g.right == kLinNrRight))) {
      const double* F = i == 1 ? tleft : tright;
      for (int jj = g.nbl + 1; jj <= g.ny; ++jj) {
        const double* f = F + 4 * (jj - 1);
        const cd u = W(1, jj), t = W(4, jj);
        W(0, jj) = cd{(f[3] * u.x - f[1] * t.x) / f[2], (f[3] * u.y - f[1] * t.y) / f[2]};
      }
    }
  } else if (g.xper) {
    const int j = t - ncol + 2;
    if (j <= g.ny - 1)
      for (int m = 0; m < 5; ++m) v[m + 5 * pix(g, g.nx, j)] = v[m + 5 * pix(g, 1, j)];
  }
}

__global__ void bc_kernel(Grid g, cd* __restrict__ v, const double* __restrict__ ttop,
                          const double* __restrict__ bump, const double* __restrict__ tleft,
                          const double* __restrict__ tright) {
  bc_body(g, v, ttop, bump, tleft, tright, blockIdx.x);
}

// ------------------------------------------------------------- batching
// Per-problem arguments of the per-step kernels of a batch (lns_batch3d):
// one launch of a batched kernel runs one phase of every problem, block b
// doing block table[b].y (and .z) of problem table[b].x; problems whose
// active flag is zero are skipped.
struct StepArgs {
  Grid g;
  Ops o;
  cd *v, *vold, *c1v, *r64;
  cf* r32;
  double* part;  // RHS block partials
  int nbx, nrhs;  // RHS blocks along x, partial count
  double tol;    // the problem stops (active = 0) at the first residual <= tol; 0: never
};

// The batched kernels are persistent: a fixed grid strides over the phase's
// work table, whose length (and the problem count) the kernels read from
// device memory, so a captured step stays valid when the batch's problems
// change and only the tables are rewritten.
__global__ void copy_batch_kernel(const StepArgs* __restrict__ list, const int2* __restrict__ table,
                                  const int* __restrict__ active, const int* __restrict__ cnt) {
  for (int k = blockIdx.x; k < *cnt; k += gridDim.x) {
    const int2 w = table[k];
    if (!active[w.x]) continue;
    const StepArgs& a = list[w.x];
    const long long e = (long long)w.y * blockDim.x + threadIdx.x;
    if (e < 5 * a.o.np) a.vold[e] = a.v[e];
  }
}
__global__ void bc_batch_kernel(const StepArgs* __restrict__ list, const int2* __restrict__ table,
                                const int* __restrict__ active, const int* __restrict__ cnt) {
  for (int k = blockIdx.x; k < *cnt; k += gridDim.x) {
    const int2 w = table[k];
    if (!active[w.x]) continue;
    bc_body(list[w.x].g, list[w.x].v, list[w.x].o.ttop, list[w.x].o.bump, list[w.x].o.tleft, list[w.x].o.tright,
            w.y);
  }
}
__global__ void grad1_batch_kernel(const StepArgs* __restrict__ list, const int4* __restrict__ table,
                                   const int* __restrict__ active, const int* __restrict__ cnt) {
  for (int k = blockIdx.x; k < *cnt; k += gridDim.x) {
    const int4 w = table[k];
    if (!active[w.x]) continue;
    const StepArgs& a = list[w.x];
    grad1_body(a.g, a.v, a.c1v, w.y, w.z);
  }
}
template <bool NARROW>
__global__ void __launch_bounds__(128, 4) rhs_batch_kernel(const StepArgs* __restrict__ list,
                                                        const int4* __restrict__ table,
                                                        const int* __restrict__ active, const int* __restrict__ cnt,
                                                        int mixed) {
  for (int k = blockIdx.x; k < *cnt; k += gridDim.x) {
    const int4 w = table[k];
    if (!active[w.x]) continue;
    const StepArgs& a = list[w.x];
    rhs_body<NARROW>(a.g, a.o, a.v, a.v, a.vold, nullptr, a.c1v, mixed ? nullptr : a.r64, mixed ? a.r32 : nullptr,
                     a.part, w.y, w.z, a.nbx);
  }
}
// residual of each problem into hist[step * P + p] (src/resstat3d.f90:37-60),
// P = *nprob.  A problem whose residual reaches its tolerance is switched off
// here, so the rest of this step and later steps leave its state as it was
// when the residual was measured.
__global__ void resid_batch_kernel(const StepArgs* __restrict__ list, int* active, double* __restrict__ hist,
                                   const int* __restrict__ step, const int* __restrict__ nprob) {
  __shared__ double red[256];
  const int P = *nprob;
  for (int p = blockIdx.x; p < P; p += gridDim.x) {
    if (!active[p]) continue;
    const StepArgs& a = list[p];
    double s = 0.0;
    for (int k = threadIdx.x; k < a.nrhs; k += blockDim.x) s += a.part[k];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
      if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
      __syncthreads();
    }
    if (threadIdx.x == 0) {
      const double r = sqrt(red[0] / (double)a.o.np);
      hist[(long long)(*step) * P + p] = r;
      if (a.tol > 0.0 && r <= a.tol) active[p] = 0;
    }
    __syncthreads();  // red is refilled for the next problem
  }
}
template <typename RT>
__global__ void add_batch_kernel(const StepArgs* __restrict__ list, const int2* __restrict__ table,
                                 const int* __restrict__ active, const int* __restrict__ cnt) {
  for (int k = blockIdx.x; k < *cnt; k += gridDim.x) {
    const int2 w = table[k];
    if (!active[w.x]) continue;
    const StepArgs& a = list[w.x];
    const long long e = (long long)w.y * blockDim.x + threadIdx.x;
    if (e >= 5 * a.o.np) continue;
    const RT* r = reinterpret_cast<const RT*>(std::is_same<RT, cd>::value ? (const void*)a.r64 : (const void*)a.r32);
    a.v[e] = add(a.v[e], to_hi(r[e]));
  }
}
__global__ void step_incr_kernel(int* step) { *step += 1; }

}  // namespace a3
}  // namespace lns

// ======================================================================
// Context and C ABI
// ======================================================================
using lns::cd;
using lns::cf;
using lns::a3::Grid;
using lns::a3::Metrics;
using lns::a3::Ops;

struct lns_ctx3d {
  lns_params3d prm;
  Grid g;
  int device = -1;
  long long np = 0;
  size_t bytes = 0;
  std::vector<void*> allocs;
  double* metrics = nullptr;  // (nx,ny,10)
  double* vm = nullptr;       // (5,nx,ny)
  double* opbuf = nullptr;    // Ah Bh Dh Dhi (25 np each), V11 V12 V22 AB (6 np each), dtl (np)
  Ops ops{};
  cd *v = nullptr, *vold = nullptr, *r64 = nullptr, *c1v = nullptr;
  cf* r32 = nullptr;
  // FP64 factors in the reference storage (both modes), and the same
  // factors in the scaled block form of penta_chain.cuh in the precision of
  // the sweeps; periodic lines add W (fillE, aliasing perx in the FP64 mode)
  // and their border data (bordx: S^-1, A21)
  void *matx = nullptr, *maty = nullptr, *perx = nullptr, *per2x = nullptr;
  void *chnx = nullptr, *chny = nullptr, *fillE = nullptr, *bordx = nullptr;
  // a periodic eta direction (yper): the same for the eta lines
  void *pery = nullptr, *per2y = nullptr, *fillEy = nullptr, *bordy = nullptr;
  // FP64 periodic lines with an odd band solved in row pairs (penta_chain.cuh):
  // their pair arrays (allocated at the first factorisation), and whether the
  // records are in the paired form; a batch's contexts stay row by row
  void *pairx = nullptr, *pairy = nullptr;
  bool pair_ok = true, paired_x = false, paired_y = false;
  int sms = 0;  // the device's SMs
  double* part = nullptr;  // block partials (residual, CFL)
  int nparts = 0;
  double* dscal = nullptr;  // [0] cfl, [1..] residual of the inspection call
  double* res_dev = nullptr;  // residual history of the host-form steps
  int res_cap = 0;
  int* status = nullptr;
  bool have_metrics = false, have_mean = false, factored = false;
  bool have_sponge = false;   // ispg != 0: lns_upload_sponge3d called
  double* spg = nullptr;      // spg (ispg 1), else spg + spg2
  double *spg_a = nullptr, *spg_b = nullptr, *vt = nullptr;  // the target sponges (ispg 2-4)
  double *xc = nullptr, *wamp = nullptr;  // ispg 2, 3 or top 1: x(nx,ny), wamp(nx) (ones until uploaded)
  double* ttop = nullptr;                 // top 1: the wave of row ny, complex (5,nx)
  double* tleft = nullptr;                // left 1: the wave of column 1; left 4: the eigenfunction; complex (5,ny)
  double* tright = nullptr;               // right 4: the eigenfunction times exp(i lalpha x(nx,j)), complex (5,ny)
  bool have_profile = false;              // left 4: lns_upload_profile3d called
  double* bump = nullptr;                 // wall 3: u1w, u2w, u3w, tw, twp, complex (5,nx)
  bool have_bump = false;
  double x0 = 0.0;
  bool have_inflow = false, have_target = false;
  double* buff = nullptr;     // eps_e != 0: buff(nx,ny), ones until uploaded
  // time scheme (src/impdrv3d.f90:130-199): the previous-previous state
  // (impl 2), the averaged field (impl 3), steps taken, alfa of the factors
  cd *v2old = nullptr, *wavg = nullptr;
  long long lstep = 0;
  double alfa_fac = -1.0;
  // phase timing (lns_ctx3d_profile): per corrector, events around the RHS,
  // the scaling, recurrences, tail and fill kernels of both sweeps, and the
  // update (LNS_PROFILE_SEGMENTS segments)
  bool profile = false;
  std::vector<cudaEvent_t> events;
  size_t ev_used = 0;
};

namespace {

int fail3(int code, const std::string& msg) { return lns_fail(code, msg); }
int cuda3(cudaError_t e, const char* where) { return lns_cuda_fail(e, where); }

// interior stencil coefficients, src/cgrad.f90:35-75 and src/cgrad2.f90:38-100
void coef1(int opt, double dinv, double g[6]) {
  double c, a, b;
  if (opt == 0) c = 1.0 / 60.0;
  else if (opt == -1) c = 0.0;
  else {
    const double w = 2.0 * 3.1415926535897932385e+0 / 12.0;
    c = (w / 2.0 - 2.0 * sin(w) / 3.0 + sin(2.0 * w) / 12.0) / (5.0 * sin(w) - 4.0 * sin(2.0 * w) + sin(3.0 * w));
  }
  a = (2.0 + 15.0 * c) / 3.0;
  b = -(1.0 + 48.0 * c) / 12.0;
  g[0] = -c * dinv; g[1] = -b * dinv; g[2] = -a * dinv;
  g[3] = a * dinv;  g[4] = b * dinv;  g[5] = c * dinv;
}
void coef2(int opt, double dsinv, double d[7]) {
  double c, a, b;
  if (opt == 0) c = 1.0 / 90.0;
  else if (opt == -1) c = 0.0;
  else {
    const double w = 2.0 * 3.1415926535897932385e+0 / 12.0;
    const double s1 = sin(w / 2.0), s2 = sin(w), s3 = sin(3.0 * w / 2.0);
    c = -(3.0 * (w * w) - 16.0 * (s1 * s1) + (s2 * s2)) / (12.0 * (-15.0 * (s1 * s1) + 6.0 * (s2 * s2) - (s3 * s3)));
  }
  a = (4.0 + 45.0 * c) / 3.0;
  b = -(1.0 + 72.0 * c) / 12.0;
  d[0] = c * dsinv; d[1] = b * dsinv; d[2] = a * dsinv; d[3] = -2.0 * (a + b + c) * dsinv;
  d[4] = a * dsinv; d[5] = b * dsinv; d[6] = c * dsinv;
}

int dalloc(lns_ctx3d* c, size_t bytes, void** out) {
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    *out = nullptr;
    return fail3(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  c->allocs.push_back(*out);
  c->bytes += bytes;
  return LNS_OK;
}

void free_all(lns_ctx3d* c) {
  for (void* p : c->allocs) cudaFree(p);
  c->allocs.clear();
  for (cudaEvent_t e : c->events) cudaEventDestroy(e);
  c->events.clear();
}

// records the next profiling event on `st` (no-op unless profiling)
int mark(lns_ctx3d* c, cudaStream_t st) {
  if (!c->profile) return LNS_OK;
  if (c->ev_used == c->events.size()) {
    cudaEvent_t e;
    cudaError_t r = cudaEventCreate(&e);
    if (r != cudaSuccess) return cuda3(r, "cudaEventCreate");
    c->events.push_back(e);
  }
  cudaError_t r = cudaEventRecord(c->events[c->ev_used++], st);
  return r == cudaSuccess ? LNS_OK : cuda3(r, "cudaEventRecord");
}

int check_device(const lns_ctx3d* c) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda3(e, "cudaGetDevice");
  if (dev != c->device) return fail3(LNS_ERR_ARG, "context belongs to another device");
  return LNS_OK;
}

Metrics metrics_of(const lns_ctx3d* c) {
  const double* m = c->metrics;
  const long long np = c->np;
  return Metrics{m, m + np, m + 2 * np, m + 3 * np, m + 4 * np, m + 5 * np, m + 6 * np, m + 7 * np, m + 8 * np,
                 m + 9 * np};
}

dim3 pt_grid(const Grid& g) { return dim3((g.nx + 127) / 128, g.ny); }

// residual history buffer of at least n entries
int res_reserve(lns_ctx3d* c, int n) {
  if (c->res_cap >= n) return LNS_OK;
  void* p = nullptr;
  int rc = dalloc(c, sizeof(double) * (size_t)n, &p);
  if (rc) return rc;
  c->res_dev = (double*)p;
  c->res_cap = n;
  return LNS_OK;
}

// r = RHS of one corrector into r64 (FP64) and / or r32 (FP32); totres to *res.
// The operator acts on the field v; vs is the state (rbe3D / rtb3D and the
// boundary rows); v2old selects rtb3D.
int launch_rhs(lns_ctx3d* c, const cd* v, const cd* vs, const cd* vold, const cd* v2old, cd* r64, cf* r32,
               double* res, cudaStream_t st) {
  const Grid& g = c->g;
  lns::a3::grad1_kernel<<<pt_grid(g), 128, 0, st>>>(g, v, c->c1v);
  if (lns::a3::narrow_stencils(g))
    lns::a3::rhs_kernel<true><<<pt_grid(g), 128, 0, st>>>(g, c->ops, v, vs, vold, v2old, c->c1v, r64, r32, c->part);
  else
    lns::a3::rhs_kernel<false><<<pt_grid(g), 128, 0, st>>>(g, c->ops, v, vs, vold, v2old, c->c1v, r64, r32,
                                                           c->part);
  const int nrhs = (int)(pt_grid(g).x * pt_grid(g).y);  // rhs_kernel block partials
  lns::a3::resid_kernel<<<1, 256, 0, st>>>(nrhs, c->part, c->np, res);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda3(e, "rhs kernels launch");
}

template <typename T>
int launch_lhs(lns_ctx3d* c, int dir, T* mat, cudaStream_t st) {
  const long long nq = 125 * c->np;
  const lns::a3::LhsCoef lc = lns::a3::lhs_coef(c->g.alfa, dir == 1 ? c->g.dxi : c->g.deta);
  lns::a3::lhs_kernel<T><<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(c->g, c->ops, dir, lc, mat);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda3(e, "lhs_kernel launch");
}

// Arguments of the xi sweep (periodic lines along i, one per j: np = nx,
// n = nx - 1 unknowns) and of the eta sweep (lines along j, one per i;
// periodic lines with yper: n = ny - 1 unknowns).
lns::chain::Args xargs(lns_ctx3d* c, void* rhs) {
  const Grid& g = c->g;
  if (!g.xper) return lns::chain::Args{c->matx, c->chnx, nullptr, nullptr, nullptr, rhs, g.nx, g.ny, 1, g.nx};
  return lns::chain::Args{c->matx, c->chnx, c->perx, c->per2x, c->fillE, rhs, g.nx - 1, g.ny, 1, g.nx,
                          c->bordx, c->paired_x ? c->pairx : nullptr};
}
lns::chain::Args yargs(lns_ctx3d* c, void* rhs) {
  const Grid& g = c->g;
  if (g.yper) return lns::chain::Args{c->maty, c->chny, c->pery, c->per2y, c->fillEy, rhs, g.ny - 1, g.nx,
                                      g.nx, 1, c->bordy, c->paired_y ? c->pairy : nullptr};
  return lns::chain::Args{c->maty, c->chny, nullptr, nullptr, nullptr, rhs, g.ny, g.nx, g.nx, 1, nullptr,
                          c->paired_y ? c->pairy : nullptr};
}

// A periodic sweep (xi, or eta with yper), bordered: s = D^-1 r on rows
// 1..n-2, the two recurrences (z = A11^-1 b1), the border unknowns x2 =
// S^-1 (b2 - A21 z) and the correction x1 = z - W x2.
// xi_marks: the profiling marks of the xi sweep (after the scaling and each
// recurrence; the border and correction close the segment); an eta sweep
// marks as a non-periodic one (after the scaling and the forward recurrence).
// FP64 lines in the paired form: the two recurrences advance two rows per
// step (pair_chain_kernel), each after even_kernel has formed the even rows'
// combined right-hand sides.
template <typename T>
int sweep_periodic(lns_ctx3d* c, const lns::chain::Args& a, bool xi_marks, cudaStream_t st) {
  namespace ch = lns::chain;
  const long long fill = (long long)(a.n - 2) * a.nsys;
  if constexpr (std::is_same<T, cd>::value) {
    if (a.pairs) {
      const long long pts = (long long)a.n * a.nsys;
      const int cta = (a.nsys + ch::kPairLines - 1) / ch::kPairLines;
      const size_t sm = ch::pair_smem_bytes();
      const int rows = (a.n - 3) / 2;  // even band rows 2..n-3
      const unsigned eb = (unsigned)((5LL * rows * a.nsys + 255) / 256);
      ch::scale_kernel<T><<<(unsigned)ch::scale_blocks(pts), 256, 0, st>>>(a);
      int rc = mark(c, st);
      ch::even_kernel<false><<<eb, 256, 0, st>>>(a, 2, rows);
      ch::pair_chain_kernel<false><<<cta, 128 * ch::kPairLines, sm, st>>>(a);
      if (!rc) rc = mark(c, st);
      ch::even_kernel<true><<<eb, 256, 0, st>>>(a, 2, rows);
      ch::pair_chain_kernel<true><<<cta, 128 * ch::kPairLines, sm, st>>>(a);
      if (!rc && xi_marks) rc = mark(c, st);
      ch::btail_kernel<T><<<(a.nsys + ch::kBTailLines - 1) / ch::kBTailLines, 32 * ch::kBTailLines, 0, st>>>(a);
      ch::fill_kernel<T><<<(unsigned)ch::fill_blocks(fill), 256, 0, st>>>(a);
      if (rc) return rc;
      cudaError_t e = cudaGetLastError();
      return e == cudaSuccess ? LNS_OK : cuda3(e, "paired periodic sweep launch");
    }
  }
  const long long pts = (long long)a.n * a.nsys;
  const int cta = (a.nsys + ch::kChainWarps - 1) / ch::kChainWarps;
  const size_t sm = ch::chain_smem_bytes<T>();
  ch::scale_kernel<T><<<(unsigned)ch::scale_blocks(pts), 256, 0, st>>>(a);
  int rc = mark(c, st);
  ch::chain_fwd_kernel<T, true><<<cta, ch::chain_threads<T>(), sm, st>>>(a);
  if (!rc) rc = mark(c, st);
  ch::chain_bwd_kernel<T, true><<<cta, ch::chain_threads<T>(), sm, st>>>(a);
  if (!rc && xi_marks) rc = mark(c, st);
  ch::btail_kernel<T><<<(a.nsys + ch::kBTailLines - 1) / ch::kBTailLines, 32 * ch::kBTailLines, 0, st>>>(a);
  ch::fill_kernel<T><<<(unsigned)ch::fill_blocks(fill), 256, 0, st>>>(a);
  if (rc) return rc;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda3(e, "periodic sweep launch");
}

// A sweep of lines with boundary-closure rows: s = D^-1 r, forward and
// backward recurrences.  xi_marks: the profiling marks of the xi sweep
// (after the scaling, the forward and the backward recurrence, leaving the
// border segment of the periodic xi sweep empty).
template <typename T>
int sweep_bc(lns_ctx3d* c, const lns::chain::Args& a, bool xi_marks, cudaStream_t st) {
  namespace ch = lns::chain;
  const long long pts = (long long)a.n * a.nsys;
  const int cta = (a.nsys + ch::kChainWarps - 1) / ch::kChainWarps;
  const size_t sm = ch::chain_smem_bytes<T>();
  ch::scale_kernel<T><<<(unsigned)ch::scale_blocks(pts), 256, 0, st>>>(a);
  int rc = mark(c, st);
  ch::chain_fwd_kernel<T, false><<<cta, ch::chain_threads<T>(), sm, st>>>(a);
  if (!rc) rc = mark(c, st);
  ch::chain_bwd_kernel<T, false><<<cta, ch::chain_threads<T>(), sm, st>>>(a);
  if (!rc && xi_marks) rc = mark(c, st);
  if (rc) return rc;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda3(e, "sweep launch");
}

template <typename T>
int sweep_x(lns_ctx3d* c, T* r, cudaStream_t st) {
  if (!c->g.xper) return sweep_bc<T>(c, xargs(c, r), true, st);
  return sweep_periodic<T>(c, xargs(c, r), true, st);
}

// The eta sweep: s = D^-1 r, forward and backward recurrences (periodic
// lines as the xi sweep).
template <typename T>
int sweep_y(lns_ctx3d* c, T* r, cudaStream_t st) {
  namespace ch = lns::chain;
  const ch::Args a = yargs(c, r);
  if (c->g.yper) return sweep_periodic<T>(c, a, false, st);
  if constexpr (std::is_same<T, cd>::value) {
    if (a.pairs) {  // rows in pairs: forward second rows even, backward ones odd
      const long long pts = (long long)a.n * a.nsys;
      const int cta = (a.nsys + ch::kPairLines - 1) / ch::kPairLines, rows = a.n / 2;
      const size_t sm = ch::pair_smem_bytes();
      const unsigned eb = (unsigned)((5LL * rows * a.nsys + 255) / 256);
      ch::scale_kernel<T><<<(unsigned)ch::scale_blocks(pts), 256, 0, st>>>(a);
      int rc = mark(c, st);
      ch::even_kernel<false><<<eb, 256, 0, st>>>(a, 2, rows);
      ch::pair_chain_kernel<false, true><<<cta, 128 * ch::kPairLines, sm, st>>>(a);
      if (!rc) rc = mark(c, st);
      ch::even_kernel<true><<<eb, 256, 0, st>>>(a, 1, rows);
      ch::pair_chain_kernel<true, true><<<cta, 128 * ch::kPairLines, sm, st>>>(a);
      if (rc) return rc;
      cudaError_t e = cudaGetLastError();
      return e == cudaSuccess ? LNS_OK : cuda3(e, "paired eta sweep launch");
    }
  }
  const long long pts = (long long)a.n * a.nsys;
  const int cta = (a.nsys + ch::kChainWarps - 1) / ch::kChainWarps;
  const size_t sm = ch::chain_smem_bytes<T>();
  ch::scale_kernel<T><<<(unsigned)ch::scale_blocks(pts), 256, 0, st>>>(a);
  int rc = mark(c, st);
  ch::chain_fwd_kernel<T, false><<<cta, ch::chain_threads<T>(), sm, st>>>(a);
  if (!rc) rc = mark(c, st);
  ch::chain_bwd_kernel<T, false><<<cta, ch::chain_threads<T>(), sm, st>>>(a);
  if (rc) return rc;
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda3(e, "eta sweep launch");
}

// W, S^-1 and A21 of the periodic lines of a (their border blocks copied by
// bcopy_kernel before the factorisation, their records prepared): ten
// solves z = A11^-1 (column j of A12) through the recurrences, then the
// Schur complement.  a.rhs is a sweep-sized scratch buffer.
template <typename TC>
int form_border(lns_ctx3d* c, const lns::chain::Args& a, cudaStream_t st) {
  namespace ch = lns::chain;
  const long long pts = (long long)a.n * a.nsys;
  const int cta = (a.nsys + ch::kChainWarps - 1) / ch::kChainWarps;
  const size_t sm = ch::chain_smem_bytes<TC>();
  for (int j = 0; j < 10; ++j) {
    cudaError_t e = cudaMemsetAsync(a.rhs, 0, sizeof(TC) * 5 * (size_t)c->np, st);
    if (e != cudaSuccess) return cuda3(e, "cudaMemsetAsync border");
    ch::brhs_kernel<TC><<<(unsigned)((a.nsys * 30LL + 255) / 256), 256, 0, st>>>(a, j);
    ch::scale_kernel<TC><<<(unsigned)ch::scale_blocks(pts), 256, 0, st>>>(a);
    ch::chain_fwd_kernel<TC, true><<<cta, ch::chain_threads<TC>(), sm, st>>>(a);
    ch::chain_bwd_kernel<TC, true><<<cta, ch::chain_threads<TC>(), sm, st>>>(a);
    ch::bw_kernel<TC><<<(unsigned)((a.nsys * (a.n - 2) * 5LL + 255) / 256), 256, 0, st>>>(a, j);
  }
  ch::bschur_kernel<TC><<<(a.nsys + 63) / 64, 64, 0, st>>>(a, c->status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda3(e, "border kernels launch");
}

// Forms both LHS and factors them in FP64 (code 0), checks the pivots, and
// writes the scaled block form in the precision TC of the sweeps.
template <typename TC>
int factor_all(lns_ctx3d* c, cudaStream_t st) {
  const Grid& g = c->g;
  cd* mx = (cd*)c->matx;
  cd* my = (cd*)c->maty;
  cd* rr = c->c1v;  // a right-hand-side argument; code 0 does not touch it
  cudaError_t e = cudaMemsetAsync(c->status, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda3(e, "cudaMemsetAsync");
  namespace ch = lns::chain;
  const ch::Args ax = xargs(c, nullptr), ay = yargs(c, nullptr);
  // the periodic factorisation mode, read once for both directions: the
  // reference's (its row n-5 fill placement) unless the exact LU is chosen
  const int exact = g_periodic_exact.load() ? 1 : 0;
  c->paired_x = c->paired_y = false;  // the records are formed row by row again below
  int rc = launch_lhs<cd>(c, 1, mx, st);
  if (!rc && g.xper) {
    ch::bcopy_kernel<<<(unsigned)((ax.nsys * 400LL + 255) / 256), 256, 0, st>>>(ax);
    rc = lns::host::launch_p<cd>(mx, rr, c->perx, c->per2x, g.nx, g.ny, 1, g.nx, 0, st, c->status, exact);
    if (!rc && !exact) ch::bquirk_kernel<<<(unsigned)((ax.nsys * 25LL + 255) / 256), 256, 0, st>>>(ax);
  } else if (!rc) {
    rc = lns::host::launch_bc<cd>(mx, rr, g.nx, g.ny, 1, g.nx, 0, st, c->status);
  }
  if (!rc) rc = launch_lhs<cd>(c, 2, my, st);
  if (!rc && g.yper) {
    ch::bcopy_kernel<<<(unsigned)((ay.nsys * 400LL + 255) / 256), 256, 0, st>>>(ay);
    rc = lns::host::launch_p<cd>(my, rr, c->pery, c->per2y, g.ny, g.nx, g.nx, 1, 0, st, c->status, exact);
    if (!rc && !exact) ch::bquirk_kernel<<<(unsigned)((ay.nsys * 25LL + 255) / 256), 256, 0, st>>>(ay);
  } else if (!rc) {
    rc = lns::host::launch_bc<cd>(my, rr, g.ny, g.nx, g.nx, 1, 0, st, c->status);
  }
  if (rc) return rc;
  const long long tx = (long long)ax.n * ax.nsys, ty = (long long)ay.n * ay.nsys;
  const unsigned bx = (unsigned)((tx + ch::kPrepWarps - 1) / ch::kPrepWarps);
  const unsigned by = (unsigned)((ty + ch::kPrepWarps - 1) / ch::kPrepWarps);
  if (g.xper) ch::prep_kernel<cd, TC, true><<<bx, 32 * ch::kPrepWarps, 0, st>>>(ax);
  else ch::prep_kernel<cd, TC, false><<<bx, 32 * ch::kPrepWarps, 0, st>>>(ax);
  if (g.yper) ch::prep_kernel<cd, TC, true><<<by, 32 * ch::kPrepWarps, 0, st>>>(ay);
  else ch::prep_kernel<cd, TC, false><<<by, 32 * ch::kPrepWarps, 0, st>>>(ay);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda3(e, "prep kernels launch");
  // periodic lines: W = A11^-1 A12 column by column through the sweeps'
  // own recurrences (on the sweep buffer, free before the first RHS), then
  // S^-1 and A21
  TC* scratch = reinterpret_cast<TC*>(std::is_same<TC, cf>::value ? (void*)c->r32 : (void*)c->r64);
  if (!rc && g.xper) rc = form_border<TC>(c, xargs(c, scratch), st);
  if (!rc && g.yper) rc = form_border<TC>(c, yargs(c, scratch), st);
  if (rc) return rc;
  // FP64 lines in the paired form, where the row count allows it and the
  // lines are few: with four warps a line the pairs pay while a direction's
  // lines leave the SMs' sub-partitions at most two warps each (more lines
  // already fill the FP64 pipes row by row, and pairs only add instructions)
  if constexpr (std::is_same<TC, cd>::value) {
    const bool few_x = g.ny <= 2 * c->sms, few_y = g.nx <= 2 * c->sms;
    if (c->pair_ok && few_x && g.xper && (g.nx - 3) % 2 == 1) {
      if (!c->pairx) rc = dalloc(c, sizeof(cd) * 50 * (size_t)c->np, &c->pairx);
      if (!rc) {
        ch::Args pa = xargs(c, nullptr);
        pa.pairs = c->pairx;
        const long long tasks = (long long)(pa.n - 3) / 2 * pa.nsys;
        ch::pair_prep_kernel<<<(unsigned)((tasks + ch::kPrepWarps - 1) / ch::kPrepWarps), 32 * ch::kPrepWarps, 0,
                               st>>>(pa);
        c->paired_x = true;
      }
    }
    if (!rc && c->pair_ok && few_y && !g.yper && g.ny % 2 == 0) {  // eta lines with boundary-closure rows
      if (!c->pairy) rc = dalloc(c, sizeof(cd) * 50 * (size_t)c->np, &c->pairy);
      if (!rc) {
        ch::Args pa = yargs(c, nullptr);
        pa.pairs = c->pairy;
        const long long tasks = (long long)pa.n * pa.nsys;
        ch::pair_prep_bc_kernel<<<(unsigned)((tasks + ch::kPrepWarps - 1) / ch::kPrepWarps), 32 * ch::kPrepWarps, 0,
                                  st>>>(pa);
        c->paired_y = true;
      }
    }
    if (!rc && c->pair_ok && few_y && g.yper && (g.ny - 3) % 2 == 1) {
      if (!c->pairy) rc = dalloc(c, sizeof(cd) * 50 * (size_t)c->np, &c->pairy);
      if (!rc) {
        ch::Args pa = yargs(c, nullptr);
        pa.pairs = c->pairy;
        const long long tasks = (long long)(pa.n - 3) / 2 * pa.nsys;
        ch::pair_prep_kernel<<<(unsigned)((tasks + ch::kPrepWarps - 1) / ch::kPrepWarps), 32 * ch::kPrepWarps, 0,
                               st>>>(pa);
        c->paired_y = true;
      }
    }
    if (rc) return rc;
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda3(e, "pair prep launch");
  }
  int status = 0;
  e = cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda3(e, "LHS factorisation");
  if (status) return fail3(LNS_ERR_PIVOT, "zero or non-finite pivot in the LHS factorisation");
  c->factored = true;
  return LNS_OK;
}

// v += r and the boundary values (itrBC3D); add = 0 applies only the latter.
template <typename RT>
int launch_update(lns_ctx3d* c, cd* v, const RT* r, int add, cudaStream_t st) {
  const Grid& g = c->g;
  const long long n = 5 * c->np;
  if (add) lns::a3::add_kernel<cd, RT><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, v, r);
  const int nt = g.nx + g.ny;
  lns::a3::bc_kernel<<<(nt + 127) / 128, 128, 0, st>>>(g, v, c->ops.ttop, c->ops.bump, c->ops.tleft,
                                                        c->ops.tright);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda3(e, "update kernels launch");
}

// nsteps steps of niter correctors on device v (src/impdrv3d.f90:130-356)
__global__ void avg_kernel(long long n, const cd* __restrict__ a, const cd* __restrict__ b, cd* __restrict__ w) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k < n) w[k] = cd{0.5 * (a[k].x + b[k].x), 0.5 * (a[k].y + b[k].y)};
}

// nsteps steps of the time scheme impl (src/impdrv3d.f90:130-356): 1
// backward Euler with the deck's alfa; 2 two-step backward, backward Euler
// for the first step of the context and rtb3D with alfa = 2/3 after it
// (the LHS formed and factored again once); 3 the midpoint rule, the
// operator applied to (v + vold)/2 with alfa = 1/2.
int run_steps(lns_ctx3d* c, cd* v, int nsteps, int niter, double* totres_dev, cudaStream_t st) {
  const bool mixed = c->prm.precision == LNS_MIXED;
  const int impl = c->prm.impl == 0 ? 1 : c->prm.impl;
  int rc;
  const size_t vbytes = sizeof(cd) * 5 * (size_t)c->np;
  for (int s = 0; s < nsteps; ++s) {
    const bool rtb = impl == 2 && c->lstep > 0;
    const double alfa = impl == 3 ? 0.5 : rtb ? 6.6666666666666666666e-1 : (impl == 2 ? 1.0 : c->prm.alfa);
    if (!c->factored || c->alfa_fac != alfa) {
      c->g.alfa = alfa;
      rc = mixed ? factor_all<cf>(c, st) : factor_all<cd>(c, st);
      if (rc) return rc;
      c->alfa_fac = alfa;
    }
    cudaError_t e = cudaSuccess;
    if (rtb) e = cudaMemcpyAsync(c->v2old, c->vold, vbytes, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(c->vold, v, vbytes, cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda3(e, "cudaMemcpyAsync vold");
    rc = launch_update<cd>(c, v, (const cd*)nullptr, 0, st);
    if (rc) return rc;
    for (int it = 0; it < niter; ++it) {
      double* res = (it == niter - 1 && totres_dev) ? totres_dev + s : c->dscal + 1;
      rc = mark(c, st);
      const cd* field = v;
      if (impl == 3) {
        const long long n = 5 * c->np;
        avg_kernel<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, v, c->vold, c->wavg);
        field = c->wavg;
      }
      const cd* v2 = rtb ? c->v2old : nullptr;
      if (mixed) {
        if (!rc) rc = launch_rhs(c, field, v, c->vold, v2, nullptr, c->r32, res, st);
        if (!rc) rc = mark(c, st);
        if (!rc) rc = sweep_x<cf>(c, c->r32, st);
        if (!rc) rc = mark(c, st);
        if (!rc) rc = sweep_y<cf>(c, c->r32, st);
        if (!rc) rc = mark(c, st);
        if (!rc) rc = launch_update<cf>(c, v, c->r32, 1, st);
      } else {
        if (!rc) rc = launch_rhs(c, field, v, c->vold, v2, c->r64, nullptr, res, st);
        if (!rc) rc = mark(c, st);
        if (!rc) rc = sweep_x<cd>(c, c->r64, st);
        if (!rc) rc = mark(c, st);
        if (!rc) rc = sweep_y<cd>(c, c->r64, st);
        if (!rc) rc = mark(c, st);
        if (!rc) rc = launch_update<cd>(c, v, c->r64, 1, st);
      }
      if (!rc) rc = mark(c, st);
      if (rc) return rc;
    }
    c->lstep += 1;
  }
  return LNS_OK;
}

}  // namespace

int lns_ctx3d_create_planes(const lns_params3d* p, lns_ctx3d** out, bool lin2d_planes);

// the rows j <= nbl that the linear 2D nonreflecting planes leave alone
int lns_ctx3d_set_nbl(lns_ctx3d* c, int nbl) {
  if (!c) return fail3(LNS_ERR_ARG, "set_nbl: null context");
  if (nbl < 0 || nbl > c->g.ny) return fail3(LNS_ERR_ARG, "set_nbl: nbl must be in 0..ny");
  c->g.nbl = nbl;
  c->factored = false;
  return LNS_OK;
}

extern "C" {

int lns_ctx3d_create(const lns_params3d* p, lns_ctx3d** out) { return lns_ctx3d_create_planes(p, out, false); }

}  // extern "C"

// lin2d_planes: the linear 2D context's plane codes are accepted as well
int lns_ctx3d_create_planes(const lns_params3d* p, lns_ctx3d** out, bool lin2d_planes) {
  if (!p || !out) return fail3(LNS_ERR_ARG, "ctx3d_create: null argument");
  *out = nullptr;
  if (p->nx < 8 || p->ny < 7) return fail3(LNS_ERR_ARG, "ctx3d_create: need nx >= 8 and ny >= 7");
  if ((long long)p->nx * p->ny > (1LL << 31) / 125)
    return fail3(LNS_ERR_ARG, "ctx3d_create: nx*ny too large for 32-bit launch indexing");
  if (!(p->dxi > 0.0) || !(p->deta > 0.0)) return fail3(LNS_ERR_ARG, "ctx3d_create: dxi and deta must be > 0");
  if (p->xper != 0 && p->xper != 1) return fail3(LNS_ERR_ARG, "ctx3d_create: xper must be 0 or 1");
  if (!p->xper) {
    if (p->left != 0 && p->left != 1 && p->left != 4 && p->left != 5 && p->left != 7 &&
        !(lin2d_planes && (p->left == lns::a3::kLinSymLeft || p->left == lns::a3::kLinNrLeft)))
      return fail3(LNS_ERR_ARG, "ctx3d_create: left must be 0, 1, 4, 5 or 7 (xper = 0)");
    if (p->right != 0 && p->right != 4 && p->right != 5 && p->right != 7 && p->right != 8 &&
        !(lin2d_planes && p->right == lns::a3::kLinNrRight))
      return fail3(LNS_ERR_ARG, "ctx3d_create: right must be 0, 4, 5, 7 or 8 (xper = 0)");
    // right 5's wave reads x(j,nx) of the (nx,ny) array (src/rhsbc3d.f90:299), inside it only when ny >= nx
    if (p->right == 5 && p->ny < p->nx) return fail3(LNS_ERR_ARG, "ctx3d_create: right 5 needs ny >= nx");
    // the symmetric xi LHS rows read ABhi through a (6,ny,nx) view of the (6,nx,ny) array
    // (src/lhsbs1f3d.f90:17), which stays inside it only when ny <= nx
    if ((p->left == 7 || p->left == lns::a3::kLinSymLeft || p->right == 7) && p->ny > p->nx)
      return fail3(LNS_ERR_ARG, "ctx3d_create: symmetry planes (left or right 7) need ny <= nx");
    // the reference reads the eigenfunction only for left 4 (src/gendist.f90:18)
    if (p->right == 4 && p->left != 4) return fail3(LNS_ERR_ARG, "ctx3d_create: right 4 needs left 4");
  }
  if (p->yper != 0 && p->yper != 1) return fail3(LNS_ERR_ARG, "ctx3d_create: yper must be 0 or 1");
  if (p->navier != 0 && p->navier != 1) return fail3(LNS_ERR_ARG, "ctx3d_create: navier must be 0 or 1");
  if (p->yper == 1 && p->ny < 8) return fail3(LNS_ERR_ARG, "ctx3d_create: a periodic eta direction needs ny >= 8");
  if (!p->yper) {  // the wall and top rows (a periodic eta direction has neither, src/input.f90:126-132)
    if (p->navier != 1)
      return fail3(LNS_ERR_ARG, "ctx3d_create: an inviscid run (navier = 0) needs a periodic eta direction");
    if (p->wall != 1 && p->wall != 2 && p->wall != 3) return fail3(LNS_ERR_ARG, "ctx3d_create: wall must be 1, 2 or 3");
    if (p->wallt != 0 && p->wallt != 1) return fail3(LNS_ERR_ARG, "ctx3d_create: wallt must be 0 or 1");
    if (p->top != 0 && p->top != 1) return fail3(LNS_ERR_ARG, "ctx3d_create: top must be 0 or 1");
  } else if (p->top == 1 || p->wall == 3) {
    return fail3(LNS_ERR_ARG, "ctx3d_create: a periodic eta direction has no forced top or bump wall");
  }
  if (p->loctime != 0 && p->loctime != 1) return fail3(LNS_ERR_ARG, "ctx3d_create: loctime must be 0 or 1");
  if (p->precision != LNS_FP64 && p->precision != LNS_MIXED)
    return fail3(LNS_ERR_ARG, "ctx3d_create: precision must be LNS_FP64 or LNS_MIXED");
  if (p->impl < 0 || p->impl > 3) return fail3(LNS_ERR_ARG, "ctx3d_create: impl must be 1, 2 or 3 (0 means 1)");
  if (!(p->eps_e >= 0.0) || !std::isfinite(p->eps_e))
    return fail3(LNS_ERR_ARG, "ctx3d_create: eps_e must be finite and >= 0");
  if (p->ispg < 0) return fail3(LNS_ERR_ARG, "ctx3d_create: ispg must be >= 0");
  lns_ctx3d* c = new lns_ctx3d();
  c->prm = *p;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->device);
  if (e != cudaSuccess) {
    delete c;
    return cuda3(e, "cudaGetDevice");
  }
  Grid& g = c->g;
  g.nx = p->nx; g.ny = p->ny; g.dxi = p->dxi; g.deta = p->deta;
  g.Ma = p->Ma; g.Re = p->Re; g.Pr = p->Pr; g.gamma = p->gamma;
  g.gamma1 = p->gamma1 != 0.0 ? p->gamma1 : p->gamma - 1.0;
  g.omega = p->omega; g.kz = p->beta; g.alfa = p->alfa;
  g.xper = p->xper; g.yper = p->yper; g.navier = p->navier; g.wall = p->wall; g.wallt = p->wallt; g.top = p->top;
  g.left = p->xper ? -1 : p->left;
  g.right = p->xper ? -1 : p->right;
  g.dxinv = 1.0 / p->dxi; g.dyinv = 1.0 / p->deta;
  g.dxsinv = 1.0 / (p->dxi * p->dxi); g.dysinv = 1.0 / (p->deta * p->deta);
  coef1(p->optx, g.dxinv, g.gx);
  coef1(p->opty, g.dyinv, g.gy);
  coef2(p->optx, g.dxsinv, g.dx2);
  coef2(p->opty, g.dysinv, g.dy2);
  const long long np = (long long)p->nx * p->ny;
  c->np = np;
  c->nparts = std::max(((p->nx + 127) / 128) * p->ny, (int)((np + 255) / 256));
  const bool mixed = p->precision == LNS_MIXED;
  const size_t el = mixed ? sizeof(cf) : sizeof(cd);
  void* q = nullptr;
  int rc = LNS_OK;
  auto A = [&](size_t bytes, void** dst) {
    if (!rc) rc = dalloc(c, bytes, dst);
  };
  A(sizeof(double) * 10 * np, &q); c->metrics = (double*)q;
  A(sizeof(double) * 5 * np, &q); c->vm = (double*)q;
  A(sizeof(double) * (4 * 25 + 4 * 6 + 1) * np, &q); c->opbuf = (double*)q;
  A(sizeof(cd) * 5 * np, &q); c->v = (cd*)q;
  A(sizeof(cd) * 5 * np, &q); c->vold = (cd*)q;
  A(sizeof(cd) * 5 * np, &q); c->c1v = (cd*)q;
  if (p->impl == 2) { A(sizeof(cd) * 5 * np, &q); c->v2old = (cd*)q; }
  if (p->impl == 3) { A(sizeof(cd) * 5 * np, &q); c->wavg = (cd*)q; }
  if (p->ispg != 0) { A(sizeof(double) * np, &q); c->spg = (double*)q; }
  if (p->ispg >= 2 && p->ispg <= 4) {
    A(sizeof(double) * np, &q); c->spg_b = (double*)q;
    A(sizeof(double) * 10 * np, &q); c->vt = (double*)q;
  }
  if (p->ispg == 2 || p->ispg == 3) { A(sizeof(double) * np, &q); c->spg_a = (double*)q; }
  const bool left_wave = !p->xper && p->left == 1;
  const bool plane5 = !p->xper && (p->left == 5 || p->right == 5);
  if (p->ispg == 2 || p->ispg == 3 || p->top == 1 || left_wave || plane5) {
    A(sizeof(double) * np, &q); c->xc = (double*)q;
    A(sizeof(double) * p->nx, &q); c->wamp = (double*)q;
  }
  if (p->top == 1) { A(sizeof(double) * 10 * p->nx, &q); c->ttop = (double*)q; }
  if (left_wave || (!p->xper && (p->left == 4 || p->left == 5))) {
    A(sizeof(double) * 10 * p->ny, &q);
    c->tleft = (double*)q;
  }
  if (!p->xper && (p->right == 4 || p->right == 5)) { A(sizeof(double) * 10 * p->ny, &q); c->tright = (double*)q; }
  // the linear 2D nonreflecting planes' factors; right 1 also writes column 1's row
  if (!p->xper && (p->left == lns::a3::kLinNrLeft || p->right == lns::a3::kLinNrRight)) {
    A(sizeof(double) * 4 * p->ny, &q);
    c->tleft = (double*)q;
  }
  if (!p->xper && p->right == lns::a3::kLinNrRight) { A(sizeof(double) * 4 * p->ny, &q); c->tright = (double*)q; }
  if (p->wall == 3) { A(sizeof(double) * 10 * p->nx, &q); c->bump = (double*)q; }
  if (p->eps_e != 0.0) { A(sizeof(double) * np, &q); c->buff = (double*)q; }
  if (mixed) { A(sizeof(cf) * 5 * np, &q); c->r32 = (cf*)q; }
  else { A(sizeof(cd) * 5 * np, &q); c->r64 = (cd*)q; }
  A(sizeof(cd) * 125 * np, &c->matx);
  A(sizeof(cd) * 125 * np, &c->maty);
  if (p->xper) {
    A(sizeof(cd) * 50 * np, &c->perx);
    A(sizeof(cd) * 50 * np, &c->per2x);
  }
  A(el * 125 * np, &c->chnx);
  A(el * 125 * np, &c->chny);
  if (p->xper) {
    if (mixed) A(el * 50 * np, &c->fillE);
    else c->fillE = c->perx;  // W replaces the reference fill after the factorisation
    A(sizeof(cd) * lns::chain::kBordCd * p->ny, &c->bordx);
  }
  if (p->yper) {
    A(sizeof(cd) * 50 * np, &c->pery);
    A(sizeof(cd) * 50 * np, &c->per2y);
    if (mixed) A(el * 50 * np, &c->fillEy);
    else c->fillEy = c->pery;
    A(sizeof(cd) * lns::chain::kBordCd * p->nx, &c->bordy);
  }
  A(sizeof(double) * c->nparts, &q); c->part = (double*)q;
  A(sizeof(double) * 3, &q); c->dscal = (double*)q;  // cfl, scratch residual, running residual
  A(sizeof(int), &q); c->status = (int*)q;
  if (!rc) rc = res_reserve(c, 64);
  if (rc) {
    free_all(c);
    delete c;
    return rc;
  }
  if (!mixed) c->r32 = nullptr;
  cudaError_t ez = cudaMemset(c->dscal, 0, sizeof(double) * 3);
  if (ez != cudaSuccess) {
    free_all(c);
    delete c;
    return cuda3(ez, "cudaMemset");
  }
  double* o = c->opbuf;
  c->ops.np = np;
  c->ops.Ah = o; c->ops.Bh = o + 25 * np; c->ops.Dh = o + 50 * np; c->ops.Dhi = o + 75 * np;
  c->ops.V11 = o + 100 * np; c->ops.V12 = o + 106 * np; c->ops.V22 = o + 112 * np; c->ops.AB = o + 118 * np;
  c->ops.dtl = o + 124 * np;
  if (c->wamp) {  // the reference's default amplitudes (useAmp false): ones
    std::vector<double> ones((size_t)p->nx, 1.0);
    ez = cudaMemcpy(c->wamp, ones.data(), sizeof(double) * p->nx, cudaMemcpyHostToDevice);
    if (ez != cudaSuccess) {
      free_all(c);
      delete c;
      return cuda3(ez, "wamp init");
    }
  }
  if (c->buff) {
    // the reference's default buffer (ibuff = 0, src/buffer.f90): ones
    std::vector<double> ones((size_t)np, 1.0);
    ez = cudaMemcpy(c->buff, ones.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
    if (ez != cudaSuccess) {
      free_all(c);
      delete c;
      return cuda3(ez, "buffer init");
    }
    c->ops.buff = c->buff;
    c->ops.eps_e = p->eps_e;
  }
  *out = c;
  return LNS_OK;
}

extern "C" {

int lns_ctx3d_destroy(lns_ctx3d* c) {
  if (!c) return LNS_OK;
  free_all(c);
  delete c;
  return LNS_OK;
}

size_t lns_ctx3d_bytes(const lns_ctx3d* c) { return c ? c->bytes : 0; }

}  // extern "C"

namespace {
int need_data(const lns_ctx3d* c, const char* who) {
  if (!c->have_mean) return fail3(LNS_ERR_ARG, std::string(who) + ": upload the metrics and the mean flow first");
  if (c->prm.ispg != 0 && !c->have_sponge)
    return fail3(LNS_ERR_ARG, std::string(who) + ": ispg != 0: upload the sponge first");
  if (!c->prm.xper && c->prm.left == 4 && !c->have_profile)
    return fail3(LNS_ERR_ARG, std::string(who) + ": left 4: upload the eigenfunction (lns_upload_profile3d) first");
  const bool wave_planes = !c->prm.xper && (c->prm.left == 1 || c->prm.left == 5 || c->prm.right == 5);
  if ((c->prm.ispg == 2 || c->prm.ispg == 3 || c->prm.top == 1 || wave_planes) && !c->have_inflow)
    return fail3(LNS_ERR_ARG,
                 std::string(who) + ": ispg 2, 3, top 1 or left 1: upload the wave data (lns_upload_inflow3d) first");
  if (c->prm.wall == 3 && !c->have_bump)
    return fail3(LNS_ERR_ARG, std::string(who) + ": wall 3: upload the bump (lns_upload_bump3d) first");
  if (c->prm.ispg == 4 && !c->have_target)
    return fail3(LNS_ERR_ARG, std::string(who) + ": ispg 4: upload the sponge target (lns_upload_sponge_target3d) first");
  return LNS_OK;
}

// the inflow sponge's target, once the mean flow and the inflow data are in
int make_inflow_target(lns_ctx3d* c) {
  if (!c->have_inflow || !c->have_mean) return LNS_OK;
  const long long np = c->np;
  if (c->prm.ispg == 2 || c->prm.ispg == 3)
    lns::a3::inflow_target_kernel<<<(unsigned)((np + 255) / 256), 256>>>(
        c->g, c->prm.ispg == 3, 0, 0, c->vm, c->xc, c->wamp, c->x0, reinterpret_cast<cd*>(c->vt));
  if (c->prm.top == 1) {
    lns::a3::inflow_target_kernel<<<(unsigned)((c->g.nx + 127) / 128), 128>>>(
        c->g, 1, c->g.ny, 0, c->vm, c->xc, c->wamp, c->x0, reinterpret_cast<cd*>(c->ttop));
    c->ops.ttop = c->ttop;
  }
  if (!c->prm.xper && c->prm.left == 5) {
    lns::a3::plane5_target_kernel<<<(unsigned)((c->g.ny + 127) / 128), 128>>>(c->g, 1, c->vm, c->xc,
                                                                             reinterpret_cast<cd*>(c->tleft));
    c->ops.tleft = c->tleft;
  }
  if (!c->prm.xper && c->prm.right == 5) {
    lns::a3::plane5_target_kernel<<<(unsigned)((c->g.ny + 127) / 128), 128>>>(c->g, c->g.nx, c->vm, c->xc,
                                                                             reinterpret_cast<cd*>(c->tright));
    c->ops.tright = c->tright;
  }
  if (c->tleft && c->prm.left == 1) {
    lns::a3::inflow_target_kernel<<<(unsigned)((c->g.ny + 127) / 128), 128>>>(
        c->g, 0, 0, 1, c->vm, c->xc, c->wamp, c->x0, reinterpret_cast<cd*>(c->tleft));
    c->ops.tleft = c->tleft;
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  return e == cudaSuccess ? LNS_OK : cuda3(e, "inflow_target_kernel");
}
}  // namespace

extern "C" {

int lns_upload_sponge3d(lns_ctx3d* c, const double* spg, const double* spg2) {
  if (!c || !spg) return fail3(LNS_ERR_ARG, "upload_sponge3d: null argument");
  if (c->prm.ispg == 0) return fail3(LNS_ERR_ARG, "upload_sponge3d: the context was created with ispg = 0");
  if (c->prm.ispg > 1 && !spg2) return fail3(LNS_ERR_ARG, "upload_sponge3d: ispg > 1 needs spg2");
  int rc = check_device(c);
  if (rc) return rc;
  // the LHS (src/lhs2f3d.f90:207-224) and the double sponge's RHS
  // (src/lrhs3d.f90:232-240) use spg + spg2, the eigenfunction sponge's RHS
  // too (src/sponge.f90:600): add once here
  std::vector<double> h(spg, spg + c->np);
  if (c->prm.ispg > 1)
    for (long long k = 0; k < c->np; ++k) h[k] = spg[k] + spg2[k];
  cudaError_t e = cudaMemcpy(c->spg, h.data(), sizeof(double) * c->np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && c->spg_a) e = cudaMemcpy(c->spg_a, spg, sizeof(double) * c->np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && c->spg_b)
    e = cudaMemcpy(c->spg_b, c->spg_a ? spg2 : h.data(), sizeof(double) * c->np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload sponge");
  c->ops.spg = c->spg;
  c->ops.spg_a = c->spg_a;
  c->ops.spg_b = c->spg_b;
  c->ops.vt = c->vt;
  c->have_sponge = true;
  c->factored = false;
  return LNS_OK;
}

int lns_upload_inflow3d(lns_ctx3d* c, const double* x, const double* wamp, double x0) {
  if (!c || !x) return fail3(LNS_ERR_ARG, "upload_inflow3d: null argument");
  if (c->prm.ispg != 2 && c->prm.ispg != 3 && c->prm.top != 1 &&
      !(!c->prm.xper && (c->prm.left == 1 || c->prm.left == 5 || c->prm.right == 5)))
    return fail3(LNS_ERR_ARG, "upload_inflow3d: needs ispg 2 or 3, top 1, left 1 or 5, or right 5");
  if (c->prm.ispg == 3 && !wamp) return fail3(LNS_ERR_ARG, "upload_inflow3d: ispg 3 needs wamp");
  if (!std::isfinite(x0)) return fail3(LNS_ERR_ARG, "upload_inflow3d: x0 must be finite");
  int rc = check_device(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->xc, x, sizeof(double) * c->np, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && wamp) e = cudaMemcpy(c->wamp, wamp, sizeof(double) * c->g.nx, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload inflow data");
  c->x0 = x0;
  c->have_inflow = true;
  return make_inflow_target(c);
}

int lns_upload_profile3d(lns_ctx3d* c, const double* prof, const double* xr, double lalpha_re, double lalpha_im) {
  if (!c || !prof) return fail3(LNS_ERR_ARG, "upload_profile3d: null argument");
  if (c->prm.xper || c->prm.left != 4) return fail3(LNS_ERR_ARG, "upload_profile3d: needs xper = 0 and left 4");
  if (c->prm.right == 4 && !xr) return fail3(LNS_ERR_ARG, "upload_profile3d: right 4 needs x of column nx");
  if (!std::isfinite(lalpha_re) || !std::isfinite(lalpha_im))
    return fail3(LNS_ERR_ARG, "upload_profile3d: lalpha must be finite");
  int rc = check_device(c);
  if (rc) return rc;
  const int ny = c->g.ny;
  cudaError_t e = cudaMemcpy(c->tleft, prof, sizeof(double) * 10 * ny, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && c->tright) {
    // src/itrbc3d.f90:357-381: cmplx(re, im) * exp(im * lalpha * x(nx,j))
    std::vector<double> h((size_t)10 * ny);
    const std::complex<double> ia(-lalpha_im, lalpha_re);
    for (int j = 0; j < ny; ++j) {
      const std::complex<double> f = std::exp(ia * xr[j]);
      for (int m = 0; m < 5; ++m) {
        const std::complex<double> z = std::complex<double>(prof[10 * j + 2 * m], prof[10 * j + 2 * m + 1]) * f;
        h[10 * j + 2 * m] = z.real();
        h[10 * j + 2 * m + 1] = z.imag();
      }
    }
    e = cudaMemcpy(c->tright, h.data(), sizeof(double) * 10 * ny, cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) return cuda3(e, "upload profile");
  c->ops.tleft = c->tleft;
  c->ops.tright = c->tright;
  c->have_profile = true;
  return LNS_OK;
}

int lns_upload_bump3d(lns_ctx3d* c, const double* bump) {
  if (!c || !bump) return fail3(LNS_ERR_ARG, "upload_bump3d: null argument");
  if (c->prm.wall != 3) return fail3(LNS_ERR_ARG, "upload_bump3d: needs wall 3");
  int rc = check_device(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->bump, bump, sizeof(double) * 10 * c->g.nx, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload bump");
  c->ops.bump = c->bump;
  c->have_bump = true;
  return LNS_OK;
}

int lns_upload_sponge_target3d(lns_ctx3d* c, const double* cvic) {
  if (!c || !cvic) return fail3(LNS_ERR_ARG, "upload_sponge_target3d: null argument");
  if (c->prm.ispg != 4) return fail3(LNS_ERR_ARG, "upload_sponge_target3d: needs ispg 4");
  int rc = check_device(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->vt, cvic, sizeof(double) * 10 * c->np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload sponge target");
  c->have_target = true;
  return LNS_OK;
}

int lns_upload_buffer3d(lns_ctx3d* c, const double* buff) {
  if (!c || !buff) return fail3(LNS_ERR_ARG, "upload_buffer3d: null argument");
  if (!c->buff) return fail3(LNS_ERR_ARG, "upload_buffer3d: the context was created with eps_e = 0");
  int rc = check_device(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->buff, buff, sizeof(double) * c->np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload buffer");
  c->factored = false;
  return LNS_OK;
}

int lns_upload_metrics3d(lns_ctx3d* c, const double* metrics) {
  if (!c || !metrics) return fail3(LNS_ERR_ARG, "upload_metrics3d: null argument");
  int rc = check_device(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->metrics, metrics, sizeof(double) * 10 * c->np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload metrics");
  c->have_metrics = true;
  c->have_mean = false;
  c->factored = false;
  return LNS_OK;
}

int lns_upload_mean3d(lns_ctx3d* c, const double* vm, double* cfl) {
  if (!c || !vm) return fail3(LNS_ERR_ARG, "upload_mean3d: null argument");
  if (!c->have_metrics) return fail3(LNS_ERR_ARG, "upload_mean3d: upload the metrics first");
  int rc = check_device(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->vm, vm, sizeof(double) * 5 * c->np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload mean flow");
  const Grid& g = c->g;
  const Metrics mt = metrics_of(c);
  lns::a3::genmtrx_kernel<<<pt_grid(g), 128>>>(g, c->vm, mt, c->ops);
  const int nb = (int)((c->np + 255) / 256);
  lns::a3::cfl_kernel<<<nb, 256>>>(g, c->vm, mt, c->ops.dtl, c->part);
  lns::a3::dtl_kernel<<<152, 256>>>(c->np, nb, c->part, c->ops.dtl, c->prm.cflmax, c->prm.dtmax, c->prm.loctime,
                                    c->dscal);
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda3(e, "operator kernels launch");
  double h = 0.0;
  e = cudaMemcpy(&h, c->dscal, sizeof(double), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda3(e, "operator build");
  if (cfl) *cfl = h;
  c->have_mean = true;
  c->factored = false;
  if (!c->prm.xper && (c->prm.left == lns::a3::kLinNrLeft || c->prm.right == lns::a3::kLinNrRight)) {
    const unsigned nbj = (unsigned)((g.ny + 127) / 128);
    lns::a3::nr_coef_kernel<<<nbj, 128>>>(g, 1, c->vm, c->tleft);
    c->ops.tleft = c->tleft;
    if (c->prm.right == lns::a3::kLinNrRight) {
      lns::a3::nr_coef_kernel<<<nbj, 128>>>(g, g.nx, c->vm, c->tright);
      c->ops.tright = c->tright;
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) return cuda3(e, "nr_coef_kernel");
  }
  return make_inflow_target(c);
}

int lns_itrbc3d_dev(lns_ctx3d* c, double* v, void* stream) {
  if (!c || !v) return fail3(LNS_ERR_ARG, "itrbc3d: null argument");
  if (int rn = need_data(c, "itrbc3d")) return rn;
  int rc = check_device(c);
  if (rc) return rc;
  return launch_update<cd>(c, (cd*)v, nullptr, 0, (cudaStream_t)stream);
}

int lns_step3d_dev(lns_ctx3d* c, double* v, int32_t nsteps, int32_t niter, double* totres_dev, void* stream) {
  if (!c || !v) return fail3(LNS_ERR_ARG, "step3d: null argument");
  if (nsteps < 0 || niter < 1) return fail3(LNS_ERR_ARG, "step3d: need nsteps >= 0 and niter >= 1");
  if (int rn = need_data(c, "step3d")) return rn;
  int rc = check_device(c);
  if (rc) return rc;
  return run_steps(c, (cd*)v, nsteps, niter, totres_dev, (cudaStream_t)stream);
}

int lns_step3d(lns_ctx3d* c, double* v, int32_t nsteps, int32_t niter, double* totres) {
  if (!c || !v) return fail3(LNS_ERR_ARG, "step3d: null argument");
  if (nsteps < 0 || niter < 1) return fail3(LNS_ERR_ARG, "step3d: need nsteps >= 0 and niter >= 1");
  if (int rn = need_data(c, "step3d")) return rn;
  int rc = check_device(c);
  if (rc) return rc;
  if (totres && (rc = res_reserve(c, nsteps))) return rc;
  const size_t vbytes = sizeof(cd) * 5 * (size_t)c->np;
  cudaError_t e = cudaMemcpy(c->v, v, vbytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload v");
  rc = run_steps(c, c->v, nsteps, niter, totres ? c->res_dev : nullptr, 0);
  if (rc) return rc;
  e = cudaMemcpy(v, c->v, vbytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda3(e, "download v");
  if (totres && nsteps > 0) {
    e = cudaMemcpy(totres, c->res_dev, sizeof(double) * nsteps, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda3(e, "download totres");
  }
  return LNS_OK;
}

int lns_rhs3d_dev(lns_ctx3d* c, const double* v, const double* vold, double* r, double* totres_dev, void* stream) {
  if (!c || !v || !vold || !r) return fail3(LNS_ERR_ARG, "rhs3d: null argument");
  if (int rn = need_data(c, "rhs3d")) return rn;
  int rc = check_device(c);
  if (rc) return rc;
  return launch_rhs(c, (const cd*)v, (const cd*)v, (const cd*)vold, nullptr, (cd*)r, nullptr,
                    totres_dev ? totres_dev : c->dscal + 1, (cudaStream_t)stream);
}

int lns_lhs3d_dev(lns_ctx3d* c, int32_t dir, double* mat, void* stream) {
  if (!c || !mat) return fail3(LNS_ERR_ARG, "lhs3d: null argument");
  if (dir != 1 && dir != 2) return fail3(LNS_ERR_ARG, "lhs3d: dir must be 1 or 2");
  if (int rn = need_data(c, "lhs3d")) return rn;
  int rc = check_device(c);
  if (rc) return rc;
  return launch_lhs<cd>(c, dir, (cd*)mat, (cudaStream_t)stream);
}

int lns_ctx3d_set_row_pairs(lns_ctx3d* c, int32_t on) {
  if (!c) return fail3(LNS_ERR_ARG, "ctx3d_set_row_pairs: null context");
  if (on != 0 && on != 1) return fail3(LNS_ERR_ARG, "ctx3d_set_row_pairs: on must be 0 or 1");
  if (c->pair_ok != (on == 1)) {
    c->pair_ok = on == 1;
    c->factored = false;  // the records are formed again in the chosen form
  }
  return LNS_OK;
}

int lns_ctx3d_profile(lns_ctx3d* c, int32_t on) {
  if (!c) return fail3(LNS_ERR_ARG, "ctx3d_profile: null context");
  c->profile = on != 0;
  c->ev_used = 0;
  return LNS_OK;
}

int lns_ctx3d_profile_read(lns_ctx3d* c, double* ms, int32_t* ncorr) {
  if (!c || !ms || !ncorr) return fail3(LNS_ERR_ARG, "ctx3d_profile_read: null argument");
  constexpr int kSeg = LNS_PROFILE_SEGMENTS;
  for (int k = 0; k < kSeg; ++k) ms[k] = 0.0;
  *ncorr = 0;
  const size_t n = c->ev_used / (kSeg + 1);
  for (size_t q = 0; q < n; ++q) {
    for (int k = 0; k < kSeg; ++k) {
      cudaError_t e = cudaEventSynchronize(c->events[(kSeg + 1) * q + k + 1]);
      float t = 0.f;
      if (e == cudaSuccess)
        e = cudaEventElapsedTime(&t, c->events[(kSeg + 1) * q + k], c->events[(kSeg + 1) * q + k + 1]);
      if (e != cudaSuccess) return cuda3(e, "profile events");
      ms[k] += t;
    }
  }
  *ncorr = (int32_t)n;
  c->ev_used = 0;
  return LNS_OK;
}

int lns_get_field3d(lns_ctx3d* c, int32_t which, double* out) {
  if (!c || !out) return fail3(LNS_ERR_ARG, "get_field3d: null argument");
  if (which < 0 || which > 8) return fail3(LNS_ERR_ARG, "get_field3d: which must be 0..8");
  if (int rn = need_data(c, "get_field3d")) return rn;
  int rc = check_device(c);
  if (rc) return rc;
  const long long np = c->np;
  const double* src[9] = {c->ops.Ah, c->ops.Bh, c->ops.Dh, c->ops.Dhi, c->ops.V11,
                          c->ops.V12, c->ops.V22, c->ops.AB, c->ops.dtl};
  const int nel = which < 4 ? 25 : (which < 8 ? 6 : 1);
  std::vector<double> h((size_t)nel * np);
  cudaError_t e = cudaMemcpy(h.data(), src[which], sizeof(double) * h.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda3(e, "get_field3d copy");
  for (long long p = 0; p < np; ++p)
    for (int k = 0; k < nel; ++k) out[k + (long long)nel * p] = h[(size_t)k * np + p];
  return LNS_OK;
}

}  // extern "C"

// ======================================================================
// Batches of problems (lns_batch3d_*): one launch per phase for all
// problems, the step captured once as a CUDA graph
// ======================================================================
struct lns_batch3d {
  int P = 0;
  int cap = 0;            // problems the per-problem device arrays hold
  bool owns_ctx = true;   // a server's batch borrows its requests' contexts
  bool mixed = false;
  int device = -1;
  int W = lns::chain::kChainWarps;  // lines per CTA of the recurrences
  std::vector<lns_ctx3d*> ctx;
  std::vector<void*> allocs;
  size_t bytes = 0;
  cudaStream_t st = nullptr;
  lns::a3::StepArgs* d_args = nullptr;
  lns::chain::Args *d_ax = nullptr, *d_ay = nullptr;
  int* d_active = nullptr;
  int* d_step = nullptr;
  double* d_hist = nullptr;
  long long hist_cap = 0;  // entries (steps x problems)
  // the work tables of the phases (kTables of them), each in a buffer that
  // only grows; their lengths and the problem count in d_cnt
  int2 *t_elem = nullptr, *t_col = nullptr, *t_sx = nullptr, *t_fx = nullptr, *t_tx = nullptr, *t_lx = nullptr,
       *t_sy = nullptr, *t_fy = nullptr;
  int4* t_pts = nullptr;
  int t_cap[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // entries each table buffer holds
  int* d_cnt = nullptr;  // [0..8] table lengths (kCnt*), [9] problems
  int* d_next = nullptr;  // the recurrences' entry counters, four per corrector
  int next_cap = 0;
  int sms = 0;           // the device's SMs
  // persistent grids (CTAs) of the batched kernels, as many as stay resident
  unsigned g_elem = 0, g_col = 0, g_pts = 0, g_rhs = 0, g_res = 0, g_scale = 0, g_chain = 0, g_tail = 0,
           g_fill = 0;
  cudaGraphExec_t exec = nullptr;
  int exec_W = 0, exec_niter = 0;
  bool exec_narrow = true;
  int captures = 0;      // step graphs captured so far
  std::vector<void*> table_allocs;  // the table buffers
  std::vector<int> active;
  std::vector<bool> uploaded;
};

namespace {

int balloc(lns_batch3d* b, size_t bytes, void** out) {
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    *out = nullptr;
    return fail3(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  b->allocs.push_back(*out);
  b->bytes += bytes;
  return LNS_OK;
}

// slots of the table lengths in lns_batch3d::d_cnt
enum { kCntElem, kCntCol, kCntPts, kCntSx, kCntFx, kCntTx, kCntLx, kCntSy, kCntFy, kCntProb, kCnt };

void drop_exec(lns_batch3d* b) {
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
}

// Writes table `slot` into its buffer, growing the buffer (and dropping the
// captured step, which holds the old address) when it is too small.
template <typename E>
int upload_table(lns_batch3d* b, const std::vector<E>& h, E** d, int slot, std::vector<int>& len) {
  if ((int)h.size() > b->t_cap[slot] || !*d) {
    const int cap = std::max(std::max((int)h.size(), 2 * b->t_cap[slot]), 1);
    void* q = nullptr;
    cudaError_t ea = cudaMalloc(&q, sizeof(E) * (size_t)cap);
    if (ea != cudaSuccess) return fail3(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(ea));
    if (*d) {
      cudaFree(*d);
      b->table_allocs.erase(std::find(b->table_allocs.begin(), b->table_allocs.end(), (void*)*d));
    }
    b->table_allocs.push_back(q);
    *d = (E*)q;
    b->t_cap[slot] = cap;
    drop_exec(b);
  }
  cudaError_t e = cudaMemcpy(*d, h.data(), sizeof(E) * h.size(), cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload work table");
  len[slot] = (int)h.size();
  return LNS_OK;
}

// The work tables of every phase, from the problems' sizes and the
// recurrences' lines per CTA W, and their lengths; a captured step stays
// valid unless a table buffer had to grow.
int build_tables(lns_batch3d* b) {
  if (!b->d_cnt) {
    cudaError_t e = cudaMalloc(&b->d_cnt, sizeof(int) * kCnt);
    if (e != cudaSuccess) return fail3(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    b->table_allocs.push_back(b->d_cnt);
  }
  std::vector<int> len(kCnt, 0);
  len[kCntProb] = b->P;
  std::vector<int2> te, tc, tsx, tfx, ttx, tlx, tsy, tfy;
  std::vector<int4> tp;
  for (int p = 0; p < b->P; ++p) {
    const Grid& g = b->ctx[p]->g;
    const long long np = b->ctx[p]->np;
    for (long long k = 0; k < (5 * np + 255) / 256; ++k) te.push_back(make_int2(p, (int)k));
    for (int k = 0; k < (g.nx + g.ny + 127) / 128; ++k) tc.push_back(make_int2(p, k));
    const int nbx = (g.nx + 127) / 128;
    for (int by = 0; by < g.ny; ++by)
      for (int bx = 0; bx < nbx; ++bx) tp.push_back(make_int4(p, bx, by, 0));
    const long long nxp = (long long)(g.nx - 1) * g.ny, nyp = (long long)g.ny * g.nx;
    for (long long k = 0; k < lns::chain::scale_blocks(nxp); ++k) tsx.push_back(make_int2(p, (int)k));
    for (int k = 0; k < (g.ny + b->W - 1) / b->W; ++k) tfx.push_back(make_int2(p, k));
    for (int k = 0; k < (g.ny + lns::chain::kBTailLines - 1) / lns::chain::kBTailLines; ++k)
      ttx.push_back(make_int2(p, k));
    for (long long k = 0; k < lns::chain::fill_blocks((long long)(g.nx - 1 - 2) * g.ny); ++k) tlx.push_back(make_int2(p, (int)k));
    for (long long k = 0; k < lns::chain::scale_blocks(nyp); ++k) tsy.push_back(make_int2(p, (int)k));
    for (int k = 0; k < (g.nx + b->W - 1) / b->W; ++k) tfy.push_back(make_int2(p, k));
  }
  int rc = upload_table(b, te, &b->t_elem, kCntElem, len);
  if (!rc) rc = upload_table(b, tc, &b->t_col, kCntCol, len);
  if (!rc) rc = upload_table(b, tp, &b->t_pts, kCntPts, len);
  if (!rc) rc = upload_table(b, tsx, &b->t_sx, kCntSx, len);
  if (!rc) rc = upload_table(b, tfx, &b->t_fx, kCntFx, len);
  if (!rc) rc = upload_table(b, ttx, &b->t_tx, kCntTx, len);
  if (!rc) rc = upload_table(b, tlx, &b->t_lx, kCntLx, len);
  if (!rc) rc = upload_table(b, tsy, &b->t_sy, kCntSy, len);
  if (!rc) rc = upload_table(b, tfy, &b->t_fy, kCntFy, len);
  if (!rc) {
    cudaError_t e = cudaMemcpy(b->d_cnt, len.data(), sizeof(int) * kCnt, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda3(e, "upload table lengths");
  }
  return rc;
}

// One step of niter correctors of every active problem, enqueued on b->st.
template <typename T, int W>
int enqueue_step(lns_batch3d* b, int niter) {
  namespace a3 = lns::a3;
  namespace ch = lns::chain;
  cudaStream_t st = b->st;
  const size_t sm = ch::chain_smem_bytes<T>(W);
  const bool narrow = b->exec_narrow;  // every problem's stencils are five-point
  // persistent grids (set_grids), the tables' lengths in d_cnt, and the
  // recurrences' entry counters cleared at the start of the step
  const int* n = b->d_cnt;
  cudaError_t em = cudaMemsetAsync(b->d_next, 0, sizeof(int) * 4 * niter, st);
  if (em != cudaSuccess) return cuda3(em, "clear entry counters");
  a3::copy_batch_kernel<<<b->g_elem, 256, 0, st>>>(b->d_args, b->t_elem, b->d_active, n + kCntElem);
  a3::bc_batch_kernel<<<b->g_col, 128, 0, st>>>(b->d_args, b->t_col, b->d_active, n + kCntCol);
  for (int it = 0; it < niter; ++it) {
    int* next = b->d_next + 4 * it;
    a3::grad1_batch_kernel<<<b->g_pts, 128, 0, st>>>(b->d_args, b->t_pts, b->d_active, n + kCntPts);
    if (narrow)
      a3::rhs_batch_kernel<true><<<b->g_rhs, 128, 0, st>>>(b->d_args, b->t_pts, b->d_active, n + kCntPts,
                                                           b->mixed ? 1 : 0);
    else
      a3::rhs_batch_kernel<false><<<b->g_rhs, 128, 0, st>>>(b->d_args, b->t_pts, b->d_active, n + kCntPts,
                                                            b->mixed ? 1 : 0);
    a3::resid_batch_kernel<<<b->g_res, 256, 0, st>>>(b->d_args, b->d_active, b->d_hist, b->d_step, n + kCntProb);
    ch::scale_batch_kernel<T><<<b->g_scale, 256, 0, st>>>(b->d_ax, b->t_sx, b->d_active, n + kCntSx);
    ch::chain_fwd_batch_kernel<T, true, W><<<b->g_chain, ch::chain_threads<T>(W), sm, st>>>(
        b->d_ax, b->t_fx, b->d_active, n + kCntFx, next + 0);
    ch::chain_bwd_batch_kernel<T, true, W><<<b->g_chain, ch::chain_threads<T>(W), sm, st>>>(
        b->d_ax, b->t_fx, b->d_active, n + kCntFx, next + 1);
    ch::btail_batch_kernel<T><<<b->g_tail, 32 * ch::kBTailLines, 0, st>>>(b->d_ax, b->t_tx, b->d_active, n + kCntTx);
    ch::fill_batch_kernel<T><<<b->g_fill, 256, 0, st>>>(b->d_ax, b->t_lx, b->d_active, n + kCntLx);
    ch::scale_batch_kernel<T><<<b->g_scale, 256, 0, st>>>(b->d_ay, b->t_sy, b->d_active, n + kCntSy);
    ch::chain_fwd_batch_kernel<T, false, W><<<b->g_chain, ch::chain_threads<T>(W), sm, st>>>(
        b->d_ay, b->t_fy, b->d_active, n + kCntFy, next + 2);
    ch::chain_bwd_batch_kernel<T, false, W><<<b->g_chain, ch::chain_threads<T>(W), sm, st>>>(
        b->d_ay, b->t_fy, b->d_active, n + kCntFy, next + 3);
    a3::add_batch_kernel<T><<<b->g_elem, 256, 0, st>>>(b->d_args, b->t_elem, b->d_active, n + kCntElem);
    a3::bc_batch_kernel<<<b->g_col, 128, 0, st>>>(b->d_args, b->t_col, b->d_active, n + kCntCol);
  }
  a3::step_incr_kernel<<<1, 1, 0, st>>>(b->d_step);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda3(e, "batched step launch");
}

template <typename T>
int enqueue_step_w(lns_batch3d* b, int niter) {
  switch (b->W) {
    case 1: return enqueue_step<T, 1>(b, niter);
    case 2: return enqueue_step<T, 2>(b, niter);
    case 4: return enqueue_step<T, 4>(b, niter);
    default: return fail3(LNS_ERR_ARG, "batch: lines per CTA must be 1, 2 or 4");
  }
}

// CTAs of kernel k with `threads` threads and `smem` dynamic bytes that stay
// resident on the device at once (at least one per SM).
template <typename K>
unsigned resident(const lns_batch3d* b, K k, int threads, size_t smem) {
  int nb = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k, threads, smem) != cudaSuccess || nb < 1) nb = 1;
  return (unsigned)(nb * b->sms);
}

// The persistent grids of the batched kernels for the precision T and lines
// per CTA W, and room for the recurrences' entry counters.
template <typename T, int W>
int set_grids(lns_batch3d* b, int niter) {
  namespace a3 = lns::a3;
  namespace ch = lns::chain;
  b->g_elem = resident(b, a3::add_batch_kernel<T>, 256, 0);
  b->g_col = resident(b, a3::bc_batch_kernel, 128, 0);
  b->g_pts = resident(b, a3::grad1_batch_kernel, 128, 0);
  b->g_rhs = b->exec_narrow ? resident(b, a3::rhs_batch_kernel<true>, 128, 0)
                            : resident(b, a3::rhs_batch_kernel<false>, 128, 0);
  b->g_res = resident(b, a3::resid_batch_kernel, 256, 0);
  b->g_scale = resident(b, ch::scale_batch_kernel<T>, 256, 0);
  b->g_chain = resident(b, ch::chain_fwd_batch_kernel<T, true, W>, ch::chain_threads<T>(W), ch::chain_smem_bytes<T>(W));
  b->g_tail = resident(b, ch::btail_batch_kernel<T>, 32 * ch::kBTailLines, 0);
  b->g_fill = resident(b, ch::fill_batch_kernel<T>, 256, 0);
  cudaGetLastError();  // an occupancy query that failed leaves no error behind
  if (4 * niter > b->next_cap) {
    if (b->d_next) cudaFree(b->d_next);
    b->d_next = nullptr;
    cudaError_t e = cudaMalloc(&b->d_next, sizeof(int) * 4 * niter);
    if (e != cudaSuccess) return fail3(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    b->next_cap = 4 * niter;
  }
  return LNS_OK;
}
template <typename T>
int set_grids_w(lns_batch3d* b, int niter) {
  switch (b->W) {
    case 1: return set_grids<T, 1>(b, niter);
    case 2: return set_grids<T, 2>(b, niter);
    case 4: return set_grids<T, 4>(b, niter);
    default: return fail3(LNS_ERR_ARG, "batch: lines per CTA must be 1, 2 or 4");
  }
}

// (Re)captures the step as a graph for the current W, niter and stencil
// width; problems joining or leaving need none (the tables are rewritten).
int capture(lns_batch3d* b, int niter) {
  bool narrow = true;  // every problem's stencils are five-point
  for (int p = 0; p < b->P; ++p) narrow = narrow && lns::a3::narrow_stencils(b->ctx[p]->g);
  if (b->exec && b->exec_W == b->W && b->exec_niter == niter && b->exec_narrow == narrow) return LNS_OK;
  b->exec_narrow = narrow;
  int rg = b->mixed ? set_grids_w<cf>(b, niter) : set_grids_w<cd>(b, niter);
  if (rg) return rg;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda3(e, "cudaStreamBeginCapture");
  int rc = b->mixed ? enqueue_step_w<cf>(b, niter) : enqueue_step_w<cd>(b, niter);
  e = cudaStreamEndCapture(b->st, &graph);
  if (rc) {
    if (graph) cudaGraphDestroy(graph);
    return rc;
  }
  if (e != cudaSuccess) return cuda3(e, "cudaStreamEndCapture");
  e = cudaGraphInstantiate(&b->exec, graph, 0);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) return cuda3(e, "cudaGraphInstantiate");
  ++b->captures;
  b->exec_W = b->W;
  b->exec_niter = niter;
  return LNS_OK;
}

// Forms and factors the LHS of every problem not yet factored, and writes
// the per-problem argument tables.
int prepare(lns_batch3d* b, double tol) {
  std::vector<lns::a3::StepArgs> args(b->P);
  std::vector<lns::chain::Args> ax(b->P), ay(b->P);
  for (int p = 0; p < b->P; ++p) {
    lns_ctx3d* c = b->ctx[p];
    if (!b->uploaded[p]) return fail3(LNS_ERR_ARG, "batch: problem " + std::to_string(p) + " not uploaded");
    if (!c->factored) {
      int rc = b->mixed ? factor_all<cf>(c, b->st) : factor_all<cd>(c, b->st);
      if (rc) return rc;
    }
    lns::a3::StepArgs& a = args[p];
    a.g = c->g;
    a.o = c->ops;
    a.v = c->v;
    a.vold = c->vold;
    a.c1v = c->c1v;
    a.r64 = c->r64;
    a.r32 = c->r32;
    a.part = c->part;
    a.nbx = (c->g.nx + 127) / 128;
    a.nrhs = a.nbx * c->g.ny;
    a.tol = tol;
    void* r = b->mixed ? (void*)c->r32 : (void*)c->r64;
    ax[p] = xargs(c, r);
    ay[p] = yargs(c, r);
  }
  cudaError_t e = cudaMemcpy(b->d_args, args.data(), sizeof(args[0]) * b->P, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_ax, ax.data(), sizeof(ax[0]) * b->P, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(b->d_ay, ay.data(), sizeof(ay[0]) * b->P, cudaMemcpyHostToDevice);
  return e == cudaSuccess ? LNS_OK : cuda3(e, "upload batch arguments");
}

// Per-problem device arrays for at least n problems.
int reserve_problems(lns_batch3d* b, int n) {
  if (n <= b->cap) return LNS_OK;
  void* q = nullptr;
  int rc = balloc(b, sizeof(lns::a3::StepArgs) * n, &q);
  if (!rc) b->d_args = (lns::a3::StepArgs*)q, rc = balloc(b, sizeof(lns::chain::Args) * n, &q);
  if (!rc) b->d_ax = (lns::chain::Args*)q, rc = balloc(b, sizeof(lns::chain::Args) * n, &q);
  if (!rc) b->d_ay = (lns::chain::Args*)q, rc = balloc(b, sizeof(int) * n, &q);
  if (!rc) b->d_active = (int*)q, b->cap = n;
  if (b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  return rc;
}

int set_active(lns_batch3d* b) {
  cudaError_t e = cudaMemcpyAsync(b->d_active, b->active.data(), sizeof(int) * b->P, cudaMemcpyHostToDevice, b->st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
  return e == cudaSuccess ? LNS_OK : cuda3(e, "upload active flags");
}

// Residual history for `steps` steps of `probs` problems (default: the
// current ones): the step kernels write hist[step * P + p], so the capacity
// is counted in entries and grows with the number of problems as well as
// with the steps.
int reserve_hist(lns_batch3d* b, long long steps, int probs = -1) {
  const long long need = steps * (long long)(probs < 0 ? b->P : probs);
  if (need <= b->hist_cap) return LNS_OK;
  void* q = nullptr;
  cudaError_t e = cudaStreamSynchronize(b->st);  // no step in flight writes the old buffer
  if (e != cudaSuccess) return cuda3(e, "history: synchronize");
  e = cudaMalloc(&q, sizeof(double) * (size_t)need);
  if (e != cudaSuccess) return fail3(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  if (b->d_hist) {
    cudaFree(b->d_hist);
    b->bytes -= sizeof(double) * (size_t)b->hist_cap;
  }
  b->d_hist = (double*)q;
  b->hist_cap = need;
  b->bytes += sizeof(double) * (size_t)need;
  if (b->exec) {  // the graph holds the old history pointer
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  return LNS_OK;
}

void destroy_batch(lns_batch3d* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->d_hist) cudaFree(b->d_hist);
  if (b->d_next) cudaFree(b->d_next);
  for (void* p : b->allocs) cudaFree(p);
  for (void* p : b->table_allocs) cudaFree(p);
  if (b->owns_ctx)
    for (lns_ctx3d* c : b->ctx) lns_ctx3d_destroy(c);
  if (b->st) cudaStreamDestroy(b->st);
  delete b;
}

}  // namespace

extern "C" {

int lns_batch3d_create(int32_t nprob, const lns_params3d* params, lns_batch3d** out) {
  if (!params || !out || nprob < 1) return fail3(LNS_ERR_ARG, "batch3d_create: need nprob >= 1 and parameters");
  *out = nullptr;
  for (int p = 1; p < nprob; ++p)
    if (params[p].precision != params[0].precision)
      return fail3(LNS_ERR_ARG, "batch3d_create: every problem must use the same precision");
  for (int p = 0; p < nprob; ++p)
    if (params[p].impl > 1) return fail3(LNS_ERR_ARG, "batch3d_create: batches run impl = 1 (backward Euler)");
  for (int p = 0; p < nprob; ++p)
    if (params[p].yper != 0 || params[p].navier != 1 || params[p].xper != 1)
      return fail3(LNS_ERR_ARG, "batch3d_create: batches run a periodic xi direction and a viscous wall-bounded eta "
                                "direction (xper = 1, yper = 0)");
  for (int p = 0; p < nprob; ++p)
    if (params[p].ispg != 0 || params[p].eps_e != 0.0 || params[p].top != 0 || params[p].wall == 3)
      return fail3(LNS_ERR_ARG, "batch3d_create: batches run without a sponge, smoother or forced top (ispg = 0, "
                                "eps_e = 0, top = 0)");
  lns_batch3d* b = new lns_batch3d();
  b->P = nprob;
  b->mixed = params[0].precision == LNS_MIXED;
  cudaError_t e = cudaGetDevice(&b->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
  if (e != cudaSuccess) {
    delete b;
    return cuda3(e, "cudaGetDevice");
  }
  int rc = LNS_OK;
  for (int p = 0; p < nprob && !rc; ++p) {
    lns_ctx3d* c = nullptr;
    rc = lns_ctx3d_create(&params[p], &c);
    if (!rc) {
      c->pair_ok = false;  // one launch per phase serves all problems row by row
      b->ctx.push_back(c);
      b->bytes += lns_ctx3d_bytes(c);
    }
  }
  void* q = nullptr;
  if (!rc) {
    e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = cuda3(e, "cudaStreamCreate");
  }
  if (!rc) rc = reserve_problems(b, nprob);
  if (!rc) rc = balloc(b, sizeof(int), &q), b->d_step = (int*)q;
  if (!rc) rc = reserve_hist(b, 64);
  if (!rc) rc = build_tables(b);
  if (rc) {
    destroy_batch(b);
    return rc;
  }
  b->active.assign(nprob, 1);
  b->uploaded.assign(nprob, false);
  *out = b;
  return LNS_OK;
}

int lns_batch3d_destroy(lns_batch3d* b) {
  if (b) destroy_batch(b);
  return LNS_OK;
}

size_t lns_batch3d_bytes(const lns_batch3d* b) { return b ? b->bytes : 0; }

int lns_batch3d_upload(lns_batch3d* b, int32_t prob, const double* metrics, const double* vm, const double* v) {
  if (!b || !metrics || !vm || !v) return fail3(LNS_ERR_ARG, "batch3d_upload: null argument");
  if (prob < 0 || prob >= b->P) return fail3(LNS_ERR_ARG, "batch3d_upload: problem index out of range");
  lns_ctx3d* c = b->ctx[prob];
  int rc = lns_upload_metrics3d(c, metrics);
  if (!rc) rc = lns_upload_mean3d(c, vm, nullptr);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->v, v, sizeof(cd) * 5 * c->np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload v");
  b->uploaded[prob] = true;
  return LNS_OK;
}

int lns_batch3d_get_state(lns_batch3d* b, int32_t prob, double* v) {
  if (!b || !v) return fail3(LNS_ERR_ARG, "batch3d_get_state: null argument");
  if (prob < 0 || prob >= b->P) return fail3(LNS_ERR_ARG, "batch3d_get_state: problem index out of range");
  lns_ctx3d* c = b->ctx[prob];
  cudaError_t e = cudaStreamSynchronize(b->st);
  if (e == cudaSuccess) e = cudaMemcpy(v, c->v, sizeof(cd) * 5 * c->np, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? LNS_OK : cuda3(e, "download v");
}

int lns_batch3d_run(lns_batch3d* b, int32_t max_steps, int32_t niter, double tol, int32_t check_every,
                    int32_t* steps, double* final_res) {
  if (!b || !steps || !final_res) return fail3(LNS_ERR_ARG, "batch3d_run: null argument");
  if (max_steps < 0 || niter < 1 || check_every < 1) return fail3(LNS_ERR_ARG, "batch3d_run: bad step counts");
  int rc = check_device(b->ctx[0]);
  if (!rc) rc = prepare(b, tol);
  if (!rc) rc = reserve_hist(b, max_steps);
  if (!rc) rc = capture(b, niter);
  if (rc) return rc;
  if ((long long)max_steps * b->P > b->hist_cap) return fail3(LNS_ERR_ARG, "batch3d_run: residual history too small");
  for (int p = 0; p < b->P; ++p) {
    b->active[p] = 1;
    steps[p] = -1;
    final_res[p] = -1.0;
  }
  rc = set_active(b);
  if (rc) return rc;
  cudaError_t e = cudaMemsetAsync(b->d_step, 0, sizeof(int), b->st);
  if (e != cudaSuccess) return cuda3(e, "cudaMemsetAsync");
  std::vector<double> hist;
  std::vector<int> act(b->P);
  int done = 0;
  while (done < max_steps) {
    const int n = std::min(check_every, max_steps - done);
    for (int s = 0; s < n; ++s) {
      e = cudaGraphLaunch(b->exec, b->st);
      if (e != cudaSuccess) return cuda3(e, "cudaGraphLaunch");
    }
    hist.resize((size_t)n * b->P);
    e = cudaMemcpyAsync(hist.data(), b->d_hist + (size_t)done * b->P, sizeof(double) * hist.size(),
                        cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(act.data(), b->d_active, sizeof(int) * b->P, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cuda3(e, "batched steps");
    int left = 0;
    for (int p = 0; p < b->P; ++p) {
      if (!b->active[p]) continue;
      for (int s = 0; s < n; ++s) {
        const double r = hist[(size_t)s * b->P + p];
        final_res[p] = r;
        if (!act[p] && r <= tol) {  // the device stopped the problem at this step
          steps[p] = done + s + 1;
          break;
        }
      }
      b->active[p] = act[p];
      left += act[p];
    }
    done += n;
    if (!left) break;
  }
  return LNS_OK;
}

int lns_batch3d_tune(lns_batch3d* b, int32_t niter, int32_t* lines_per_cta) {
  if (!b || !lines_per_cta || niter < 1) return fail3(LNS_ERR_ARG, "batch3d_tune: bad argument");
  int rc = check_device(b->ctx[0]);
  if (!rc) rc = prepare(b, 0.0);
  if (rc) return rc;
  // keep the states: tuning steps run on copies that are restored after
  std::vector<void*> save(b->P, nullptr);
  for (int p = 0; p < b->P && !rc; ++p) {
    cudaError_t e = cudaMalloc(&save[p], sizeof(cd) * 5 * b->ctx[p]->np + 3 * sizeof(double));
    if (e == cudaSuccess)
      e = cudaMemcpy(save[p], b->ctx[p]->v, sizeof(cd) * 5 * b->ctx[p]->np, cudaMemcpyDeviceToDevice);
    if (e == cudaSuccess)
      e = cudaMemcpy((char*)save[p] + sizeof(cd) * 5 * b->ctx[p]->np, b->ctx[p]->dscal, 3 * sizeof(double),
                     cudaMemcpyDeviceToDevice);
    if (e != cudaSuccess) rc = cuda3(e, "tune: save states");
  }
  int best = b->W;
  float best_ms = 1e30f;
  const int cands[3] = {1, 2, 4};
  if (!rc) rc = reserve_hist(b, 16);
  for (int k = 0; k < 3 && !rc; ++k) {
    b->W = cands[k];
    rc = build_tables(b);
    if (!rc) rc = capture(b, niter);
    if (rc) break;
    b->active.assign(b->P, 1);
    rc = set_active(b);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int rep = 0; rep < 2 && !rc; ++rep) {  // warm-up, then timed
      cudaMemsetAsync(b->d_step, 0, sizeof(int), b->st);
      cudaEventRecord(e0, b->st);
      for (int s = 0; s < 4; ++s) cudaGraphLaunch(b->exec, b->st);
      cudaEventRecord(e1, b->st);
      cudaError_t e = cudaEventSynchronize(e1);
      if (e != cudaSuccess) rc = cuda3(e, "tune: timed steps");
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!rc && ms < best_ms) best_ms = ms, best = cands[k];
  }
  for (int p = 0; p < b->P; ++p) {
    if (!save[p]) continue;
    if (!rc) {
      cudaError_t e = cudaMemcpy(b->ctx[p]->v, save[p], sizeof(cd) * 5 * b->ctx[p]->np, cudaMemcpyDeviceToDevice);
      if (e == cudaSuccess)
        e = cudaMemcpy(b->ctx[p]->dscal, (char*)save[p] + sizeof(cd) * 5 * b->ctx[p]->np, 3 * sizeof(double),
                       cudaMemcpyDeviceToDevice);
      if (e != cudaSuccess) rc = cuda3(e, "tune: restore states");
    }
    cudaFree(save[p]);
  }
  if (rc) return rc;
  b->W = best;
  rc = build_tables(b);
  if (!rc && b->exec) {
    cudaGraphExecDestroy(b->exec);
    b->exec = nullptr;
  }
  *lines_per_cta = best;
  return rc;
}

}  // extern "C"

// ======================================================================
// Serving (lns_server3d_*): requests admitted by device-memory footprint
// into a running batch that is re-formed whenever requests join or leave
// ======================================================================
namespace {

struct SrvReq {
  int64_t id = 0;
  lns_params3d prm{};
  std::vector<double> metrics, vm, v;  // host inputs until admission; v holds the result at completion
  double tol = 0.0;
  int max_steps = 0;
  lns_ctx3d* ctx = nullptr;
  int state = 0;  // LNS_REQ_*
  int steps = 0, conv = -1;
  double res = -1.0;
  double t_submit = 0.0, t_admit = 0.0, t_done = 0.0;
};

double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// device bytes lns_ctx3d_create allocates for these parameters
size_t ctx_bytes_for(const lns_params3d& p) {
  const size_t np = (size_t)p.nx * p.ny;
  const bool mixed = p.precision == LNS_MIXED;
  const size_t el = mixed ? sizeof(cf) : sizeof(cd);
  size_t b = sizeof(double) * (10 + 5 + 125) * np + sizeof(cd) * 15 * np;
  b += mixed ? sizeof(cf) * 5 * np : sizeof(cd) * 5 * np;
  b += sizeof(cd) * (250 + 100) * np + el * 250 * np;
  if (mixed) b += el * 100 * np;
  b += sizeof(double) * (((size_t)p.nx + 127) / 128 * p.ny + np / 256 + 2) + 1024;
  return b;
}

}  // namespace

struct lns_server3d {
  lns_batch3d* b = nullptr;
  size_t budget = 0, used = 0;
  int max_slots = 0, niter = 1;
  int precision = LNS_MIXED;
  std::deque<SrvReq*> queue;
  std::vector<SrvReq*> running;
  std::map<int64_t, SrvReq*> all;
  int64_t next_id = 1;
  bool dirty = true;
};

namespace {

// Forms the batch of the running requests: per-problem arguments (factoring
// new ones), work tables and the captured step.
int reform(lns_server3d* s) {
  lns_batch3d* b = s->b;
  b->ctx.clear();
  for (SrvReq* r : s->running) b->ctx.push_back(r->ctx);
  b->P = (int)b->ctx.size();
  b->uploaded.assign(b->P, true);
  b->active.assign(b->P, 1);
  if (!b->P) return LNS_OK;
  int rc = reserve_problems(b, b->P);
  if (!rc) rc = prepare(b, 0.0);
  if (rc) return rc;
  // per-request tolerances
  std::vector<lns::a3::StepArgs> args(b->P);
  cudaError_t e = cudaMemcpy(args.data(), b->d_args, sizeof(args[0]) * b->P, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda3(e, "read batch arguments");
  for (int p = 0; p < b->P; ++p) args[p].tol = s->running[p]->tol;
  e = cudaMemcpy(b->d_args, args.data(), sizeof(args[0]) * b->P, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda3(e, "upload batch arguments");
  rc = build_tables(b);  // keeps the captured step unless a table buffer grew
  if (!rc) rc = set_active(b);
  s->dirty = false;
  return rc;
}

int admit(lns_server3d* s) {
  while (!s->queue.empty() && (int)s->running.size() < s->max_slots) {
    SrvReq* r = s->queue.front();
    const size_t need = ctx_bytes_for(r->prm);
    if (s->used + need > s->budget && !s->running.empty()) break;  // wait for memory
    lns_ctx3d* c = nullptr;
    int rc = lns_ctx3d_create(&r->prm, &c);
    if (!rc) c->pair_ok = false;  // served in a batch
    if (!rc) rc = lns_upload_metrics3d(c, r->metrics.data());
    if (!rc) rc = lns_upload_mean3d(c, r->vm.data(), nullptr);
    if (!rc) {
      cudaError_t e = cudaMemcpy(c->v, r->v.data(), sizeof(cd) * 5 * c->np, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) rc = cuda3(e, "upload v");
    }
    s->queue.pop_front();
    if (rc) {
      if (c) lns_ctx3d_destroy(c);
      r->state = LNS_REQ_FAILED;
      r->t_done = now_s();
      // a failed request returns nothing: drop its host copies now
      std::vector<double>().swap(r->metrics);
      std::vector<double>().swap(r->vm);
      std::vector<double>().swap(r->v);
      continue;
    }
    r->ctx = c;
    r->state = LNS_REQ_RUNNING;
    r->t_admit = now_s();
    r->metrics.clear();
    r->metrics.shrink_to_fit();
    r->vm.clear();
    r->vm.shrink_to_fit();
    s->used += lns_ctx3d_bytes(c);
    s->running.push_back(r);
    s->dirty = true;
  }
  return LNS_OK;
}

void retire(lns_server3d* s, SrvReq* r, int state) {
  // a result that cannot be read back is a failed request, not the input state
  if (cudaMemcpy(r->v.data(), r->ctx->v, sizeof(cd) * 5 * r->ctx->np, cudaMemcpyDeviceToHost) != cudaSuccess)
    state = LNS_REQ_FAILED;
  s->used -= lns_ctx3d_bytes(r->ctx);
  lns_ctx3d_destroy(r->ctx);
  r->ctx = nullptr;
  r->state = state;
  r->t_done = now_s();
  s->dirty = true;
}

}  // namespace

extern "C" {

int lns_server3d_create(size_t budget_bytes, int32_t max_slots, int32_t precision, int32_t niter,
                        lns_server3d** out) {
  if (!out || max_slots < 1 || niter < 1) return fail3(LNS_ERR_ARG, "server3d_create: bad argument");
  if (precision != LNS_FP64 && precision != LNS_MIXED)
    return fail3(LNS_ERR_ARG, "server3d_create: precision must be LNS_FP64 or LNS_MIXED");
  *out = nullptr;
  lns_server3d* s = new lns_server3d();
  s->budget = budget_bytes;
  s->max_slots = max_slots;
  s->precision = precision;
  s->niter = niter;
  lns_batch3d* b = new lns_batch3d();
  b->owns_ctx = false;
  b->mixed = precision == LNS_MIXED;
  int rc = LNS_OK;
  cudaError_t e = cudaGetDevice(&b->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
  if (e != cudaSuccess) rc = cuda3(e, "cudaGetDevice");
  void* q = nullptr;
  if (!rc) {
    e = cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking);
    if (e != cudaSuccess) rc = cuda3(e, "cudaStreamCreate");
  }
  // the per-problem arrays for every slot at once, so that requests joining
  // never move them (and the captured step stays valid)
  if (!rc) rc = reserve_problems(b, max_slots);
  if (!rc) rc = balloc(b, sizeof(int), &q), b->d_step = (int*)q;
  if (rc) {
    destroy_batch(b);
    delete s;
    return rc;
  }
  s->b = b;
  *out = s;
  return LNS_OK;
}

int lns_server3d_destroy(lns_server3d* s) {
  if (!s) return LNS_OK;
  for (auto& kv : s->all) {
    if (kv.second->ctx) lns_ctx3d_destroy(kv.second->ctx);
    delete kv.second;
  }
  destroy_batch(s->b);
  delete s;
  return LNS_OK;
}

int lns_server3d_submit(lns_server3d* s, const lns_params3d* prm, const double* metrics, const double* vm,
                        const double* v, double tol, int32_t max_steps, int64_t* id) {
  if (!s || !prm || !metrics || !vm || !v || !id) return fail3(LNS_ERR_ARG, "server3d_submit: null argument");
  if (prm->precision != s->precision) return fail3(LNS_ERR_ARG, "server3d_submit: precision differs from the server's");
  if (prm->impl > 1) return fail3(LNS_ERR_ARG, "server3d_submit: servers run impl = 1 (backward Euler)");
  if (prm->yper != 0 || prm->navier != 1 || prm->xper != 1)
    return fail3(LNS_ERR_ARG, "server3d_submit: servers run a periodic xi direction and a viscous wall-bounded eta "
                              "direction (xper = 1, yper = 0)");
  if (prm->ispg != 0 || prm->eps_e != 0.0 || prm->top != 0 || prm->wall == 3)
    return fail3(LNS_ERR_ARG, "server3d_submit: servers run without a sponge, smoother or forced top (ispg = 0, "
                              "eps_e = 0, top = 0)");
  if (!(tol > 0.0) || max_steps < 1) return fail3(LNS_ERR_ARG, "server3d_submit: need tol > 0 and max_steps >= 1");
  if (ctx_bytes_for(*prm) > s->budget) return fail3(LNS_ERR_ARG, "server3d_submit: request larger than the budget");
  SrvReq* r = new SrvReq();
  r->id = s->next_id++;
  r->prm = *prm;
  const size_t np = (size_t)prm->nx * prm->ny;
  r->metrics.assign(metrics, metrics + 10 * np);
  r->vm.assign(vm, vm + 5 * np);
  r->v.assign(v, v + 10 * np);
  r->tol = tol;
  r->max_steps = max_steps;
  r->state = LNS_REQ_QUEUED;
  r->t_submit = now_s();
  s->queue.push_back(r);
  s->all[r->id] = r;
  *id = r->id;
  return LNS_OK;
}

int lns_server3d_tick(lns_server3d* s, int32_t nsteps, int32_t* running, int32_t* queued) {
  if (!s || nsteps < 1) return fail3(LNS_ERR_ARG, "server3d_tick: bad argument");
  int rc = admit(s);
  if (!rc && s->dirty) rc = reform(s);
  if (rc) return rc;
  lns_batch3d* b = s->b;
  if (b->P) {
    // no request runs past its step limit: the tick is cut to the fewest
    // steps any running request has left
    rc = reserve_hist(b, nsteps, s->max_slots);  // sized for every slot: joins keep it
    for (const SrvReq* r : s->running) nsteps = std::min(nsteps, r->max_steps - r->steps);
    if (!rc) rc = capture(b, s->niter);
    if (rc) return rc;
    if ((long long)nsteps * b->P > b->hist_cap) return fail3(LNS_ERR_ARG, "server3d_tick: residual history too small");
    cudaError_t e = cudaMemsetAsync(b->d_step, 0, sizeof(int), b->st);
    for (int k = 0; k < nsteps && e == cudaSuccess; ++k) e = cudaGraphLaunch(b->exec, b->st);
    std::vector<double> hist((size_t)nsteps * b->P);
    std::vector<int> act(b->P);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(hist.data(), b->d_hist, sizeof(double) * hist.size(), cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(act.data(), b->d_active, sizeof(int) * b->P, cudaMemcpyDeviceToHost, b->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(b->st);
    if (e != cudaSuccess) return cuda3(e, "served steps");
    std::vector<SrvReq*> keep;
    for (int p = 0; p < b->P; ++p) {
      SrvReq* r = s->running[p];
      int st = 0;
      for (int k = 0; k < nsteps; ++k) {
        r->steps += 1;
        r->res = hist[(size_t)k * b->P + p];
        if (!act[p] && r->res <= r->tol) {
          r->conv = r->steps;
          st = LNS_REQ_DONE;
          break;
        }
        if (r->steps >= r->max_steps) {
          st = LNS_REQ_STOPPED;
          break;
        }
      }
      if (st) retire(s, r, st);
      else keep.push_back(r);
    }
    s->running.swap(keep);
  }
  if (running) *running = (int32_t)s->running.size();
  if (queued) *queued = (int32_t)s->queue.size();
  return LNS_OK;
}

int lns_server3d_poll(lns_server3d* s, int64_t id, int32_t* state, int32_t* steps, double* res, double* latency_s) {
  if (!s || !state) return fail3(LNS_ERR_ARG, "server3d_poll: null argument");
  auto it = s->all.find(id);
  if (it == s->all.end()) return fail3(LNS_ERR_ARG, "server3d_poll: unknown request");
  const SrvReq* r = it->second;
  *state = r->state;
  if (steps) *steps = r->conv >= 0 ? r->conv : r->steps;
  if (res) *res = r->res;
  if (latency_s) *latency_s = r->t_done > 0.0 ? r->t_done - r->t_submit : -1.0;
  return LNS_OK;
}

int lns_server3d_fetch(lns_server3d* s, int64_t id, double* v) {
  if (!s || !v) return fail3(LNS_ERR_ARG, "server3d_fetch: null argument");
  auto it = s->all.find(id);
  if (it == s->all.end()) return fail3(LNS_ERR_ARG, "server3d_fetch: unknown request");
  SrvReq* r = it->second;
  if (r->state == LNS_REQ_FAILED) {  // nothing to return; forget it and its host copies
    s->all.erase(it);
    delete r;
    return fail3(LNS_ERR_ARG, "server3d_fetch: the request failed");
  }
  if (r->state != LNS_REQ_DONE && r->state != LNS_REQ_STOPPED)
    return fail3(LNS_ERR_ARG, "server3d_fetch: request not finished");
  std::copy(r->v.begin(), r->v.end(), v);
  s->all.erase(it);
  delete r;
  return LNS_OK;
}

size_t lns_server3d_bytes_in_use(const lns_server3d* s) { return s ? s->used : 0; }

int32_t lns_server3d_graph_captures(const lns_server3d* s) { return s && s->b ? s->b->captures : 0; }

}  // extern "C"
