// The nonlinear two-dimensional implicit ADI step on the GPU
// (src/impdrv.f90:171-400 with linear = 0, impl = 1, iLHS = 1) and its C
// ABI (lns_ctx2d_*, include/lns3d_gb300.h).
//
// Per step: set_time_step on the state (cfl_kernel, dtl_kernel), vold = v,
// itrBC (bc2d_kernel); per corrector: the nonlinear RHS with rbe, rhsBC and
// the residual partials and the operators of the LHS (rhs2d_kernel), the xi
// LHS (lhs2d_kernel) and its periodic solve (penta2p), the eta LHS and its
// boundary solve (penta1bc), v += r, itrBC.  Everything is FP64, as the
// reference; the LHS is formed and factored every corrector, as the
// reference does for the nonlinear equations.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

#include "../../include/lns3d_gb300.h"
#include "adi3d.cuh"
#include "launch.cuh"
#include "penta_rows.cuh"

namespace lns {
namespace a2 {

using a3::d1_at;
using a3::d2_at;
using a3::Grid;
using a3::Metrics;
using a3::Ops;
using a3::pix;
using namespace a3;  // stencil constants

// One far-field boundary: the unit outward normals bn(n,2) of its n nodes
// (src/gengrid.f90:133-155) and the potential-flow values pot(5,n), the
// rho u v w T rows of top.pot, left.pot or right.pot (src/potential.f90).
struct Side {
  const double* bn;
  const double* pot;
  int n;
};

// The boundaries of the step besides the wall: the top (j = ny) and, with
// a non-periodic xi direction, the left (i = 1) and right (i = nx) planes.
struct Far {
  Side top, left, right;
  double theta;     // wall recovery-temperature angle (wallt 0)
  int extrap;       // extrapolation of the right plane over the viscous layer: -1 off, 0, 1, 2
  const int* nbl;   // device: rows of the viscous layer (itrBC keeps it current)
};

// ------------------------------------------------------- Riemann far field
// src/reimann.f90:60-72: invariants of boundary node k of a side from the
// node and the two nodes inside it along the normal grid line.
struct RmState {
  double vn, vint[5], R1, R2, rho, p, vt;
  bool inflow;
};

__device__ inline RmState rm_state(const Grid& g, const Side& sd, int k, const double* vb, const double* vb1,
                                   const double* vb2) {
  const double bn1 = sd.bn[k - 1], bn2 = sd.bn[sd.n + k - 1];
  const double* pt = sd.pot + 5 * (k - 1);
  RmState s;
  s.vn = bn1 * vb[1] + bn2 * vb[2];
  for (int k = 0; k < 5; ++k) s.vint[k] = two * vb1[k] - vb2[k];
  const double cb = sqrt(pt[4]) / g.Ma;
  s.R1 = bn1 * pt[1] + bn2 * pt[2] - two * cb / g.gamma1;
  const double c = sqrt(s.vint[4]) / g.Ma;
  s.R2 = bn1 * s.vint[1] + bn2 * s.vint[2] + two * c / g.gamma1;
  s.inflow = s.vn <= 0.0;
  if (s.inflow) {
    s.rho = pt[0];
    s.p = pt[0] * pt[4] / (g.gamma * (g.Ma * g.Ma));
    s.vt = bn2 * pt[1] - bn1 * pt[2];
  } else {
    s.rho = s.vint[0];
    s.p = s.vint[0] * s.vint[4] / (g.gamma * (g.Ma * g.Ma));
    s.vt = bn2 * s.vint[1] - bn1 * s.vint[2];
  }
  return s;
}

// the boundary state the invariants give, src/reimann.f90:104-150
__device__ inline void rm_values(const Grid& g, const Side& sd, int k, const RmState& s, double out[5]) {
  const double bn1 = sd.bn[k - 1], bn2 = sd.bn[sd.n + k - 1];
  const double gamma = g.gamma, gamma1 = g.gamma1;
  const double vn = pt5 * (s.R1 + s.R2);
  const double gq = gamma1 / four, dR = s.R2 - s.R1;
  out[0] = pow(pow(s.rho, gamma) / (gamma * s.p) * (gq * gq) * (dR * dR), 1.0 / gamma1);
  out[1] = (-(bn1 * vn) - bn2 * s.vt) / (-(bn1 * bn1) - bn2 * bn2);
  out[2] = (-(bn2 * vn) + bn1 * s.vt) / (-(bn1 * bn1) - bn2 * bn2);
  out[3] = s.inflow ? sd.pot[5 * (k - 1) + 3] : s.vint[3];
  const double q = g.Ma * gamma1 / four * dR;
  out[4] = q * q;
}

// Coefficient F(a,b) of ReimannLHS (src/reimann.f90:238-401): the boundary
// row holds -I in the diagonal slot 3, 2F in the slot of the next node
// inside and -F in the slot of the one after it (slots 2 and 1 at the top
// and right planes, 4 and 5 at the left plane).
__device__ inline double rm_coef(const Grid& g, const Side& sd, int k, const RmState& s, int a, int b) {
  const double bn1 = sd.bn[k - 1], bn2 = sd.bn[sd.n + k - 1];
  const double gamma = g.gamma, gamma1 = g.gamma1, Ma = g.Ma;
  const double dR = s.R2 - s.R1, gq = gamma1 / four, sq = sqrt(s.vint[4]);
  const double bb = bn1 * bn1 + bn2 * bn2;
  if (s.inflow) {
    if (a == 1) {
      const double f = pow(pow(s.rho, gamma) / (gamma * s.p) * (gq * gq), 1.0 / gamma1) * two / gamma1 *
                       pow(dR, (two - gamma1) / gamma1);
      return b == 2 ? f * bn1 : b == 3 ? f * bn2 : b == 5 ? f / (gamma1 * Ma * sq) : 0.0;
    }
    if (a == 2 || a == 3) {
      const double f = pt5 * (a == 2 ? bn1 : bn2) / bb;
      return b == 2 ? f * bn1 : b == 3 ? f * bn2 : b == 5 ? f / (gamma1 * Ma * sq) : 0.0;
    }
    if (a == 5) {
      const double f = (Ma * gamma1 / four) * (Ma * gamma1 / four) * two * dR;
      return b == 2 ? f * bn1 : b == 3 ? f * bn2 : b == 5 ? f / (gamma1 * Ma * sq) : 0.0;
    }
    return 0.0;
  }
  if (a == 1) {
    const double rg = pow(s.rho, gamma) / (gamma * s.p);
    const double f1 =
        pow(rg, 1.0 / gamma1) * pow(gq, two / gamma1) * (two / gamma1) * pow(dR, (two - gamma1) / gamma1);
    if (b == 2) return f1 * bn1 + gamma1 * pow(s.rho, gamma1) / s.p;
    if (b == 3) return f1 * bn2;
    if (b == 5) {
      const double f2 = pow(gq * dR, two / gamma1) * 1.0 / (gamma * gamma1) * pow(rg, (two - gamma) / gamma1);
      return f1 / (gamma1 * Ma * sq) - f2 * pow(s.rho, gamma + 1) / (gamma * (Ma * Ma) * (s.p * s.p));
    }
    return 0.0;
  }
  if (a == 2 || a == 3) {
    const double f1 = pt5 * (a == 2 ? bn1 : bn2) / bb, f2 = (a == 2 ? bn2 : bn1) / bb;
    if (b == 2) return a == 2 ? f1 * bn1 + f2 * bn2 : f1 * bn1 - f2 * bn2;
    if (b == 3) return a == 2 ? f1 * bn2 - f2 * bn1 : f1 * bn2 + f2 * bn1;
    if (b == 5) return f1 / (gamma1 * Ma * sq);
    return 0.0;
  }
  if (a == 4) return b == 4 ? 1.0 : 0.0;  // outflow: 2 in slot 2, -1 in slot 1
  const double f = (Ma * gamma1 / four) * (Ma * gamma1 / four) * two * dR;
  return b == 2 ? f * bn1 : b == 3 ? f * bn2 : b == 5 ? f / (gamma1 * Ma * sq) : 0.0;
}

__device__ __forceinline__ double tw_wall(const Grid& g, double theta) {
  const double tt = tan(theta);
  return 1.0 + pt5 * g.gamma1 * (g.Ma * g.Ma) * (1.0 + tt * tt) * sqrt(g.Pr);
}

// -------------------------------------------------------------------- RHS
// The nonlinear RHS and the operators (src/genmtrx.f90 with linear = 0,
// general = true, mattyp = 0, kzl = 0), rbe (src/impdrv.f90:482-505), the
// boundary rows (src/rhsbc.f90:256-370) and the block sums of resstat
// (src/resstat.f90:37-50).  One thread per point; r may be null (operators
// only, when vold is null too).  genmtrx acts on the state vs (v itself, or
// pt5 (v + vold) for the midpoint rule, src/impdrv.f90:271-279); rbe and the
// boundary rows use v; a non-null v2old selects rtb (src/impdrv.f90:511-539)
// in place of rbe.
__global__ void __launch_bounds__(128) rhs2d_kernel(Grid g, Ops o, Metrics mt, Far fr, const double* __restrict__ vs,
                                                    const double* __restrict__ v, const double* __restrict__ vold,
                                                    const double* __restrict__ v2old, double* __restrict__ r,
                                                    double* part) {
  __shared__ double red[128];
  const int i = blockIdx.x * blockDim.x + threadIdx.x + 1;
  const int j = blockIdx.y + 1;
  double resnod = 0.0;
  if (i <= g.nx) {
    const long long p = pix(g, i, j), np = o.np;
    auto V = [&](int k, int ii, int jj) { return vs[k + 5 * pix(g, ii, jj)]; };
    auto VF = [&](int k, int ii, int jj) { return v[k + 5 * pix(g, ii, jj)]; };
    double g1v[5], g2v[5], g11v[5], g12v[5], g22v[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
      const int sym = xsym(g);
      const double sg = k == 2 ? -1.0 : 1.0;  // v changes sign across a symmetry plane
      g1v[k] = d1_at(i, g.nx, g.xper, g.gx, g.dxinv, [&](int ii) { return V(k, ii, j); }, sym, sg);
      g2v[k] = d1_at(j, g.ny, g.yper, g.gy, g.dyinv, [&](int jj) { return V(k, i, jj); });
      g11v[k] = d2_at(i, g.nx, g.xper, g.dx2, g.dxsinv, [&](int ii) { return V(k, ii, j); }, sym, sg);
      g22v[k] = d2_at(j, g.ny, g.yper, g.dy2, g.dysinv, [&](int jj) { return V(k, i, jj); });
      g12v[k] = d1_at(j, g.ny, g.yper, g.gy, g.dyinv, [&](int jj) {
        return d1_at(i, g.nx, g.xper, g.gx, g.dxinv, [&](int ii) { return V(k, ii, jj); }, sym, sg);
      });
    }
    if (g.navier && (g.wallt == 1 || g.wallt == 2) && j == 1) g2v[4] = 0.0;  // src/gradbc.f90:15
    const double m1 = mt.m1[p], m2 = mt.m2[p], n1 = mt.n1[p], n2 = mt.n2[p];
    const double m11 = mt.m11[p], m12 = mt.m12[p], m22 = mt.m22[p], n11 = mt.n11[p], n12 = mt.n12[p],
                 n22 = mt.n22[p];
    const double m1m1 = m1 * m1, m1m2 = m1 * m2, m2m2 = m2 * m2, n1n1 = n1 * n1, n1n2 = n1 * n2, n2n2 = n2 * n2;
    const double m1n1 = m1 * n1, m1n2 = m1 * n2, m2n1 = m2 * n1, m2n2 = m2 * n2;
    double g1vl[5], g2vl[5], g11vl[5], g12vl[5], g22vl[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {  // src/genmtrx.f90:116-136
      g11vl[k] = g11v[k] * m1m1 + two * g12v[k] * m1n1 + g22v[k] * n1n1 + g1v[k] * m11 + g2v[k] * n11;
      g12vl[k] = g11v[k] * m1m2 + g12v[k] * (m1n2 + m2n1) + g22v[k] * n1n2 + g1v[k] * m12 + g2v[k] * n12;
      g22vl[k] = g11v[k] * m2m2 + two * g12v[k] * m2n2 + g22v[k] * n2n2 + g1v[k] * m22 + g2v[k] * n22;
      g1vl[k] = g1v[k] * m1 + g2v[k] * n1;
      g2vl[k] = g1v[k] * m2 + g2v[k] * n2;
    }
    const double gamma = g.gamma, gamma1 = g.gamma1, Ma2 = g.Ma * g.Ma, Re = g.Re, Pr = g.Pr;
    const double fact = 1.0 / (gamma * Ma2);
    double fact1 = 1.0 / Re, fact2 = gamma / (Pr * Re);
    const double fact3 = gamma * gamma1 * Ma2 / Re;
    const double rho = V(0, i, j), u1 = V(1, i, j), u2 = V(2, i, j), t = V(4, i, j);
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
    const double gp[3] = {fact * (grho[0] * t + rho * gt[0]), fact * (grho[1] * t + rho * gt[1]),
                          fact * (grho[2] * t + rho * gt[2])};
    const double S[3][3] = {{gu[0][0], pt5 * (gu[0][1] + gu[1][0]), pt5 * gu[2][0]},
                            {pt5 * (gu[1][0] + gu[0][1]), gu[1][1], pt5 * gu[2][1]},
                            {pt5 * gu[2][0], pt5 * gu[2][1], 0.0}};
    const double mu = 1.0, dmu = 0.0, d2mu = 0.0, con = mu, dcon = dmu, d2con = d2mu;
    const double lm = -pt66 * mu, dlm = -pt66 * dmu, d2lm = -pt66 * d2mu;
    const double g1mu = dmu * gt[0], g2mu = dmu * gt[1], g3mu = dmu * gt[2];
    const double g1dmu = d2mu * gt[0], g2dmu = d2mu * gt[1], g3dmu = d2mu * gt[2];
    const double g1con = dcon * gt[0], g2con = dcon * gt[1], g3con = dcon * gt[2];
    const double g1dcon = d2con * gt[0], g2dcon = d2con * gt[1], g3dcon = d2con * gt[2];
    const double g1lm = dlm * gt[0], g2lm = dlm * gt[1], g3lm = dlm * gt[2];
    const double g1dlm = d2lm * gt[0], g2dlm = d2lm * gt[1], g3dlm = d2lm * gt[2];
    double rr[5];
    // nonlinear RHS, src/genmtrx.f90:282-312
    rr[0] = rho * divu + grho[0] * u1 + grho[1] * u2;
    rr[1] = u1 * gu[0][0] + u2 * gu[0][1] + rhoinv * gp[0] -
            fact1 * (g1lm * divu + lm * g1divu + two * (g1mu * S[0][0] + g2mu * S[0][1] + mu * S1jj)) * rhoinv;
    rr[2] = u1 * gu[1][0] + u2 * gu[1][1] + rhoinv * gp[1] -
            fact1 * (g2lm * divu + lm * g2divu + two * (g1mu * S[1][0] + g2mu * S[1][1] + mu * S2jj)) * rhoinv;
    rr[3] = u1 * gu[2][0] + u2 * gu[2][1] - fact1 * (two * (g1mu * S[2][0] + g2mu * S[2][1] + mu * S3jj)) * rhoinv;
    {
      const double s8 = S[0][0] * S[0][0] + S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][0] * S[1][0] +
                        S[1][1] * S[1][1] + S[1][2] * S[1][2] + S[2][0] * S[2][0] + S[2][1] * S[2][1];
      rr[4] = u1 * gt[0] + u2 * gt[1] + gamma1 * t * divu -
              rhoinv * (fact2 * (g1con * gt[0] + g2con * gt[1] + con * Lapt) +
                        fact3 * (lm * (divu * divu) + two * mu * s8));
    }
    double A[5][5] = {}, B[5][5] = {}, D[5][5] = {}, Vij[4];
    const double gmsinv = 1.0 / (gamma * Ma2);
    fact1 = rhoinv / Re;
    // A, src/genmtrx.f90:458-503; B, :525-575
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
    // D, src/genmtrx.f90:702-782 (linear = 0)
    D[0][0] = divu; D[0][1] = grho[0]; D[0][2] = grho[1]; D[0][3] = grho[2];
    D[1][0] = rhoinv * (gmsinv * gt[0] - rhoinv * gp[0] + fact1 * (g1lm * divu + lm * g1divu) +
                        fact1 * two * (g1mu * S[0][0] + g2mu * S[0][1] + g3mu * S[0][2] + mu * S1jj));
    D[1][1] = gu[0][0]; D[1][2] = gu[0][1]; D[1][3] = gu[0][2];
    D[1][4] = rhoinv * gmsinv * grho[0] - fact1 * (g1dlm * divu + dlm * g1divu) -
              fact1 * two * (g1dmu * S[0][0] + g2dmu * S[0][1] + g3dmu * S[0][2] + dmu * S1jj);
    D[2][0] = rhoinv * (gmsinv * gt[1] - rhoinv * gp[1] + fact1 * (g2lm * divu + lm * g2divu) +
                        fact1 * two * (g1mu * S[1][0] + g2mu * S[1][1] + g3mu * S[1][2] + mu * S2jj));
    D[2][1] = gu[1][0]; D[2][2] = gu[1][1]; D[2][3] = gu[1][2];
    D[2][4] = rhoinv * gmsinv * grho[1] - fact1 * (g2dlm * divu + dlm * g2divu) -
              fact1 * two * (g1dmu * S[1][0] + g2dmu * S[1][1] + g3dmu * S[1][2] + dmu * S2jj);
    D[3][0] = rhoinv * (gmsinv * gt[2] - rhoinv * gp[2] + fact1 * (g3lm * divu + lm * g3divu) +
                        fact1 * two * (g1mu * S[2][0] + g2mu * S[2][1] + g3mu * S[2][2] + mu * S3jj));
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
    {
      const double ssq = S[0][0] * S[0][0] + S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][0] * S[1][0] +
                         S[1][1] * S[1][1] + S[1][2] * S[1][2] + S[2][0] * S[2][0] + S[2][1] * S[2][1] +
                         S[2][2] * S[2][2];
      D[4][0] = fact1 * rhoinv * (g1con * gt[0] + g2con * gt[1] + g3con * gt[2] + con * Lapt) +
                fact2 * rhoinv * lm * (divu * divu) + two * fact2 * rhoinv * mu * ssq;
      D[4][1] = gt[0]; D[4][2] = gt[1]; D[4][3] = gt[2];
      D[4][4] = gamma1 * divu;
      D[4][4] = D[4][4] - fact1 * (g1dcon * gt[0] + g2dcon * gt[1] + g3dcon * gt[2] + dcon * Lapt) -
                fact2 * dlm * (divu * divu) - two * fact2 * dmu * ssq;
    }
    // Vij, src/genmtrx.f90:586-600
    fact1 = 1.0 / Re;
    fact2 = gamma / (Pr * Re);
    Vij[0] = fact1 * rhoinv * (lm + two * mu);
    Vij[1] = fact1 * rhoinv * mu;
    Vij[2] = fact2 * rhoinv * con;
    Vij[3] = fact1 * rhoinv * (lm + mu);
    // \hat{A}, \hat{B}, src/genmtrx.f90:602-700
#pragma unroll
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
        for (int b = 0; b < 5; ++b) H[(long long)(a + 5 * b) * np + p] = h[a][b];
    }
    for (int a = 0; a < 5; ++a)
      for (int b = 0; b < 5; ++b) o.Dh[(long long)(a + 5 * b) * np + p] = D[a][b];
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
    if (r) {
      // the sponge towards the free stream (ispg 2, src/genmtrx.f90:436-446)
      // and the explicit smoother at the end of genmtrx (src/smoother.f90,
      // without symmetry planes; no periodic wrap), both on genmtrx's state
      if (o.spg) {
        const double sp = o.spg[p];
        rr[0] = rr[0] + sp * (V(0, i, j) - 1.0);
        for (int m = 1; m <= 3; ++m) rr[m] = rr[m] + sp * (V(m, i, j));
        rr[4] = rr[4] + sp * (V(4, i, j) - 1.0);
      }
      if (o.buff) {
        const double eb = o.eps_e * o.buff[p];
        const double fa[7] = {-1.666666666666667E-01, 2.0, -6.5, 9.333333333333333, -6.5, 2.0,
                              -1.666666666666667E-01};
        for (int pass = 0; pass < 2; ++pass) {
          const int c = pass == 0 ? j : i, n = pass == 0 ? g.ny : g.nx;
          // beside a symmetry plane the xi pass takes the sixth-order stencil
          // at points 1..3 (n-2..n) over the mirrored values (src/smoother.f90:89-250)
          const int sx_ = pass == 1 ? xsym(g) : 0;
          const bool mirror = ((sx_ & 1) && c <= 3) || ((sx_ & 2) && c >= n - 2);
          if (!mirror && (c < 2 || c > n - 1)) continue;
          for (int m = 0; m < 5; ++m) {
            auto S = [&](int dd) { return pass == 0 ? V(m, i, j + dd) : V(m, i + dd, j); };
            double sm;
            if (mirror) {
              const double sgm = m == 2 ? -1.0 : 1.0;
              auto M = [&](int dd) {
                const int kk = c + dd;
                return kk < 1 ? sgm * V(m, 2 - kk, j) : kk > n ? sgm * V(m, 2 * n - kk, j) : V(m, kk, j);
              };
              sm = fa[0] * M(-3) + fa[1] * M(-2) + fa[2] * M(-1) + fa[3] * M(0) + fa[4] * M(1) + fa[5] * M(2) +
                   fa[6] * M(3);
            } else if (c == 2 || c == n - 1) sm = -1.0 * S(-1) + 2.0 * S(0) - 1.0 * S(1);
            else if (c == 3 || c == n - 2) sm = S(-2) - 4.0 * S(-1) + 6.0 * S(0) - 4.0 * S(1) + 1.0 * S(2);
            else
              sm = fa[0] * S(-3) + fa[1] * S(-2) + fa[2] * S(-1) + fa[3] * S(0) + fa[4] * S(1) + fa[5] * S(2) +
                   fa[6] * S(3);
            rr[m] = rr[m] + eb * sm;
          }
        }
      }
      // rbe
      const double dtl = o.dtl[p];
      if (v2old) {
        const double onept33 = 1.3333333333333333333e+0, pt33 = 3.3333333333333333333e-1,
                     pt66 = 6.6666666666666666666e-1;
        for (int m = 0; m < 5; ++m)
          rr[m] = onept33 * vold[m + 5 * p] - pt33 * v2old[m + 5 * p] - VF(m, i, j) - pt66 * dtl * rr[m];
      } else {
        for (int m = 0; m < 5; ++m) rr[m] = vold[m + 5 * p] - VF(m, i, j) - dtl * rr[m];
      }
      // boundary rows, src/rhsbc.f90:258-362
      if (!g.yper) {
        if (g.navier && j == 1) {
          for (int m = 1; m <= 3; ++m) rr[m] = 0.0;
          if (g.wall == 1)
            rr[0] = gc1 * VF(0, i, 1) + gc2 * VF(0, i, 2) + gc3 * VF(0, i, 3) + gc4 * VF(0, i, 4) + gc5 * VF(0, i, 5);
          if (g.wall == 3)
            rr[0] = VF(0, i, 1) - (4.0 * VF(0, i, 2) - 6.0 * VF(0, i, 3) + 4.0 * VF(0, i, 4) - VF(0, i, 5));
          if (g.wallt == 0) rr[4] = VF(4, i, 1) - tw_wall(g, fr.theta);
          if (g.wallt == 1)
            rr[4] = gc1 * VF(4, i, 1) + gc2 * VF(4, i, 2) + gc3 * VF(4, i, 3) + gc4 * VF(4, i, 4) + gc5 * VF(4, i, 5);
        }
        if (j == g.ny) {
          if (g.Ma > 1.0) {
            for (int m = 0; m < 5; ++m) rr[m] = 0.0;
          } else if (g.top == 0) {
            const RmState s = rm_state(g, fr.top, i, v + 5 * pix(g, i, g.ny), v + 5 * pix(g, i, g.ny - 1),
                                       v + 5 * pix(g, i, g.ny - 2));
            double b[5];
            rm_values(g, fr.top, i, s, b);
            for (int m = 0; m < 5; ++m) rr[m] = VF(m, i, j) - b[m];
          }
        }
      } else if (j == g.ny) {
        for (int m = 0; m < 5; ++m) rr[m] = 0.0;
      }
      // the xi boundary rows, src/rhsbc.f90:364-482, after the wall and top
      // rows they overwrite at the corners: the Riemann far field (left 0,
      // right 0) and the symmetry plane (left 2) below Ma 1; then, at any
      // Ma, the extrapolation of the right plane over the viscous layer
      // (rows 1..nbl) and the held right plane (right 8)
      if (!g.xper && (i == 1 || i == g.nx)) {
        const bool left = i == 1;
        if (g.Ma < 1.0 && (left ? g.left : g.right) == 0) {
          const Side& sd = left ? fr.left : fr.right;
          const int i1 = left ? 2 : g.nx - 1, i2 = left ? 3 : g.nx - 2;
          const RmState s = rm_state(g, sd, j, v + 5 * p, v + 5 * pix(g, i1, j), v + 5 * pix(g, i2, j));
          double b[5];
          rm_values(g, sd, j, s, b);
          for (int m = 0; m < 5; ++m) rr[m] = VF(m, i, j) - b[m];
        }
        if (g.Ma < 1.0 && (left ? g.left : g.right) == 7) rr[2] = 0.0;  // symmetry plane: v = 0
        if (g.Ma < 1.0 && left && g.left == 2)
          for (int m = 0; m < 5; ++m)
            rr[m] = m == 2 ? 0.0
                           : gc1 * VF(m, 1, j) + gc2 * VF(m, 2, j) + gc3 * VF(m, 3, j) + gc4 * VF(m, 4, j) +
                                 gc5 * VF(m, 5, j);
        if (!left && fr.extrap >= 0 && j <= *fr.nbl)
          for (int m = 0; m < 5; ++m) {
            const double e = fr.extrap == 0   ? VF(m, g.nx - 1, j)
                             : fr.extrap == 1 ? two * VF(m, g.nx - 1, j) - VF(m, g.nx - 2, j)
                                              : 3.0 * VF(m, g.nx - 1, j) - 3.0 * VF(m, g.nx - 2, j) +
                                                    VF(m, g.nx - 3, j);
            rr[m] = VF(m, g.nx, j) - e;
          }
        if (!left && g.right == 8)
          for (int m = 0; m < 5; ++m) rr[m] = 0.0;
      }
      if (g.xper && i == g.nx)
        for (int m = 0; m < 5; ++m) rr[m] = 0.0;
      for (int m = 0; m < 5; ++m) r[m + 5 * p] = rr[m];
      resnod = (rr[0] * rr[0] + rr[1] * rr[1] + rr[2] * rr[2] + rr[3] * rr[3] + rr[4] * rr[4]) / (dtl * dtl);
    }
  }
  if (!part) return;
  red[threadIdx.x] = resnod;
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s) red[threadIdx.x] += red[threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x + gridDim.x * blockIdx.y] = red[0];
}

// -------------------------------------------------------------------- LHS
// Entry (k, a, b) of the LHS of point (i, j): lhs1f / lhs2f
// (src/lhsf.f90:42-110, 198-247), the eta boundary rows (src/lhsbt2f.f90)
// and the boundary conditions (src/lhsbc1f.f90:232-605,
// src/lhsbc2f.f90:195-291).  One thread per entry.
//
// order2 selects the second-order LHS of the iLHS = 0 path: lhs1 / lhs2
// (src/lhs.f90:7-137, 140-277), lhsbt2 (src/lhsbt2.f90) and the nonlinear
// lhsbc1 / lhsbc2 rows (src/lhsbc1.f90, src/lhsbc2.f90).  Its block-
// tridiagonal rows are written in the same pentadiagonal slots (the outer
// slots of a band row hold zero blocks, the boundary rows' bc(1..14)
// blocks sit in the slots of their columns), so one set of line solvers
// serves both orders: zero blocks add exact zeros to the elimination.
__global__ void lhs2d_kernel(Grid g, Ops o, Far fr, const double* __restrict__ v, int dir, int order2, LhsCoef lc,
                             double* __restrict__ mat) {
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
  const double ident = (k == 3 && a == b) ? 1.0 : 0.0;
  const long long np = o.np;
  const double d = o.dtl[p], alfa = g.alfa;
  // the rows of the xi boundary planes (non-periodic xi), which lhsbc1f
  // and lhsbc2f set last and in full
  const bool symplane = !g.xper && ((i == 1 && g.left == 7) || (i == g.nx && g.right == 7));
  if (symplane) {
    // symmetry plane rows: the symmetric band row below, after the v row of
    // the left plane (src/lhsbc1f.f90:652-655, src/lhsbc2f.f90:525-528) and
    // the right plane's extrapolation rows, which lhsbc1f sets last
    const bool left = i == 1;
    if (left && a == 3 && (dir == 1 || g.Ma < 1.0)) {
      mat[q] = ident;
      return;
    }
    if (!left && dir == 1 && fr.extrap >= 0 && j <= *fr.nbl) {
      const double c = a == b ? 1.0 : 0.0;
      mat[q] = k == 3 ? -c : k == 2 ? (fr.extrap == 0 ? c : two * c) : (k == 1 && fr.extrap == 1 ? -c : 0.0);
      return;
    }
  } else if (!g.xper && (i == 1 || i == g.nx)) {
    const bool left = i == 1;
    if (dir == 2) {
      // identity eta rows: below Ma 1 on the Riemann (left 0, right 0),
      // symmetry (left 2) and held (right 8) planes, else over the viscous
      // layer (src/lhsbc2f.f90:489-556)
      const int bc = left ? g.left : g.right;
      if (g.Ma < 1.0 ? (bc == 0 || (left ? bc == 2 : bc == 8)) : j <= *fr.nbl) {
        mat[q] = ident;
        return;
      }
    } else {
      // src/lhsbc1f.f90:606-898: slot k holds the coefficient of node
      // i + (k - 3) for rows inside the band; the boundary rows put the
      // further nodes of their one-sided stencils in the free slots
      double val = 0.0;
      if (left && g.left == 2) {  // symmetry plane: -(gc1..gc5) on the diagonal of rows 1, 2, 4, 5
        if (a == 3) val = ident;
        else if (a == b) val = -pick5((k + 2) % 5, gc1, gc2, gc3, gc4, gc5);
      } else if (g.Ma < 1.0 && (left ? g.left : g.right) == 0) {
        const Side& sd = left ? fr.left : fr.right;
        const int i1 = left ? 2 : g.nx - 1, i2 = left ? 3 : g.nx - 2;
        const int s1 = left ? 4 : 2, s2 = left ? 5 : 1;
        const RmState s = rm_state(g, sd, j, v + 5 * p, v + 5 * pix(g, i1, j), v + 5 * pix(g, i2, j));
        if (k == 3) val = a == b ? -1.0 : 0.0;
        else if (k == s1) val = two * rm_coef(g, sd, j, s, a, b);
        else if (k == s2) val = -rm_coef(g, sd, j, s, a, b);
        if (a == 4 && s.inflow && k != 3) val = 0.0;
      }
      if (!left && fr.extrap >= 0 && j <= *fr.nbl) {  // extrapolation of the viscous layer
        const double c = a == b ? 1.0 : 0.0;
        val = k == 3 ? -c : k == 2 ? (fr.extrap == 0 ? c : two * c) : (k == 1 && fr.extrap == 1 ? -c : 0.0);
      }
      if (!left && g.right == 8) val = k == 3 ? -(a == b ? 1.0 : 0.0) : 0.0;
      mat[q] = val;
      return;
    }
  }
  // boundary conditions of the wall row j = 1
  if (!g.yper && g.navier && j == 1) {
    if (dir == 1) {
      if (a >= 2 && a <= 4) { mat[q] = ident; return; }
      if (a == 1 && g.wall >= 1 && g.wall <= 3) { mat[q] = ident; return; }
      if (a == 5 && (g.wallt == 0 || g.wallt == 1)) { mat[q] = ident; return; }
    } else {
      const int tk = (k + 2) % 5;  // coefficient of slot k: slots 3,4,5,1,2 <-> 0..4
      const double gct = pick5(tk, gc1, gc2, gc3, gc4, gc5), ext = pick5(tk, -1.0, 4.0, -6.0, 4.0, -1.0);
      if (a >= 2 && a <= 4) { mat[q] = ident; return; }
      // the second-order wall-3 row clears only mat(:,1,:,:,1) (columns 1
      // and 2): the blocks of columns 3..5 keep their closure entries off
      // the first column (src/lhsbc2.f90, wall = 3)
      const bool keep = order2 && g.wall == 3 && b != 1 && (k == 5 || k == 1 || k == 2);
      if (a == 1 && (g.wall == 1 || g.wall == 3) && !keep) {
        mat[q] = b == 1 ? (g.wall == 1 ? -gct : ext) : 0.0;
        return;
      }
      if (a == 5 && g.wallt == 0) { mat[q] = -ident; return; }
      if (a == 5 && g.wallt == 1) { mat[q] = b == 5 ? -gct : 0.0; return; }
    }
  }
  // the far-field row j = ny
  if (!g.yper && j == g.ny) {
    if (dir == 1 && g.top == 0) { mat[q] = ident; return; }
    // the held quiescent top (top 3): identity eta row, src/lhsbc2f.f90:332-339
    if (dir == 2 && g.Ma < 1.0 && g.top == 3) { mat[q] = ident; return; }
    if (dir == 2 && g.Ma < 1.0 && g.top == 0) {
      const RmState s = rm_state(g, fr.top, i, v + 5 * pix(g, i, g.ny), v + 5 * pix(g, i, g.ny - 1),
                                 v + 5 * pix(g, i, g.ny - 2));
      double val = 0.0;
      if (k == 3) val = a == b ? -1.0 : 0.0;
      else if (k == 2) val = two * rm_coef(g, fr.top, i, s, a, b);
      else if (k == 1) val = -rm_coef(g, fr.top, i, s, a, b);
      if (a == 4 && s.inflow && k != 3) val = 0.0;
      mat[q] = val;
      return;
    }
  }
  const long long eab = (long long)((a - 1) + 5 * (b - 1)) * np + p;
  const double* V = dir == 1 ? o.V11 : o.V22;
  int vk = -1;
  if (a == 2 && b == 2) vk = 0;
  else if (a == 2 && b == 3) vk = 4;
  else if (a == 3 && b == 2) vk = 5;
  else if (a == 3 && b == 3) vk = 1;
  else if (a == 4 && b == 4) vk = 2;
  else if (a == 5 && b == 5) vk = 3;
  double val;
  const bool edge = dir == 2 ? !g.yper && (j <= 2 || j >= g.ny - 1) : !g.xper && (i <= 2 || i >= g.nx - 1);
  if (order2 && !edge && (dir == 1 || j > 3 && j < g.ny - 2)) {
    // three-point band in slots 2..4 (src/lhs.f90:28-104, 176-240)
    if (k == 1 || k == 5) { mat[q] = 0.0; return; }
    const double ak = lc.ak2[k - 2], bk = lc.bk2[k - 2];
    val = ak * d * (dir == 1 ? o.Ah : o.Bh)[eab];
    if (dir == 1 && k == 3) val = val + alfa * d * o.Dh[eab];
    if (vk >= 0) val = val - bk * d * V[vk * np + p];
  } else if (order2 && !edge) {
    // rows 3 and ny-2: the central five-point stencil of lhsbt2 with a
    // literal zero diagonal block (src/lhsbt2.f90, rows 3 and ny-2)
    const double gik = pick5(k - 1, ga1, ga2, 0.0, ga3, ga4), dik = pick5(k - 1, da1, da2, da3, da4, da5);
    const double detainv = lc.hinv, detasinv = lc.hsinv;  // dir 2: h = deta
    val = k == 3 ? 0.0 : alfa * d * gik * detainv * o.Bh[eab];
    if (vk >= 0) val = val - alfa * d * dik * detasinv * V[vk * np + p];
  } else if (!edge) {
    const double ak = lc.ak[k - 1], bk = lc.bk[k - 1];
    val = ak * d * (dir == 1 ? o.Ah : o.Bh)[eab];
    if (dir == 1 && k == 3) val = val + alfa * d * o.Dh[eab];
    if (vk >= 0) val = val - bk * d * V[vk * np + p];
  } else {
    // rows 1, 2, n-1, n of a line: coefficient t of slot k (eta:
    // src/lhsbt2f.f90; xi: src/lhsbt1f.f90, whose rows also carry the D
    // term in the diagonal slot)
    const double hinv = lc.hinv, hsinv = lc.hsinv;  // h = dxi (dir 1) or deta (dir 2)
    const int c = dir == 1 ? i : j, n = dir == 1 ? g.nx : g.ny;
    auto g1 = [](int t) { return pick5(t, gc1, gc2, gc3, gc4, gc5); };
    auto d1 = [](int t) { return pick5(t, dd1, dd2, dd3, dd4, dd5); };
    auto g2 = [](int t) { return pick5(t, gb1, gb2, gb3, gb4, gb5); };
    auto d2 = [](int t) { return pick5(t, db1, db2, db3, db4, db5); };
    double gcf, dcf;
    bool neg = false;
    const int sym = dir == 1 ? xsym(g) : 0;
    if (((sym & 1) && c <= 2) || ((sym & 2) && c >= n - 1)) {
      // symmetry plane (src/lhsbs1f.f90): the band stencil with the nodes
      // beyond the plane folded onto their mirror images, times -1 in the
      // columns of v (b = 3)
      const double sg = b == 3 ? -1.0 : 1.0;
      gcf = 0.0, dcf = 0.0;
      for (int o5 = 0; o5 < 5; ++o5) {
        int m = c + o5 - 2;
        bool mir = false;
        if (m < 1) m = 2 - m, mir = true;
        if (m > n) m = 2 * n - m, mir = true;
        if (m - c + 3 != k) continue;
        const double gk = pick5(o5, ga1, ga2, 0.0, ga3, ga4), dk = pick5(o5, da1, da2, da3, da4, da5);
        gcf = gcf + (mir ? sg * gk : gk);
        dcf = dcf + (mir ? sg * dk : dk);
      }
    } else if (c == 1) { const int t = (k + 2) % 5; gcf = g1(t); dcf = d1(t); }
    else if (c == 2) { const int t = (k + 3) % 5; gcf = g2(t); dcf = d2(t); }
    else if (c == n - 1) { const int t = k == 5 ? 4 : 4 - k; gcf = g2(t); dcf = d2(t); neg = true; }
    else { const int t = k <= 3 ? 3 - k : 8 - k; gcf = g1(t); dcf = d1(t); neg = true; }
    val = alfa * d * gcf * hinv * (dir == 1 ? o.Ah : o.Bh)[eab];
    if (neg) val = -val;
    if (dir == 1 && k == 3) val = val + alfa * d * o.Dh[eab];
    if (vk >= 0) val = val - alfa * d * dcf * hsinv * V[vk * np + p];
  }
  val = val + ident;
  // implicit damping and sponge of the fourth-order LHS, after the I term:
  // band rows damping then sponge (src/lhsf.f90:113-145, 262-312); the eta
  // boundary rows the sponge through lhsbt2f's transposed spgl(ny,nx) view
  // of the (nx,ny) array, then the damping of rows 2 and ny-1 in slots 2..4
  // (src/lhsbt2f.f90:18, 84-108, 163-213, 266-316)
  // the second-order LHS: band rows damping c_k = alfa eps_i (-1, 2, -1),
  // eps_i = 4 eps_e, then the eta sponge (src/lhs.f90:23-27, 89-103,
  // 229-250); the lhsbt2 rows 1..3 and ny-2..ny the sponge through the
  // transposed spgl view, then the damping of rows 2, ny-1 (-1, 2, -1) and
  // 3, ny-2 (fb1..fb5) (src/lhsbt2.f90)
  if (order2 && a == b && (o.buff || o.spg)) {
    if (dir == 1 || (j > 3 && j < g.ny - 2)) {
      if (o.buff && k >= 2 && k <= 4) {
        const double eps_i = 4.0 * o.eps_e;
        const double ck = k == 3 ? alfa * 2.0 * eps_i : -alfa * eps_i;
        val = val + ck * d * o.buff[p];
      }
      if (dir == 2 && o.spg && k == 3) val = val + alfa * d * o.spg[p];
    } else {
      if (o.spg && k == 3) val = val + alfa * d * o.spg[(long long)(j - 1) + (long long)(i - 1) * g.ny];
      if (o.buff) {
        const double wd = alfa * d * o.eps_e * o.buff[p];
        if ((j == 2 || j == g.ny - 1) && k >= 2 && k <= 4) val = val + wd * (k == 3 ? 2.0 : -1.0);
        if (j == 3 || j == g.ny - 2) val = val + wd * pick5(k - 1, 1.0, -4.0, 6.0, -4.0, 1.0);
      }
    }
  }
  if (!order2 && a == b && (o.buff || o.spg)) {
    const double wd = o.buff ? alfa * d * o.eps_e * o.buff[p] : 0.0;
    if (!edge) {
      if (o.buff) val = val + wd * pick5(k - 1, 1.0, -4.0, 6.0, -4.0, 1.0);
      if (dir == 2 && o.spg && k == 3) val = val + alfa * d * o.spg[p];
    } else {
      const int c = dir == 1 ? i : j, n = dir == 1 ? g.nx : g.ny;
      const int sym = dir == 1 ? xsym(g) : 0;
      if (dir == 2 && o.spg && k == 3) val = val + alfa * d * o.spg[(long long)(j - 1) + (long long)(i - 1) * g.ny];
      if (((sym & 1) && c <= 2) || ((sym & 2) && c >= n - 1)) {
        // the damping stencil folded like the band (src/lhsbs1f.f90)
        if (o.buff) {
          const double sg = a == 3 ? -1.0 : 1.0;
          double fd = 0.0;
          for (int o5 = 0; o5 < 5; ++o5) {
            int m = c + o5 - 2;
            bool mir = false;
            if (m < 1) m = 2 - m, mir = true;
            if (m > n) m = 2 * n - m, mir = true;
            if (m - c + 3 != k) continue;
            const double fk = pick5(o5, 1.0, -4.0, 6.0, -4.0, 1.0);
            fd = fd + (mir ? sg * fk : fk);
          }
          if (fd != 0.0) val = val + wd * fd;
        }
      } else if (o.buff && (c == 2 || c == n - 1) && k >= 2 && k <= 4) {
        val = val + wd * (k == 3 ? 2.0 : -1.0);
      }
    }
  }
  mat[q] = val;
}

// ----------------------------------------------------------------- update
// The boundary values of src/itrbc.f90:629-760 (nonlinear branch): threads
// 0..ncol-1 own a column (wall row from rows 2..5, far-field row from rows
// ny-1, ny-2); with a periodic x direction the remaining threads copy the
// interior rows of column 1 to column nx, and the thread of column 1 copies
// its boundary rows.
__global__ void bc2d_kernel(Grid g, Far fr, double* __restrict__ v) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const int ncol = g.xper ? g.nx - 1 : g.nx;
  if (t < ncol) {
    const int i = t + 1;
    auto W = [&](int k, int jj) -> double& { return v[k + 5 * pix(g, i, jj)]; };
    if (g.yper) {
      for (int m = 0; m < 5; ++m) W(m, g.ny) = W(m, 1);
    } else {
      if (g.navier) {
        for (int m = 1; m <= 3; ++m) W(m, 1) = 0.0;
        if (g.wall == 1) W(0, 1) = -(gc2 * W(0, 2) + gc3 * W(0, 3) + gc4 * W(0, 4) + gc5 * W(0, 5)) / gc1;
        if (g.wall == 3) W(0, 1) = 4.0 * W(0, 2) - 6.0 * W(0, 3) + 4.0 * W(0, 4) - W(0, 5);
        if (g.wallt == 0) W(4, 1) = tw_wall(g, fr.theta);
        if (g.wallt == 1) W(4, 1) = -(gc2 * W(4, 2) + gc3 * W(4, 3) + gc4 * W(4, 4) + gc5 * W(4, 5)) / gc1;
      }
      if (g.Ma > 1.0) {
        W(0, g.ny) = 1.0; W(1, g.ny) = 1.0; W(2, g.ny) = 0.0; W(3, g.ny) = 0.0; W(4, g.ny) = 1.0;
      } else if (g.top == 0) {
        const RmState s = rm_state(g, fr.top, i, &W(0, g.ny), &W(0, g.ny - 1), &W(0, g.ny - 2));
        double b[5];
        rm_values(g, fr.top, i, s, b);
        for (int m = 0; m < 5; ++m) W(m, g.ny) = b[m];
      } else if (g.top == 3) {  // the held quiescent top, src/itrbc.f90 (nonlinear)
        W(0, g.ny) = 1.0; W(1, g.ny) = 0.0; W(2, g.ny) = 0.0; W(3, g.ny) = 0.0; W(4, g.ny) = 1.0;
      }
    }
    if (g.xper && i == 1)
      for (int m = 0; m < 5; ++m) {
        v[m + 5 * pix(g, g.nx, 1)] = W(m, 1);
        v[m + 5 * pix(g, g.nx, g.ny)] = W(m, g.ny);
      }
  } else if (g.xper) {
    const int j = t - ncol + 2;
    if (j <= g.ny - 1)
      for (int m = 0; m < 5; ++m) v[m + 5 * pix(g, g.nx, j)] = v[m + 5 * pix(g, 1, j)];
  }
}

// The xi boundary planes of itrBC (src/itrbc.f90:760-886, nonlinear), after
// bc2d_kernel has set the wall and top rows they read and overwrite at the
// corners.  One CTA in three phases separated by barriers: (1) on every row
// the left plane (Riemann, left 0, from columns 2 and 3; symmetry plane,
// left 2: rho, u, w and T extrapolated by the one-sided gc stencil from
// columns 2..5, v = 0) and the right plane (Riemann, right 0, from columns
// nx-1 and nx-2); (2) with update_nbl, the edge of the viscous layer: nbl =
// the first row whose u at column nx-1 exceeds 0.99 (status bit 2 when no
// row does: the reference stops there with "nbl > ny"); (3) the right plane
// extrapolated from columns nx-1.. over rows 1..nbl.
__global__ void __launch_bounds__(256) bcx2d_kernel(Grid g, Far fr, double* __restrict__ v, int* nbl,
                                                    int update_nbl, int* status) {
  __shared__ int first;
  auto W = [&](int k, int ii, int jj) -> double& { return v[k + 5 * pix(g, ii, jj)]; };
  for (int j = threadIdx.x + 1; j <= g.ny; j += blockDim.x) {
    if (g.left == 0) {
      const RmState s = rm_state(g, fr.left, j, &W(0, 1, j), &W(0, 2, j), &W(0, 3, j));
      double b[5];
      rm_values(g, fr.left, j, s, b);
      for (int m = 0; m < 5; ++m) W(m, 1, j) = b[m];
    } else if (g.left == 2) {
      for (int m = 0; m < 5; ++m)
        W(m, 1, j) = m == 2 ? 0.0 : -(gc2 * W(m, 2, j) + gc3 * W(m, 3, j) + gc4 * W(m, 4, j) + gc5 * W(m, 5, j)) / gc1;
    } else if (g.left == 7) {
      W(2, 1, j) = 0.0;
    }
    if (g.right == 7) W(2, g.nx, j) = 0.0;
    if (g.right == 0) {
      const RmState s = rm_state(g, fr.right, j, &W(0, g.nx, j), &W(0, g.nx - 1, j), &W(0, g.nx - 2, j));
      double b[5];
      rm_values(g, fr.right, j, s, b);
      for (int m = 0; m < 5; ++m) W(m, g.nx, j) = b[m];
    }
  }
  if (threadIdx.x == 0) first = g.ny + 1;
  __syncthreads();
  if (update_nbl) {
    for (int j = threadIdx.x + 1; j <= g.ny; j += blockDim.x)
      if (W(1, g.nx - 1, j) > 0.99) atomicMin(&first, j);
    __syncthreads();
    if (threadIdx.x == 0) {
      if (first > g.ny) atomicOr(status, 2);
      else *nbl = first;
    }
    __syncthreads();
  }
  const int n = *nbl;
  if (fr.extrap >= 0)
    for (int j = threadIdx.x + 1; j <= n; j += blockDim.x)
      for (int m = 0; m < 5; ++m)
        W(m, g.nx, j) = fr.extrap == 0   ? W(m, g.nx - 1, j)
                        : fr.extrap == 1 ? two * W(m, g.nx - 1, j) - W(m, g.nx - 2, j)
                                         : 3.0 * W(m, g.nx - 1, j) - 3.0 * W(m, g.nx - 2, j) + W(m, g.nx - 3, j);
}

// w = pt5 (v + vold), the midpoint state (src/impdrv.f90:273)
__global__ void avg2d_kernel(long long n, const double* __restrict__ v, const double* __restrict__ vold,
                             double* __restrict__ w) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e < n) w[e] = 0.5 * (v[e] + vold[e]);
}

}  // namespace a2
}  // namespace lns

// ======================================================================
// Context and C ABI
// ======================================================================
using lns::a3::Grid;
using lns::a3::Metrics;
using lns::a3::Ops;

struct lns_ctx2d {
  lns_params2d prm;
  Grid g;
  int device = -1;
  long long np = 0;
  size_t bytes = 0;
  std::vector<void*> allocs;
  double* metrics = nullptr;  // (nx,ny,10)
  double* opbuf = nullptr;    // Ah Bh Dh (25 np each), V11 V12 V22 (6 np each), dtl (np)
  Ops ops{};
  double *bnt = nullptr, *pot = nullptr;  // far field of the top boundary
  // far fields of the xi planes (xper = 0 with left 0 / right 0): bn(ny,2), pot(5,ny)
  double *bnl = nullptr, *potl = nullptr, *bnr = nullptr, *potr = nullptr;
  int* nbl = nullptr;                     // device: itrBC's edge of the viscous layer
  double* rowwork = nullptr;              // block-row solves: [U | z] records, 105 per point
  double *v = nullptr, *vold = nullptr, *r = nullptr, *mat = nullptr, *per = nullptr, *per2 = nullptr;
  double *v2old = nullptr, *wavg = nullptr;  // impl 2 / impl 3 state
  long long lstep = 0;                       // steps taken since creation
  double* part = nullptr;
  int nparts = 0;
  double* dscal = nullptr;  // [0] cfl, [1] scratch residual, [2] running residual
  double* res_dev = nullptr;
  int res_cap = 0;
  int* status = nullptr;
  bool have_metrics = false, have_top = false, have_left = false, have_right = false;
  bool have_sponge = false;  // ispg = 2: lns_upload_sponge2d called
  double* spg = nullptr;     // spg + spg2
  double* buff = nullptr;    // eps_e != 0: buff(nx,ny), ones until uploaded
};

namespace {

int fail2(int code, const std::string& msg) { return lns_fail(code, msg); }
int cuda2(cudaError_t e, const char* where) { return lns_cuda_fail(e, where); }

// interior stencil coefficients, src/grad.f90 and src/grad2.f90 (as cgrad)
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

int dalloc2(lns_ctx2d* c, size_t bytes, void** out) {
  cudaError_t e = cudaMalloc(out, bytes);
  if (e != cudaSuccess) {
    *out = nullptr;
    return fail2(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  c->allocs.push_back(*out);
  c->bytes += bytes;
  return LNS_OK;
}

void free2(lns_ctx2d* c) {
  for (void* p : c->allocs) cudaFree(p);
  c->allocs.clear();
}

int check_dev2(const lns_ctx2d* c) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda2(e, "cudaGetDevice");
  if (dev != c->device) return fail2(LNS_ERR_ARG, "context belongs to another device");
  return LNS_OK;
}

Metrics metrics2(const lns_ctx2d* c) {
  const double* m = c->metrics;
  const long long np = c->np;
  return Metrics{m, m + np, m + 2 * np, m + 3 * np, m + 4 * np, m + 5 * np, m + 6 * np, m + 7 * np, m + 8 * np,
                 m + 9 * np};
}

lns::a2::Far top2(const lns_ctx2d* c) {
  lns::a2::Far f;
  f.top = lns::a2::Side{c->bnt, c->pot, c->g.nx};
  f.left = lns::a2::Side{c->bnl, c->potl, c->g.ny};
  f.right = lns::a2::Side{c->bnr, c->potr, c->g.ny};
  f.theta = c->prm.theta;
  f.extrap = c->g.xper ? -1 : c->prm.extrap;
  f.nbl = c->nbl;
  return f;
}

dim3 pgrid(const Grid& g) { return dim3((g.nx + 127) / 128, g.ny); }

// set_time_step on the state v (src/temporal.f90:12-162)
int time_step(lns_ctx2d* c, const double* v, cudaStream_t st) {
  const int nb = (int)((c->np + 255) / 256);
  const Metrics mt = metrics2(c);
  lns::a3::cfl_kernel<<<nb, 256, 0, st>>>(c->g, v, mt, c->ops.dtl, c->part);
  lns::a3::dtl_kernel<<<152, 256, 0, st>>>(c->np, nb, c->part, c->ops.dtl, c->prm.cflmax, c->prm.dtmax,
                                           c->prm.loctime, c->dscal);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda2(e, "time-step kernels launch");
}

int rhs2(lns_ctx2d* c, const double* vs, const double* v, const double* vold, const double* v2old, double* r,
         double* res, cudaStream_t st) {
  const Grid& g = c->g;
  lns::a2::rhs2d_kernel<<<pgrid(g), 128, 0, st>>>(g, c->ops, metrics2(c), top2(c), vs, v, vold, v2old, r, c->part);
  const int nrhs = (int)(pgrid(g).x * pgrid(g).y);
  lns::a3::resid_kernel<<<1, 256, 0, st>>>(nrhs, c->part, c->np, res);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda2(e, "rhs kernels launch");
}

int lhs2(lns_ctx2d* c, const double* v, int dir, double* mat, double alfa, cudaStream_t st) {
  const long long nq = 125 * c->np;
  const int order2 = c->prm.lhs_order == 2 ? 1 : 0;
  Grid g = c->g;
  g.alfa = alfa;
  const lns::a3::LhsCoef lc = lns::a3::lhs_coef(alfa, dir == 1 ? g.dxi : g.deta);
  lns::a2::lhs2d_kernel<<<(unsigned)((nq + 255) / 256), 256, 0, st>>>(g, c->ops, top2(c), v, dir, order2, lc, mat);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda2(e, "lhs2d_kernel launch");
}

// A boundary-closure solve of the step's LHS in c->mat and right-hand side
// in c->r (penta1bc / penta2bc semantics): lines of n rows, block-row
// elimination (penta_rows.cuh)
int rows2(lns_ctx2d* c, int n, int nsys, long long row_stride, long long line_stride, cudaStream_t st) {
  const lns::rows::Args a{c->mat, c->r, c->rowwork, n, nsys, row_stride, line_stride, c->status};
  lns::rows::rows_bc_kernel<<<nsys, lns::rows::kThreads, 0, st>>>(a);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda2(e, "rows_bc_kernel launch");
}

int bc2(lns_ctx2d* c, double* v, cudaStream_t st) {
  const int nt = c->g.nx + c->g.ny;
  lns::a2::bc2d_kernel<<<(nt + 127) / 128, 128, 0, st>>>(c->g, top2(c), v);
  if (!c->g.xper)
    lns::a2::bcx2d_kernel<<<1, 256, 0, st>>>(c->g, top2(c), v, c->nbl, c->prm.update_nbl, c->status);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : cuda2(e, "itrBC kernels launch");
}

// nsteps steps of niter correctors (src/impdrv.f90:171-400) with the time
// scheme of the context (src/impdrv.f90:186-279): impl 1 backward Euler
// with the deck's alfa; impl 2 backward Euler at alfa = 1 for the
// context's first step, then v2old = vold and rtb at alfa = pt66; impl 3
// genmtrx on pt5 (v + vold) with rbe at alfa = pt5
int run2(lns_ctx2d* c, double* v, int nsteps, int niter, double* totres_dev, cudaStream_t st) {
  const Grid& g = c->g;
  const size_t vbytes = sizeof(double) * 5 * (size_t)c->np;
  const long long n5 = 5 * c->np;
  const int impl = c->prm.impl == 0 ? 1 : c->prm.impl;
  cudaError_t e = cudaMemsetAsync(c->status, 0, sizeof(int), st);
  if (e != cudaSuccess) return cuda2(e, "cudaMemsetAsync");
  int rc = LNS_OK;
  for (int s = 0; s < nsteps && !rc; ++s) {
    const bool rtb = impl == 2 && c->lstep > 0;
    const double alfa = impl == 3 ? 0.5 : rtb ? 6.6666666666666666666e-1 : (impl == 2 ? 1.0 : c->prm.alfa);
    rc = time_step(c, v, st);
    if (!rc && rtb) {
      e = cudaMemcpyAsync(c->v2old, c->vold, vbytes, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) rc = cuda2(e, "cudaMemcpyAsync v2old");
    }
    if (!rc) {
      e = cudaMemcpyAsync(c->vold, v, vbytes, cudaMemcpyDeviceToDevice, st);
      if (e != cudaSuccess) rc = cuda2(e, "cudaMemcpyAsync vold");
    }
    if (!rc) rc = bc2(c, v, st);
    for (int it = 0; it < niter && !rc; ++it) {
      double* res = (it == niter - 1 && totres_dev) ? totres_dev + s : c->dscal + 1;
      const double* vs = v;
      if (impl == 3) {
        lns::a2::avg2d_kernel<<<(unsigned)((n5 + 255) / 256), 256, 0, st>>>(n5, v, c->vold, c->wavg);
        e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda2(e, "avg2d_kernel launch");
        vs = c->wavg;
      }
      if (!rc) rc = rhs2(c, vs, v, c->vold, rtb ? c->v2old : nullptr, c->r, res, st);
      if (!rc) rc = lhs2(c, v, 1, c->mat, alfa, st);
      // the fourth-order path solves with penta2p (its periodic fill-slot
      // quirk kept unless the exact mode is on), the second-order path with
      // solve2p, which has no such quirk (src/nsolve2p.f90)
      if (!rc && g.xper) {
        // penta2p (solve2p for the second-order LHS, which has no fill quirk)
        const int quirk = c->prm.lhs_order == 2 ? 0 : (g_periodic_exact.load() ? 0 : 1);
        const lns::rows::PArgs pa{c->mat, c->r, c->rowwork, g.nx - 1, g.ny, 1, g.nx, quirk, c->status};
        lns::rows::rows_p_kernel<<<g.ny, lns::rows::kThreads, 0, st>>>(pa);
        e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda2(e, "rows_p_kernel launch");
      }
      else if (!rc)  // penta2bc along xi (src/impdrv.f90:353-357)
        rc = rows2(c, g.nx, g.ny, 1, g.nx, st);
      if (!rc) rc = lhs2(c, v, 2, c->mat, alfa, st);
      if (!rc) rc = rows2(c, g.ny, g.nx, g.nx, 1, st);
      if (!rc) {
        const long long n = 5 * c->np;
        lns::a3::add_kernel<double, double><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, v, c->r);
        e = cudaGetLastError();
        if (e != cudaSuccess) rc = cuda2(e, "add_kernel launch");
      }
      if (!rc) rc = bc2(c, v, st);
    }
    if (!rc) c->lstep += 1;
  }
  return rc;
}

int check_pivots2(lns_ctx2d* c, cudaStream_t st) {
  int status = 0;
  cudaError_t e = cudaMemcpyAsync(&status, c->status, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda2(e, "2D step");
  if (status & 2)
    return fail2(LNS_ERR_ARG, "itrBC: no row of column nx-1 has u > 0.99, so the viscous layer has no edge "
                              "(the reference stops with nbl > ny)");
  if (status) return fail2(LNS_ERR_PIVOT, "zero or non-finite pivot in an LHS factorisation");
  return LNS_OK;
}

}  // namespace

extern "C" {

int lns_ctx2d_create(const lns_params2d* p, lns_ctx2d** out) {
  if (!p || !out) return fail2(LNS_ERR_ARG, "ctx2d_create: null argument");
  *out = nullptr;
  if (p->nx < 8 || p->ny < 7) return fail2(LNS_ERR_ARG, "ctx2d_create: need nx >= 8 and ny >= 7");
  if ((long long)p->nx * p->ny > (1LL << 31) / 125)
    return fail2(LNS_ERR_ARG, "ctx2d_create: nx*ny too large for 32-bit launch indexing");
  if (!(p->dxi > 0.0) || !(p->deta > 0.0)) return fail2(LNS_ERR_ARG, "ctx2d_create: dxi and deta must be > 0");
  if (p->xper != 0 && p->xper != 1) return fail2(LNS_ERR_ARG, "ctx2d_create: xper must be 0 or 1");
  if (p->xper == 0) {
    // the non-periodic xi direction: the planes of src/rhsbc.f90:364-482,
    // src/lhsbc1f.f90:606-898, src/lhsbc2f.f90:489-556, src/itrbc.f90:760-886
    if (p->left != 0 && p->left != 2 && p->left != 7)
      return fail2(LNS_ERR_ARG,
                   "ctx2d_create: with xper = 0, left must be 0 (Riemann), 2 (extrapolated symmetry plane) or 7 "
                   "(mirrored symmetry plane)");
    if (p->right != 0 && p->right != 7 && p->right != 8)
      return fail2(LNS_ERR_ARG,
                   "ctx2d_create: with xper = 0, right must be 0 (Riemann), 7 (symmetry plane) or 8 (held)");
    if (!(p->Ma < 1.0)) return fail2(LNS_ERR_ARG, "ctx2d_create: with xper = 0, need Ma < 1");
    if (p->extrap < -1 || p->extrap > 1)
      return fail2(LNS_ERR_ARG, "ctx2d_create: extrap must be -1, 0 or 1 (the reference's xi LHS rejects 2)");
    if (p->nbl < 0 || p->nbl > p->ny) return fail2(LNS_ERR_ARG, "ctx2d_create: need 0 <= nbl <= ny");
    if (p->update_nbl != 0 && p->update_nbl != 1) return fail2(LNS_ERR_ARG, "ctx2d_create: update_nbl must be 0 or 1");
    if (p->lhs_order == 2)
      return fail2(LNS_ERR_ARG, "ctx2d_create: a non-periodic xi direction is supported with the fourth-order LHS");
    if (p->nx < 10) return fail2(LNS_ERR_ARG, "ctx2d_create: a non-periodic xi direction needs nx >= 10");
  }
  if (p->yper != 0 || p->navier != 1) return fail2(LNS_ERR_ARG, "ctx2d_create: need yper = 0 and navier = 1");
  if (p->wall != 0 && p->wall != 1 && p->wall != 3) return fail2(LNS_ERR_ARG, "ctx2d_create: wall must be 0, 1 or 3");
  if (p->wallt != 0 && p->wallt != 1) return fail2(LNS_ERR_ARG, "ctx2d_create: wallt must be 0 or 1");
  if (p->top != 0 && p->top != 3) return fail2(LNS_ERR_ARG, "ctx2d_create: top must be 0 or 3");
  if (p->top == 3 && p->lhs_order == 2)
    return fail2(LNS_ERR_ARG, "ctx2d_create: the held top (top 3) is supported with the fourth-order LHS");
  if (!(p->Ma > 0.0) || p->Ma == 1.0) return fail2(LNS_ERR_ARG, "ctx2d_create: need Ma > 0 and Ma != 1");
  if (p->loctime != 0 && p->loctime != 1) return fail2(LNS_ERR_ARG, "ctx2d_create: loctime must be 0 or 1");
  if (p->lhs_order != 0 && p->lhs_order != 2 && p->lhs_order != 4)
    return fail2(LNS_ERR_ARG, "ctx2d_create: lhs_order must be 0 (fourth order), 2 or 4");
  if (p->lhs_order == 2 && p->ny < 8) return fail2(LNS_ERR_ARG, "ctx2d_create: the second-order LHS needs ny >= 8");
  if (p->impl < 0 || p->impl > 3) return fail2(LNS_ERR_ARG, "ctx2d_create: impl must be 0 or 1 (backward Euler), 2 or 3");
  if (p->ispg != 0 && p->ispg != 2)
    return fail2(LNS_ERR_ARG, "ctx2d_create: ispg must be 0 or 2 (the reference's nonlinear sponge)");
  if (!(p->eps_e >= 0.0) || !std::isfinite(p->eps_e))
    return fail2(LNS_ERR_ARG, "ctx2d_create: eps_e must be finite and >= 0");
  lns_ctx2d* c = new lns_ctx2d();
  c->prm = *p;
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) {
    delete c;
    return cuda2(e, "cudaGetDevice");
  }
  Grid& g = c->g;
  g.nx = p->nx; g.ny = p->ny; g.dxi = p->dxi; g.deta = p->deta;
  g.Ma = p->Ma; g.Re = p->Re; g.Pr = p->Pr; g.gamma = p->gamma;
  g.gamma1 = p->gamma1 != 0.0 ? p->gamma1 : p->gamma - 1.0;
  g.omega = 0.0; g.kz = 0.0; g.alfa = p->alfa;
  g.xper = p->xper; g.yper = p->yper; g.navier = p->navier; g.wall = p->wall; g.wallt = p->wallt; g.top = p->top;
  g.left = p->xper ? -1 : p->left; g.right = p->xper ? -1 : p->right;
  g.dxinv = 1.0 / p->dxi; g.dyinv = 1.0 / p->deta;
  g.dxsinv = 1.0 / (p->dxi * p->dxi); g.dysinv = 1.0 / (p->deta * p->deta);
  coef1(p->optx, g.dxinv, g.gx);
  coef1(p->opty, g.dyinv, g.gy);
  coef2(p->optx, g.dxsinv, g.dx2);
  coef2(p->opty, g.dysinv, g.dy2);
  const long long np = (long long)p->nx * p->ny;
  c->np = np;
  c->nparts = std::max(((p->nx + 127) / 128) * p->ny, (int)((np + 255) / 256));
  void* q = nullptr;
  int rc = LNS_OK;
  auto A = [&](size_t bytes, void** dst) {
    if (!rc) rc = dalloc2(c, bytes, dst);
  };
  A(sizeof(double) * 10 * np, &q); c->metrics = (double*)q;
  A(sizeof(double) * (3 * 25 + 3 * 6 + 1) * np, &q); c->opbuf = (double*)q;
  A(sizeof(double) * 2 * p->nx, &q); c->bnt = (double*)q;
  A(sizeof(double) * 5 * p->nx, &q); c->pot = (double*)q;
  A(sizeof(int), &q); c->nbl = (int*)q;
  A(sizeof(double) * lns::rows::kRec * np, &q); c->rowwork = (double*)q;
  if (p->xper == 0) {
    A(sizeof(double) * 2 * p->ny, &q); c->bnl = (double*)q;
    A(sizeof(double) * 5 * p->ny, &q); c->potl = (double*)q;
    A(sizeof(double) * 2 * p->ny, &q); c->bnr = (double*)q;
    A(sizeof(double) * 5 * p->ny, &q); c->potr = (double*)q;
  }
  A(sizeof(double) * 5 * np, &q); c->v = (double*)q;
  A(sizeof(double) * 5 * np, &q); c->vold = (double*)q;
  A(sizeof(double) * 5 * np, &q); c->r = (double*)q;
  A(sizeof(double) * 125 * np, &q); c->mat = (double*)q;
  A(sizeof(double) * 50 * np, &q); c->per = (double*)q;
  A(sizeof(double) * 150 * p->ny, &q); c->per2 = (double*)q;
  A(sizeof(double) * c->nparts, &q); c->part = (double*)q;
  A(sizeof(double) * 3, &q); c->dscal = (double*)q;
  A(sizeof(int), &q); c->status = (int*)q;
  A(sizeof(double) * 64, &q); c->res_dev = (double*)q;
  if (p->impl == 2) { A(sizeof(double) * 5 * np, &q); c->v2old = (double*)q; }
  if (p->impl == 3) { A(sizeof(double) * 5 * np, &q); c->wavg = (double*)q; }
  if (p->ispg != 0) { A(sizeof(double) * np, &q); c->spg = (double*)q; }
  if (p->eps_e != 0.0) { A(sizeof(double) * np, &q); c->buff = (double*)q; }
  if (!rc) {
    c->res_cap = 64;
    e = cudaMemset(c->dscal, 0, sizeof(double) * 3);
    const int nbl0 = p->xper ? 0 : p->nbl;
    if (e == cudaSuccess) e = cudaMemcpy(c->nbl, &nbl0, sizeof(int), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) rc = cuda2(e, "context init");
  }
  if (rc) {
    free2(c);
    delete c;
    return rc;
  }
  double* o = c->opbuf;
  c->ops.np = np;
  c->ops.Ah = o; c->ops.Bh = o + 25 * np; c->ops.Dh = o + 50 * np;
  c->ops.Dhi = nullptr;
  c->ops.V11 = o + 75 * np; c->ops.V12 = o + 81 * np; c->ops.V22 = o + 87 * np;
  c->ops.AB = nullptr;
  c->ops.dtl = o + 93 * np;
  if (c->buff) {
    // the reference's default buffer (ibuff = 0, src/buffer.f90): ones
    std::vector<double> ones((size_t)np, 1.0);
    e = cudaMemcpy(c->buff, ones.data(), sizeof(double) * np, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      free2(c);
      delete c;
      return cuda2(e, "buffer init");
    }
    c->ops.buff = c->buff;
    c->ops.eps_e = p->eps_e;
  }
  *out = c;
  return LNS_OK;
}

int lns_ctx2d_destroy(lns_ctx2d* c) {
  if (!c) return LNS_OK;
  free2(c);
  delete c;
  return LNS_OK;
}

size_t lns_ctx2d_bytes(const lns_ctx2d* c) { return c ? c->bytes : 0; }

int lns_upload_metrics2d(lns_ctx2d* c, const double* metrics) {
  if (!c || !metrics) return fail2(LNS_ERR_ARG, "upload_metrics2d: null argument");
  int rc = check_dev2(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->metrics, metrics, sizeof(double) * 10 * c->np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda2(e, "upload metrics");
  c->have_metrics = true;
  return LNS_OK;
}

int lns_upload_top2d(lns_ctx2d* c, const double* bnt, const double* pot) {
  if (!c || !bnt || !pot) return fail2(LNS_ERR_ARG, "upload_top2d: null argument");
  int rc = check_dev2(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->bnt, bnt, sizeof(double) * 2 * c->g.nx, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(c->pot, pot, sizeof(double) * 5 * c->g.nx, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda2(e, "upload far field");
  c->have_top = true;
  return LNS_OK;
}

int lns_upload_side2d(lns_ctx2d* c, int32_t side, const double* bn, const double* pot) {
  if (!c || !bn || !pot) return fail2(LNS_ERR_ARG, "upload_side2d: null argument");
  if (side != 1 && side != 2) return fail2(LNS_ERR_ARG, "upload_side2d: side must be 1 (left) or 2 (right)");
  if (c->g.xper) return fail2(LNS_ERR_ARG, "upload_side2d: the context has a periodic xi direction");
  int rc = check_dev2(c);
  if (rc) return rc;
  double* b = side == 1 ? c->bnl : c->bnr;
  double* q = side == 1 ? c->potl : c->potr;
  cudaError_t e = cudaMemcpy(b, bn, sizeof(double) * 2 * c->g.ny, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(q, pot, sizeof(double) * 5 * c->g.ny, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda2(e, "upload side far field");
  (side == 1 ? c->have_left : c->have_right) = true;
  return LNS_OK;
}

int lns_upload_sponge2d(lns_ctx2d* c, const double* spg, const double* spg2) {
  if (!c || !spg || !spg2) return fail2(LNS_ERR_ARG, "upload_sponge2d: null argument");
  if (!c->spg) return fail2(LNS_ERR_ARG, "upload_sponge2d: the context was created with ispg = 0");
  int rc = check_dev2(c);
  if (rc) return rc;
  // the sponge enters the RHS and the LHS only as spg + spg2 (src/genmtrx.f90:
  // 440-444, src/lhsf.f90:307-312, src/lhsbt2f.f90:102-108): add once here
  std::vector<double> h((size_t)c->np);
  for (long long k = 0; k < c->np; ++k) h[k] = spg[k] + spg2[k];
  cudaError_t e = cudaMemcpy(c->spg, h.data(), sizeof(double) * c->np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda2(e, "upload sponge");
  c->ops.spg = c->spg;
  c->have_sponge = true;
  return LNS_OK;
}

int lns_upload_buffer2d(lns_ctx2d* c, const double* buff) {
  if (!c || !buff) return fail2(LNS_ERR_ARG, "upload_buffer2d: null argument");
  if (!c->buff) return fail2(LNS_ERR_ARG, "upload_buffer2d: the context was created with eps_e = 0");
  int rc = check_dev2(c);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(c->buff, buff, sizeof(double) * c->np, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda2(e, "upload buffer");
  return LNS_OK;
}

static int ready2(lns_ctx2d* c, const char* who) {
  if (!c->have_metrics || (!c->have_top && c->prm.top == 0 && c->prm.Ma < 1.0))
    return fail2(LNS_ERR_ARG, std::string(who) + ": upload the metrics and the far field first");
  if (!c->g.xper && ((c->prm.left == 0 && !c->have_left) || (c->prm.right == 0 && !c->have_right)))
    return fail2(LNS_ERR_ARG, std::string(who) + ": upload the far field of the Riemann xi planes first");
  if (c->prm.ispg != 0 && !c->have_sponge)
    return fail2(LNS_ERR_ARG, std::string(who) + ": ispg != 0: upload the sponge first");
  return check_dev2(c);
}

int lns_itrbc2d_dev(lns_ctx2d* c, double* v, void* stream) {
  if (!c || !v) return fail2(LNS_ERR_ARG, "itrbc2d: null argument");
  int rc = ready2(c, "itrbc2d");
  if (rc) return rc;
  return bc2(c, v, (cudaStream_t)stream);
}

int lns_step2d_dev(lns_ctx2d* c, double* v, int32_t nsteps, int32_t niter, double* totres_dev, void* stream) {
  if (!c || !v) return fail2(LNS_ERR_ARG, "step2d: null argument");
  if (nsteps < 0 || niter < 1) return fail2(LNS_ERR_ARG, "step2d: need nsteps >= 0 and niter >= 1");
  int rc = ready2(c, "step2d");
  if (rc) return rc;
  return run2(c, v, nsteps, niter, totres_dev, (cudaStream_t)stream);
}

int lns_step2d(lns_ctx2d* c, double* v, int32_t nsteps, int32_t niter, double* totres) {
  if (!c || !v) return fail2(LNS_ERR_ARG, "step2d: null argument");
  if (nsteps < 0 || niter < 1) return fail2(LNS_ERR_ARG, "step2d: need nsteps >= 0 and niter >= 1");
  int rc = ready2(c, "step2d");
  if (rc) return rc;
  if (totres && nsteps > c->res_cap) {
    void* q = nullptr;
    rc = dalloc2(c, sizeof(double) * nsteps, &q);
    if (rc) return rc;
    c->res_dev = (double*)q;
    c->res_cap = nsteps;
  }
  const size_t vbytes = sizeof(double) * 5 * (size_t)c->np;
  cudaError_t e = cudaMemcpy(c->v, v, vbytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda2(e, "upload v");
  rc = run2(c, c->v, nsteps, niter, totres ? c->res_dev : nullptr, 0);
  if (!rc) rc = check_pivots2(c, 0);
  if (rc) return rc;
  e = cudaMemcpy(v, c->v, vbytes, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda2(e, "download v");
  if (totres && nsteps > 0) {
    e = cudaMemcpy(totres, c->res_dev, sizeof(double) * nsteps, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda2(e, "download totres");
  }
  return LNS_OK;
}

int lns_rhs2d_dev(lns_ctx2d* c, const double* v, const double* vold, double* r, double* totres_dev, void* stream) {
  if (!c || !v || !vold || !r) return fail2(LNS_ERR_ARG, "rhs2d: null argument");
  int rc = ready2(c, "rhs2d");
  if (rc) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  rc = time_step(c, v, st);
  if (!rc) rc = rhs2(c, v, v, vold, nullptr, r, totres_dev ? totres_dev : c->dscal + 1, st);
  return rc;
}

int lns_lhs2d_dev(lns_ctx2d* c, int32_t dir, const double* v, double* mat, void* stream) {
  if (!c || !v || !mat) return fail2(LNS_ERR_ARG, "lhs2d: null argument");
  if (dir != 1 && dir != 2) return fail2(LNS_ERR_ARG, "lhs2d: dir must be 1 or 2");
  int rc = ready2(c, "lhs2d");
  if (rc) return rc;
  return lhs2(c, v, dir, mat, c->prm.alfa, (cudaStream_t)stream);
}

int lns_get_field2d(lns_ctx2d* c, int32_t which, double* out) {
  if (!c || !out) return fail2(LNS_ERR_ARG, "get_field2d: null argument");
  if (which < 0 || which > 6) return fail2(LNS_ERR_ARG, "get_field2d: which must be 0..6");
  int rc = check_dev2(c);
  if (rc) return rc;
  const long long np = c->np;
  const double* src[7] = {c->ops.Ah, c->ops.Bh, c->ops.Dh, c->ops.V11, c->ops.V12, c->ops.V22, c->ops.dtl};
  const int nel = which < 3 ? 25 : (which < 6 ? 6 : 1);
  std::vector<double> h((size_t)nel * np);
  cudaError_t e = cudaMemcpy(h.data(), src[which], sizeof(double) * h.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda2(e, "get_field2d copy");
  for (long long p = 0; p < np; ++p)
    for (int k = 0; k < nel; ++k) out[k + (long long)nel * p] = h[(size_t)k * np + p];
  return LNS_OK;
}

}  // extern "C"
