/*
 * CPU oracle for the linearised single-Fourier-mode implicit ADI step.
 * TEST INFRASTRUCTURE ONLY (see adi3d_oracle.h for scope and citations).
 * Built with -ffp-contract=off: every expression is evaluated left to right
 * with separate roundings, as the reference Fortran on x86-64.
 */
#include "adi3d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "penta_oracle.h"

#include "oracle_common.h"


/* ------------------------------------------------------------------ stencils */

/* coefficients of the 7-point first / second derivative, src/cgrad.f90:35-75,
   src/cgrad2.f90:38-100 */
static void coef1(int opt, double dinv, double g[6]) {
  double c, a, b;
  if (opt == 0) c = 1.0 / 60.0;
  else if (opt == -1) c = 0.0;
  else {
    double w = 2.0 * 3.1415926535897932385e+0 / 12.0;
    c = (w / 2.0 - 2.0 * sin(w) / 3.0 + sin(2.0 * w) / 12.0) / (5.0 * sin(w) - 4.0 * sin(2.0 * w) + sin(3.0 * w));
  }
  a = (2.0 + 15.0 * c) / 3.0;
  b = -(1.0 + 48.0 * c) / 12.0;
  g[0] = -c * dinv; g[1] = -b * dinv; g[2] = -a * dinv;
  g[3] = a * dinv;  g[4] = b * dinv;  g[5] = c * dinv;
}
static void coef2(int opt, double dsinv, double d[7]) {
  double c, a, b;
  if (opt == 0) c = 1.0 / 90.0;
  else if (opt == -1) c = 0.0;
  else {
    double w = 2.0 * 3.1415926535897932385e+0 / 12.0;
    double s1 = sin(w / 2.0), s2 = sin(w), s3 = sin(3.0 * w / 2.0);
    c = -(3.0 * (w * w) - 16.0 * (s1 * s1) + (s2 * s2)) / (12.0 * (-15.0 * (s1 * s1) + 6.0 * (s2 * s2) - (s3 * s3)));
  }
  a = (4.0 + 45.0 * c) / 3.0;
  b = -(1.0 + 72.0 * c) / 12.0;
  d[0] = c * dsinv; d[1] = b * dsinv; d[2] = a * dsinv; d[3] = -2.0 * (a + b + c) * dsinv;
  d[4] = a * dsinv; d[5] = b * dsinv; d[6] = c * dsinv;
}

/* One line of length n (stride s over u) of the first derivative:
   periodic (period n-1, point n = point 1) or with the one-sided closures
   gc, gb, ga of src/cgrad.f90:130-178. */
static void line_d1(int n, int periodic, const double* u, long s, double* out, long so, const double g[6],
                    double dinv) {
#define U(k) u[(long)((k) - 1) * s]
#define O(k) out[(long)((k) - 1) * so]
  if (periodic) {
    for (int i = 1; i <= n - 1; ++i) {
      int k[6] = {i - 3, i - 2, i - 1, i + 1, i + 2, i + 3};
      for (int t = 0; t < 6; ++t) {
        if (k[t] < 1) k[t] += n - 1;
        if (k[t] > n - 1) k[t] -= n - 1;
      }
      O(i) = g[0] * U(k[0]) + g[1] * U(k[1]) + g[2] * U(k[2]) + g[3] * U(k[3]) + g[4] * U(k[4]) + g[5] * U(k[5]);
    }
    O(n) = O(1);
  } else {
    O(1) = (gc1 * U(1) + gc2 * U(2) + gc3 * U(3) + gc4 * U(4) + gc5 * U(5)) * dinv;
    O(2) = (gb1 * U(1) + gb2 * U(2) + gb3 * U(3) + gb4 * U(4) + gb5 * U(5)) * dinv;
    O(3) = (ga1 * U(1) + ga2 * U(2) + ga3 * U(4) + ga4 * U(5)) * dinv;
    O(n - 2) = (ga1 * U(n - 4) + ga2 * U(n - 3) + ga3 * U(n - 1) + ga4 * U(n)) * dinv;
    O(n - 1) = -((gb1 * U(n) + gb2 * U(n - 1) + gb3 * U(n - 2) + gb4 * U(n - 3) + gb5 * U(n - 4)) * dinv);
    O(n) = -((gc1 * U(n) + gc2 * U(n - 1) + gc3 * U(n - 2) + gc4 * U(n - 3) + gc5 * U(n - 4)) * dinv);
    for (int i = 4; i <= n - 3; ++i)
      O(i) = g[0] * U(i - 3) + g[1] * U(i - 2) + g[2] * U(i - 1) + g[3] * U(i + 1) + g[4] * U(i + 2) +
             g[5] * U(i + 3);
  }
}
/* second derivative, src/cgrad2.f90:102-250 */
static void line_d2(int n, int periodic, const double* u, long s, double* out, long so, const double d[7],
                    double dsinv) {
  if (periodic) {
    for (int i = 1; i <= n - 1; ++i) {
      int k[7] = {i - 3, i - 2, i - 1, i, i + 1, i + 2, i + 3};
      for (int t = 0; t < 7; ++t) {
        if (k[t] < 1) k[t] += n - 1;
        if (k[t] > n - 1) k[t] -= n - 1;
      }
      O(i) = d[0] * U(k[0]) + d[1] * U(k[1]) + d[2] * U(k[2]) + d[3] * U(k[3]) + d[4] * U(k[4]) +
             d[5] * U(k[5]) + d[6] * U(k[6]);
    }
    O(n) = O(1);
  } else {
    O(1) = (dd1 * U(1) + dd2 * U(2) + dd3 * U(3) + dd4 * U(4) + dd5 * U(5)) * dsinv;
    O(2) = (db1 * U(1) + db2 * U(2) + db3 * U(3) + db4 * U(4) + db5 * U(5)) * dsinv;
    O(3) = (da1 * U(1) + da2 * U(2) + da3 * U(3) + da4 * U(4) + da5 * U(5)) * dsinv;
    O(n - 2) = (da1 * U(n - 4) + da2 * U(n - 3) + da3 * U(n - 2) + da4 * U(n - 1) + da5 * U(n)) * dsinv;
    O(n - 1) = (db1 * U(n) + db2 * U(n - 1) + db3 * U(n - 2) + db4 * U(n - 3) + db5 * U(n - 4)) * dsinv;
    O(n) = (dd1 * U(n) + dd2 * U(n - 1) + dd3 * U(n - 2) + dd4 * U(n - 3) + dd5 * U(n - 4)) * dsinv;
    for (int i = 4; i <= n - 3; ++i)
      O(i) = d[0] * U(i - 3) + d[1] * U(i - 2) + d[2] * U(i - 1) + d[3] * U(i) + d[4] * U(i + 1) +
             d[5] * U(i + 2) + d[6] * U(i + 3);
  }
#undef U
#undef O
}

/* src/cgrad.f90 (and src/grad.f90): g1v = d/dxi, g2v = d/deta */
int a3_deriv1(const A3Grid* g, int nc, const double* v, double* g1v, double* g2v) {
  double gx[6], gy[6];
  coef1(g->optx, one / g->dxi, gx);
  coef1(g->opty, one / g->deta, gy);
  const int nx = g->nx, ny = g->ny;
  OMP_FOR
  for (int j = 1; j <= ny; ++j)
    for (int c = 0; c < nc; ++c)
      line_d1(nx, g->xper, &FV(v, nc, c, g, 1, j), nc, &FV(g1v, nc, c, g, 1, j), nc, gx, one / g->dxi);
  OMP_FOR
  for (int i = 1; i <= nx; ++i)
    for (int c = 0; c < nc; ++c)
      line_d1(ny, g->yper, &FV(v, nc, c, g, i, 1), (long)nc * nx, &FV(g2v, nc, c, g, i, 1), (long)nc * nx, gy,
              one / g->deta);
  return 0;
}

/* src/cgrad2.f90 (and src/grad2.f90): g11v, g22v, and g12v = d/deta of g1v */
int a3_deriv2(const A3Grid* g, int nc, const double* v, const double* g1v, double* g11v, double* g12v,
              double* g22v) {
  double dx[7], dy[7], gy[6];
  const double dxsinv = one / (g->dxi * g->dxi), dysinv = one / (g->deta * g->deta);
  coef2(g->optx, dxsinv, dx);
  coef2(g->opty, dysinv, dy);
  coef1(g->opty, one / g->deta, gy);
  const int nx = g->nx, ny = g->ny;
  OMP_FOR
  for (int j = 1; j <= ny; ++j)
    for (int c = 0; c < nc; ++c)
      line_d2(nx, g->xper, &FV(v, nc, c, g, 1, j), nc, &FV(g11v, nc, c, g, 1, j), nc, dx, dxsinv);
  OMP_FOR
  for (int i = 1; i <= nx; ++i)
    for (int c = 0; c < nc; ++c) {
      line_d2(ny, g->yper, &FV(v, nc, c, g, i, 1), (long)nc * nx, &FV(g22v, nc, c, g, i, 1), (long)nc * nx, dy,
              dysinv);
      line_d1(ny, g->yper, &FV(g1v, nc, c, g, i, 1), (long)nc * nx, &FV(g12v, nc, c, g, i, 1), (long)nc * nx, gy,
              one / g->deta);
    }
  return 0;
}

/* ---------------------------------------------------------------- operators */

/* src/genmtrx.f90 with linear = 1, general = true, mattyp = 0, idamp = 0,
   complex_analysis = true: the frozen operators of the linear step. */
int a3_genmtrx(const A3Grid* g, const double* vl, A3Ops* o) {
  const int nx = g->nx, ny = g->ny;
  const long np = (long)nx * ny;
  double* g1v = (double*)calloc(5 * np, sizeof(double));
  double* g2v = (double*)calloc(5 * np, sizeof(double));
  double* g11v = (double*)calloc(5 * np, sizeof(double));
  double* g12v = (double*)calloc(5 * np, sizeof(double));
  double* g22v = (double*)calloc(5 * np, sizeof(double));
  if (!g1v || !g2v || !g11v || !g12v || !g22v) return 3;
  a3_deriv1(g, 5, vl, g1v, g2v);                 /* genmtrx.f90:72 */
  a3_deriv2(g, 5, vl, g1v, g11v, g12v, g22v);    /* genmtrx.f90:77 */
  if (g->navier && !g->yper && (g->wallt == 1 || g->wallt == 2))  /* gradbc.f90 */
    for (int i = 1; i <= nx; ++i) FV(g2v, 5, 4, g, i, 1) = zero;
  const double gamma = g->gamma, gamma1 = g->gamma1, Ma = g->Ma, Re = g->Re, Pr = g->Pr, kzl = g->kz;
  OMP_FOR
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const long p = IX(g, i, j);
      const double m1 = g->m1[p], m2 = g->m2[p], n1 = g->n1[p], n2 = g->n2[p];
      const double m11 = g->m11[p], m12 = g->m12[p], m22 = g->m22[p], n11 = g->n11[p], n12 = g->n12[p],
                   n22 = g->n22[p];
      /* metric products, src/gengrid.f90:96-131 */
      const double m1m1 = m1 * m1, m1m2 = m1 * m2, m2m2 = m2 * m2, n1n1 = n1 * n1, n1n2 = n1 * n2, n2n2 = n2 * n2;
      const double m1n1 = m1 * n1, m1n2 = m1 * n2, m2n1 = m2 * n1, m2n2 = m2 * n2;
      double g1vl[5], g2vl[5], g11vl[5], g12vl[5], g22vl[5];
      for (int k = 0; k < 5; ++k) { /* genmtrx.f90:116-136 */
        const double a1 = FV(g1v, 5, k, g, i, j), a2 = FV(g2v, 5, k, g, i, j);
        const double a11 = FV(g11v, 5, k, g, i, j), a12 = FV(g12v, 5, k, g, i, j), a22 = FV(g22v, 5, k, g, i, j);
        g11vl[k] = a11 * m1m1 + two * a12 * m1n1 + a22 * n1n1 + a1 * m11 + a2 * n11;
        g12vl[k] = a11 * m1m2 + a12 * (m1n2 + m2n1) + a22 * n1n2 + a1 * m12 + a2 * n12;
        g22vl[k] = a11 * m2m2 + two * a12 * m2n2 + a22 * n2n2 + a1 * m22 + a2 * n22;
        g1vl[k] = a1 * m1 + a2 * n1;
        g2vl[k] = a1 * m2 + a2 * n2;
      }
      /* genmtrx.f90:158-230 */
      const double rho = FV(vl, 5, 0, g, i, j), u1 = FV(vl, 5, 1, g, i, j), u2 = FV(vl, 5, 2, g, i, j),
                   u3 = FV(vl, 5, 3, g, i, j), t = FV(vl, 5, 4, g, i, j);
      const double rhoinv = one / rho;
      const double grho[3] = {g1vl[0], g2vl[0], zero};
      const double gu[3][3] = {{g1vl[1], g2vl[1], zero}, {g1vl[2], g2vl[2], zero}, {g1vl[3], g2vl[3], zero}};
      const double gt[3] = {g1vl[4], g2vl[4], zero};
      const double g1divu = g11vl[1] + g12vl[2];
      const double g2divu = g12vl[1] + g22vl[2];
      const double g3divu = zero;
      const double S1jj = pt5 * (g11vl[1] + g11vl[1] + g22vl[1] + g12vl[2]);
      const double S2jj = pt5 * (g11vl[2] + g12vl[1] + g22vl[2] + g22vl[2]);
      const double S3jj = pt5 * (g11vl[3] + g22vl[3]);
      const double Lapt = g11vl[4] + g22vl[4];
      const double divu = gu[0][0] + gu[1][1] + gu[2][2];
      double S[3][3] = {{0}};
      S[0][0] = gu[0][0];
      S[1][0] = pt5 * (gu[1][0] + gu[0][1]);
      S[2][0] = pt5 * gu[2][0];
      S[0][1] = pt5 * (gu[0][1] + gu[1][0]);
      S[1][1] = gu[1][1];
      S[2][1] = pt5 * gu[2][1];
      S[0][2] = pt5 * gu[2][0];
      S[1][2] = pt5 * gu[2][1];
      /* getmat, src/getmat.f90:11-20 (mattyp 0) */
      const double mu = one, dmu = zero, d2mu = zero, con = mu, dcon = dmu, d2con = d2mu;
      const double lm = -pt66 * mu, dlm = -pt66 * dmu, d2lm = -pt66 * d2mu;
      const double g1mu = dmu * gt[0], g2mu = dmu * gt[1], g3mu = dmu * gt[2];
      const double g1dmu = d2mu * gt[0], g2dmu = d2mu * gt[1], g3dmu = d2mu * gt[2];
      const double g1con = dcon * gt[0], g2con = dcon * gt[1], g3con = dcon * gt[2];
      const double g1dcon = d2con * gt[0], g2dcon = d2con * gt[1], g3dcon = d2con * gt[2];
      const double g1lm = dlm * gt[0], g2lm = dlm * gt[1], g3lm = dlm * gt[2];
      const double g1dlm = d2lm * gt[0], g2dlm = d2lm * gt[1], g3dlm = d2lm * gt[2];
      double A[5][5] = {{0}}, B[5][5] = {{0}}, C[5][5] = {{0}}, D[5][5] = {{0}}, Vij[4];
      double fact1, fact2, gmsinv;
      /* A, genmtrx.f90:463-507 */
      A[0][0] = u1; A[0][1] = rho;
      fact1 = rhoinv / Re;
      gmsinv = one / (gamma * (Ma * Ma));
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
      fact1 = gamma * rhoinv / (Pr * Re);
      fact2 = gamma * gamma1 * (Ma * Ma) * rhoinv / Re;
      A[4][1] = gamma1 * t - fact2 * two * lm * divu - four * fact2 * mu * S[0][0];
      A[4][2] = -(four * fact2 * mu * S[1][0]);
      A[4][3] = -(four * fact2 * mu * S[2][0]);
      A[4][4] = u1 - fact1 * (g1con + dcon * gt[0]);
      /* B, genmtrx.f90:530-574 */
      B[0][0] = u2; B[0][2] = rho;
      fact1 = rhoinv / Re;
      gmsinv = one / (gamma * (Ma * Ma));
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
      fact1 = gamma * rhoinv / (Pr * Re);
      fact2 = gamma * gamma1 * (Ma * Ma) * rhoinv / Re;
      B[4][1] = -(four * fact2 * mu * S[0][1]);
      B[4][2] = gamma1 * t - fact2 * two * lm * divu - four * fact2 * mu * S[1][1];
      B[4][3] = -(four * fact2 * mu * S[2][1]);
      B[4][4] = u2 - fact1 * (g2con + dcon * gt[1]);
      /* Vij, genmtrx.f90:590-600 */
      fact1 = one / Re;
      fact2 = gamma / (Pr * Re);
      Vij[0] = fact1 * rhoinv * (lm + two * mu);
      Vij[1] = fact1 * rhoinv * mu;
      Vij[2] = fact2 * rhoinv * con;
      Vij[3] = fact1 * rhoinv * (lm + mu);
      /* \hat{A} and \hat{B}, genmtrx.f90:608-694 */
      for (int pass = 0; pass < 2; ++pass) {
        double* H = pass == 0 ? o->Ah : o->Bh;
        const double e1 = pass == 0 ? m1 : n1, e2 = pass == 0 ? m2 : n2;
        const double e11 = pass == 0 ? m11 : n11, e12 = pass == 0 ? m12 : n12, e22 = pass == 0 ? m22 : n22;
#define H_(a, b) H[(a - 1) + 5 * (b - 1) + 25 * p]
        H_(1, 1) = A[0][0] * e1 + B[0][0] * e2;
        H_(1, 2) = A[0][1] * e1;
        H_(1, 3) = B[0][2] * e2;
        H_(1, 4) = zero;
        H_(1, 5) = zero;
        H_(2, 1) = A[1][0] * e1;
        H_(2, 2) = A[1][1] * e1 + B[1][1] * e2 - Vij[0] * e11 - Vij[1] * e22;
        H_(2, 3) = A[1][2] * e1 + B[1][2] * e2 - Vij[3] * e12;
        H_(2, 4) = A[1][3] * e1;
        H_(2, 5) = A[1][4] * e1 + B[1][4] * e2;
        H_(3, 1) = B[2][0] * e2;
        H_(3, 2) = A[2][1] * e1 + B[2][1] * e2 - Vij[3] * e12;
        H_(3, 3) = A[2][2] * e1 + B[2][2] * e2 - Vij[1] * e11 - Vij[0] * e22;
        H_(3, 4) = B[2][3] * e2;
        H_(3, 5) = A[2][4] * e1 + B[2][4] * e2;
        H_(4, 1) = zero;
        H_(4, 2) = A[3][1] * e1;
        H_(4, 3) = B[3][2] * e2;
        H_(4, 4) = A[3][3] * e1 + B[3][3] * e2 - Vij[1] * e11 - Vij[1] * e22;
        H_(4, 5) = A[3][4] * e1 + B[3][4] * e2;
        H_(5, 1) = A[4][0] * e1 + B[4][0] * e2;
        H_(5, 2) = A[4][1] * e1 + B[4][1] * e2;
        H_(5, 3) = A[4][2] * e1 + B[4][2] * e2;
        H_(5, 4) = A[4][3] * e1 + B[4][3] * e2;
        H_(5, 5) = A[4][4] * e1 + B[4][4] * e2 - Vij[2] * e11 - Vij[2] * e22;
        if (pass == 1 && !g->yper && g->wallt == 2 && j == 1)
          for (int a = 1; a <= 5; ++a) H_(a, 5) = zero;
#undef H_
      }
      /* D, genmtrx.f90:708-820 (linear = 1) */
      D[0][0] = divu; D[0][1] = grho[0]; D[0][2] = grho[1]; D[0][3] = grho[2]; D[0][4] = zero;
      fact1 = rhoinv / Re;
      gmsinv = one / (gamma * (Ma * Ma));
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
      fact2 = gamma * gamma1 * (Ma * Ma) * rhoinv / Re;
      D[4][0] = rhoinv * (u1 * gt[0] + u2 * gt[1] + u3 * gt[2] + gamma1 * t * divu);
      D[4][1] = gt[0]; D[4][2] = gt[1]; D[4][3] = gt[2];
      D[4][4] = -(gamma1 * rhoinv * (u1 * grho[0] + u2 * grho[1] + u3 * grho[2]));
      {
        const double ssq = S[0][0] * S[0][0] + S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][0] * S[1][0] +
                           S[1][1] * S[1][1] + S[1][2] * S[1][2] + S[2][0] * S[2][0] + S[2][1] * S[2][1] +
                           S[2][2] * S[2][2];
        D[4][4] = D[4][4] - fact1 * (g1dcon * gt[0] + g2dcon * gt[1] + g3dcon * gt[2] + dcon * Lapt) -
                  fact2 * dlm * (divu * divu) - two * fact2 * dmu * ssq;
      }
      for (int a = 0; a < 5; ++a)
        for (int b = 0; b < 5; ++b) o->Dh[a + 5 * b + 25 * p] = D[a][b];
      if (kzl != zero) { /* genmtrx.f90:843-848 */
        o->Dh[1 + 5 * 1 + 25 * p] = o->Dh[1 + 5 * 1 + 25 * p] + (kzl * kzl) * Vij[1];
        o->Dh[2 + 5 * 2 + 25 * p] = o->Dh[2 + 5 * 2 + 25 * p] + (kzl * kzl) * Vij[1];
        o->Dh[3 + 5 * 3 + 25 * p] = o->Dh[3 + 5 * 3 + 25 * p] + (kzl * kzl) * Vij[0];
        o->Dh[4 + 5 * 4 + 25 * p] = o->Dh[4 + 5 * 4 + 25 * p] + (kzl * kzl) * Vij[2];
      }
      /* \hat{V}, genmtrx.f90:867-913 */
      double* V11 = o->Vh11 + 6 * p;
      double* V12 = o->Vh12 + 6 * p;
      double* V22 = o->Vh22 + 6 * p;
      V11[0] = Vij[0] * m1m1 + Vij[1] * m2m2;
      V11[1] = Vij[1] * m1m1 + Vij[0] * m2m2;
      V11[2] = Vij[1] * m1m1 + Vij[1] * m2m2;
      V11[3] = Vij[2] * m1m1 + Vij[2] * m2m2;
      V11[4] = Vij[3] * m1m2;
      V11[5] = Vij[3] * m1m2;
      V12[0] = two * (Vij[0] * m1n1 + Vij[1] * m2n2);
      V12[1] = two * (Vij[1] * m1n1 + Vij[0] * m2n2);
      V12[2] = two * (Vij[1] * m1n1 + Vij[1] * m2n2);
      V12[3] = two * (Vij[2] * m1n1 + Vij[2] * m2n2);
      V12[4] = Vij[3] * (m1n2 + m2n1);
      V12[5] = Vij[3] * (m1n2 + m2n1);
      V22[0] = Vij[0] * n1n1 + Vij[1] * n2n2;
      V22[1] = Vij[1] * n1n1 + Vij[0] * n2n2;
      V22[2] = Vij[1] * n1n1 + Vij[1] * n2n2;
      V22[3] = Vij[2] * n1n1 + Vij[2] * n2n2;
      V22[4] = Vij[3] * n1n2;
      V22[5] = Vij[3] * n1n2;
      /* 3D terms, genmtrx.f90:919-989 */
      double* AB = o->ABhi + 6 * p;
      AB[0] = kzl * Vij[3] * m1;
      AB[1] = kzl * Vij[3] * m2;
      AB[2] = kzl * Vij[3] * n1;
      AB[3] = kzl * Vij[3] * n2;
      AB[4] = zero;
      AB[5] = zero;
      C[0][0] = u3; C[0][3] = rho;
      fact1 = rhoinv / Re;
      gmsinv = one / (gamma * (Ma * Ma));
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
      fact1 = gamma * rhoinv / (Pr * Re);
      fact2 = gamma * gamma1 * (Ma * Ma) * rhoinv / Re;
      C[4][1] = -(four * fact2 * mu * S[0][2]);
      C[4][2] = -(four * fact2 * mu * S[1][2]);
      C[4][3] = gamma1 * t - fact2 * two * lm * divu - four * fact2 * mu * S[2][2];
      C[4][4] = u3 - fact1 * (g3con + dcon * gt[2]);
      for (int a = 0; a < 5; ++a)
        for (int b = 0; b < 5; ++b) o->Dhi[a + 5 * b + 25 * p] = kzl * C[a][b];
      for (int a = 0; a < 5; ++a) o->Dhi[a + 5 * a + 25 * p] = o->Dhi[a + 5 * a + 25 * p] - g->omega;
    }
  free(g1v); free(g2v); free(g11v); free(g12v); free(g22v);
  return 0;
}

/* src/temporal.f90:12-130, acoustic CFL */
double a3_set_time_step(const A3Grid* g, const double* vl, double* dtl) {
  const int nx = g->nx, ny = g->ny;
  double cfla = -1.0;
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const long p = IX(g, i, j);
      const double m1 = g->m1[p], m2 = g->m2[p], n1 = g->n1[p], n2 = g->n2[p];
      double volinv = one / (m1 * n2 - m2 * n1);
      const double sxj = n2 * g->dxi * volinv, syj = -m2 * g->dxi * volinv;
      const double sxi = -n1 * g->deta * volinv, syi = m1 * g->deta * volinv;
      volinv = one / (g->dxi * g->deta * volinv);
      const double acoustic = sqrt((sxi * sxi) + two * sxi * syi + (syi * syi) + (sxj * sxj) + two * sxj * syj +
                                   (syj * syj)) / g->Ma;
      const double u1 = FV(vl, 5, 1, g, i, j), u2 = FV(vl, 5, 2, g, i, j);
      const double t = sqrt(FV(vl, 5, 4, g, i, j));
      dtl[p] = (fabs(u1 * sxi + u2 * syi) + fabs(u1 * sxj + u2 * syj) + t * acoustic) * volinv;
      if (dtl[p] > cfla) cfla = dtl[p];
    }
  const double cfl = cfla;
  double delt;
  if (cfl * g->dtmax <= g->cflmax) {
    delt = g->dtmax;
    for (long p = 0; p < (long)nx * ny; ++p) dtl[p] = g->dtmax;
  } else {
    delt = g->cflmax / cfl;
    for (long p = 0; p < (long)nx * ny; ++p) dtl[p] = g->loctime == 0 ? delt : g->cflmax / dtl[p];
  }
  return cfl * delt;
}

/* --------------------------------------------------------------------- RHS */

#define CRE(a, k, g, i, j) (a)[2 * ((long)(k) + 5 * IX(g, i, j))]
#define CIM(a, k, g, i, j) (a)[2 * ((long)(k) + 5 * IX(g, i, j)) + 1]

/* src/lrhs3d.f90:33-218 (ispg 0, eps_e 0) */
/* The target of the inflow sponge at point (i, j), complex (5): with
   cm = sqrt(T)/Ma, um = U of the mean flow, d = (4/3 + (gamma-1)/Pr)/(2 Re),
   kk = omega/(cm + um), a = omega^2 d/(cm + um)^3 and
   c3 = [wamp(i)] exp(-a (x - x0)) exp(i kk x) (wamp for ispg 3 only):
   (c3/(2 cm^2), c3/(2 rho cm), 0, 0,
    (gamma Ma^2 c3/2 - T c3/(2 cm^2))/rho), src/lrhs3d.f90:248-278, in the
   reference's order of operations. */
static void a3_wave(const A3Grid* g, int i, int j, int with_wamp, double t[10]);
void a3_inflow_target(const A3Grid* g, int i, int j, double t[10]) { a3_wave(g, i, j, g->ispg == 3, t); }

/* The same wave with wamp(i) always applied: the incoming acoustic wave of
   the forced top boundary (top = 1, src/rhsbc3d.f90:129-160,
   src/itrbc3d.f90:145-196) at j = ny. */
void a3_top_target(const A3Grid* g, int i, double t[10]) { a3_wave(g, i, g->ny, 1, t); }

static void a3_wave(const A3Grid* g, int i, int j, int with_wamp, double t[10]) {
  const long p = IX(g, i, j);
  const double* vm = g->vm + 5 * p;
  const double onept33 = 1.3333333333333333333e+0;
  const double cm = sqrt(vm[4]) / g->Ma, um = vm[1];
  const double d = pt5 * (onept33 + g->gamma1 / g->Pr) / g->Re;
  const double kk = g->omega / (cm + um);
  const double cu = cm + um;
  const double a = g->omega * g->omega * d / (cu * cu * cu);
  const double xl = g->xc[p];
  const double e = exp(-a * (xl - g->x0));
  const double w = with_wamp ? g->wamp[i - 1] * e : e;
  const double c3r = w * cos(kk * xl), c3i = w * sin(kk * xl);
  const double cm2 = cm * cm;
  t[0] = pt5 * c3r / cm2, t[1] = pt5 * c3i / cm2;
  t[2] = c3r * pt5 / (vm[0] * cm), t[3] = c3i * pt5 / (vm[0] * cm);
  t[4] = t[5] = t[6] = t[7] = zero;
  const double gm2 = g->gamma * (g->Ma * g->Ma);
  t[8] = (gm2 * c3r * pt5 - vm[4] * pt5 * c3r / cm2) / vm[0];
  t[9] = (gm2 * c3i * pt5 - vm[4] * pt5 * c3i / cm2) / vm[0];
}

/* smoother3D, src/smoother3d.f90:1-200 without symmetry planes (lsym and
   rsym false): rl += eps_e buff D(vl), the eta pass first (rows 2 and ny-1
   second order, 3 and ny-2 fourth order, 4..ny-3 sixth order), then the xi
   pass with the same pattern over i (no periodic wrap, as the reference). */
static void a3_smoother(const A3Grid* g, double* rl, const double* vl) {
  const int nx = g->nx, ny = g->ny;
  const double fa1 = -1.666666666666667E-01, fa2 = 2.000000000000000E+00, fa3 = -6.500000000000000E+00,
               fa4 = 9.333333333333333E+00, fa5 = -6.500000000000000E+00, fa6 = 2.000000000000000E+00,
               fa7 = -1.666666666666667E-01; /* src/stencil.f90:145-151 */
  for (int pass = 0; pass < 2; ++pass) {
    const int n = pass == 0 ? ny : nx;
    OMP_FOR
    for (int l = 1; l <= (pass == 0 ? nx : ny); ++l)
      for (int c = 2; c <= n - 1; ++c) {
        const int i = pass == 0 ? l : c, j = pass == 0 ? c : l;
        const long st = pass == 0 ? 10L * nx : 10L;
        const long p = IX(g, i, j);
        const double eb = g->eps_e * g->buff[p];
        for (int k = 0; k < 10; ++k) {
          const double* V = vl + k + 10 * p;
#define VS(d) V[(long)(d) * st]
          double s;
          if (c == 2 || c == n - 1) s = -1.0 * VS(-1) + 2.0 * VS(0) - 1.0 * VS(1);
          else if (c == 3 || c == n - 2) s = VS(-2) - 4.0 * VS(-1) + 6.0 * VS(0) - 4.0 * VS(1) + 1.0 * VS(2);
          else s = fa1 * VS(-3) + fa2 * VS(-2) + fa3 * VS(-1) + fa4 * VS(0) + fa5 * VS(1) + fa6 * VS(2) + fa7 * VS(3);
#undef VS
          rl[k + 10 * p] = rl[k + 10 * p] + eb * s;
        }
      }
  }
}

int a3_lrhs(const A3Grid* g, const A3Ops* o, const double* vl, double* rl) {
  const int nx = g->nx, ny = g->ny;
  const long n10 = 10L * nx * ny;
  double* c1v = (double*)calloc(n10, sizeof(double));
  double* c2v = (double*)calloc(n10, sizeof(double));
  double* c11v = (double*)calloc(n10, sizeof(double));
  double* c12v = (double*)calloc(n10, sizeof(double));
  double* c22v = (double*)calloc(n10, sizeof(double));
  if (!c1v || !c2v || !c11v || !c12v || !c22v) return 3;
  a3_deriv1(g, 10, vl, c1v, c2v);
  a3_deriv2(g, 10, vl, c1v, c11v, c12v, c22v);
  if (g->navier && (g->wallt == 1 || g->wallt == 2)) /* src/cgradbc.f90 */
    for (int i = 1; i <= nx; ++i) CRE(c2v, 4, g, i, 1) = zero, CIM(c2v, 4, g, i, 1) = zero;
  OMP_FOR
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const long p = IX(g, i, j);
      const double* Ah = o->Ah + 25 * p;
      const double* Bh = o->Bh + 25 * p;
      const double* Dh = o->Dh + 25 * p;
      const double* Dhi = o->Dhi + 25 * p;
      const double* V11 = o->Vh11 + 6 * p;
      const double* V12 = o->Vh12 + 6 * p;
      const double* V22 = o->Vh22 + 6 * p;
      const double* AB = o->ABhi + 6 * p;
      for (int part = 0; part < 2; ++part) { /* real and imaginary parts */
#define C1(k) c1v[2 * ((k) + 5 * p) + part]
#define C2(k) c2v[2 * ((k) + 5 * p) + part]
#define C11(k) c11v[2 * ((k) + 5 * p) + part]
#define C12(k) c12v[2 * ((k) + 5 * p) + part]
#define C22(k) c22v[2 * ((k) + 5 * p) + part]
#define VV(k) vl[2 * ((k) + 5 * p) + part]
#define R(k) rl[2 * ((k) + 5 * p) + part]
        for (int m = 0; m < 5; ++m)
          R(m) = +Ah[m] * C1(0) + Ah[m + 5] * C1(1) + Ah[m + 10] * C1(2) + Ah[m + 15] * C1(3) + Ah[m + 20] * C1(4);
        for (int m = 0; m < 5; ++m)
          R(m) = R(m) + Bh[m] * C2(0) + Bh[m + 5] * C2(1) + Bh[m + 10] * C2(2) + Bh[m + 15] * C2(3) +
                 Bh[m + 20] * C2(4);
        for (int m = 0; m < 5; ++m)
          R(m) = R(m) + Dh[m] * VV(0) + Dh[m + 5] * VV(1) + Dh[m + 10] * VV(2) + Dh[m + 15] * VV(3) +
                 Dh[m + 20] * VV(4);
        R(1) = R(1) - V11[0] * C11(1) - V11[4] * C11(2);
        R(2) = R(2) - V11[5] * C11(1) - V11[1] * C11(2);
        R(3) = R(3) - V11[2] * C11(3);
        R(4) = R(4) - V11[3] * C11(4);
        R(1) = R(1) - V12[0] * C12(1) - V12[4] * C12(2);
        R(2) = R(2) - V12[5] * C12(1) - V12[1] * C12(2);
        R(3) = R(3) - V12[2] * C12(3);
        R(4) = R(4) - V12[3] * C12(4);
        R(1) = R(1) - V22[0] * C22(1) - V22[4] * C22(2);
        R(2) = R(2) - V22[5] * C22(1) - V22[1] * C22(2);
        R(3) = R(3) - V22[2] * C22(3);
        R(4) = R(4) - V22[3] * C22(4);
#undef C11
#undef C12
#undef C22
      }
      /* 3D terms: im * z = (-Im z, Re z), src/lrhs3d.f90:176-218 */
      {
#define Z1(k, pt) c1v[2 * ((k) + 5 * p) + pt]
#define Z2(k, pt) c2v[2 * ((k) + 5 * p) + pt]
#define ZV(k, pt) vl[2 * ((k) + 5 * p) + pt]
#define RR(k, pt) rl[2 * ((k) + 5 * p) + pt]
        double s[2];
        for (int pt = 0; pt < 2; ++pt) s[pt] = AB[0] * Z1(3, pt) + AB[2] * Z2(3, pt);
        RR(1, 0) = RR(1, 0) - (-s[1]); RR(1, 1) = RR(1, 1) - s[0];
        for (int pt = 0; pt < 2; ++pt) s[pt] = AB[1] * Z1(3, pt) + AB[3] * Z2(3, pt);
        RR(2, 0) = RR(2, 0) - (-s[1]); RR(2, 1) = RR(2, 1) - s[0];
        for (int pt = 0; pt < 2; ++pt)
          s[pt] = AB[0] * Z1(1, pt) + AB[1] * Z1(2, pt) + AB[2] * Z2(1, pt) + AB[3] * Z2(2, pt);
        RR(3, 0) = RR(3, 0) - (-s[1]); RR(3, 1) = RR(3, 1) - s[0];
        for (int m = 0; m < 5; ++m) {
          for (int pt = 0; pt < 2; ++pt)
            s[pt] = Dhi[m] * ZV(0, pt) + Dhi[m + 5] * ZV(1, pt) + Dhi[m + 10] * ZV(2, pt) + Dhi[m + 15] * ZV(3, pt) +
                    Dhi[m + 20] * ZV(4, pt);
          RR(m, 0) = RR(m, 0) + (-s[1]);
          RR(m, 1) = RR(m, 1) + s[0];
        }
#undef Z1
#undef Z2
#undef ZV
#undef RR
      }
      /* sponge, src/lrhs3d.f90:222-240: rl = rl + spg vl (ispg 1) or
         rl = rl + (spg + spg2) vl (ispg > 4) */
      if (g->ispg == 1 || g->ispg > 4) {
        const double sp = g->ispg == 1 ? g->spg[p] : g->spg[p] + g->spg2[p];
        for (int k = 0; k < 10; ++k) rl[k + 10 * p] = rl[k + 10 * p] + sp * vl[k + 10 * p];
      } else if (g->ispg == 2 || g->ispg == 3) {
        /* the outflow sponge spg on v, then the inflow sponge spg2 towards
           the decaying wave c3 (src/lrhs3d.f90:242-280) */
        for (int k = 0; k < 10; ++k) rl[k + 10 * p] = rl[k + 10 * p] + g->spg[p] * vl[k + 10 * p];
        double t[10];
        a3_inflow_target(g, i, j, t);
        for (int k = 0; k < 10; ++k) rl[k + 10 * p] = rl[k + 10 * p] + g->spg2[p] * (vl[k + 10 * p] - t[k]);
      }
#undef C1
#undef C2
#undef VV
#undef R
    }
  free(c1v); free(c2v); free(c11v); free(c12v); free(c22v);
  if (g->ispg == 4) /* cspg_it, src/sponge.f90:596-604 */
    for (long p = 0; p < (long)nx * ny; ++p) {
      const double sp = g->spg[p] + g->spg2[p];
      for (int k = 0; k < 10; ++k) rl[k + 10 * p] = rl[k + 10 * p] + sp * (vl[k + 10 * p] - g->cvic[k + 10 * p]);
    }
  if (g->eps_e != zero) a3_smoother(g, rl, vl); /* src/lrhs3d.f90:294 */
  return 0;
}

/* rbe3D, src/impdrv3d.f90:444-469: r = vold - v - dtl r */
void a3_rbe(const A3Grid* g, double* r, const double* v, const double* vold, const double* dtl) {
  OMP_FOR
  for (int j = 1; j <= g->ny; ++j)
    for (int i = 1; i <= g->nx; ++i)
      for (int k = 0; k < 10; ++k) {
        const long e = k + 10 * IX(g, i, j);
        r[e] = vold[e] - v[e] - dtl[IX(g, i, j)] * r[e];
      }
}

/* src/rhsbc3d.f90:34-170 for the supported boundary conditions */
void a3_rhsbc(const A3Grid* g, double* rl, const double* vl) {
  const int nx = g->nx, ny = g->ny;
  if (g->yper) {
    for (int i = 1; i <= nx; ++i)
      for (int k = 0; k < 5; ++k) CRE(rl, k, g, i, ny) = zero, CIM(rl, k, g, i, ny) = zero;
  } else {
    if (g->navier) {
      for (int i = 1; i <= nx; ++i)
        for (int pt = 0; pt < 2; ++pt) {
#define VR(k, jj) vl[2 * ((k) + 5 * IX(g, i, jj)) + pt]
#define RV(k, jj) rl[2 * ((k) + 5 * IX(g, i, jj)) + pt]
#define BW(k) g->bump[10 * (i - 1) + 2 * (k) + pt] /* u1w u2w u3w tw twp */
          if (g->wall == 3)
            for (int k = 1; k <= 3; ++k) RV(k, 1) = -(VR(k, 1) - BW(k - 1));
          else
            for (int k = 1; k <= 3; ++k) RV(k, 1) = -(VR(k, 1) - zero);
          if (g->wall == 1)
            RV(0, 1) = gc1 * VR(0, 1) + gc2 * VR(0, 2) + gc3 * VR(0, 3) + gc4 * VR(0, 4) + gc5 * VR(0, 5);
          if (g->wall == 2) RV(0, 1) = VR(0, 1) - two * VR(0, 2) + VR(0, 3);
          if (g->wall == 3) RV(0, 1) = VR(0, 1) - (4.0 * VR(0, 2) - 6.0 * VR(0, 3) + 4.0 * VR(0, 4) - VR(0, 5));
          if (g->wallt == 0) RV(4, 1) = g->wall == 3 ? -(VR(4, 1) - BW(3)) : zero;
          if (g->wallt == 1) {
            RV(4, 1) = gc1 * VR(4, 1) + gc2 * VR(4, 2) + gc3 * VR(4, 3) + gc4 * VR(4, 4) + gc5 * VR(4, 5);
            if (g->wall == 3) RV(4, 1) = RV(4, 1) - BW(4);
          }
#undef BW
        }
    }
    if (g->top == 0)
      for (int i = 1; i <= nx; ++i)
        for (int k = 0; k < 5; ++k) CRE(rl, k, g, i, ny) = zero, CIM(rl, k, g, i, ny) = zero;
    if (g->top == 1) /* src/rhsbc3d.f90:129-160: r = -(v - t) */
      for (int i = 1; i <= nx; ++i) {
        double t[10];
        a3_top_target(g, i, t);
        for (int k = 0; k < 10; ++k) rl[k + 10 * IX(g, i, ny)] = -(vl[k + 10 * IX(g, i, ny)] - t[k]);
      }
  }
  if (g->xper)
    for (int j = 1; j <= ny; ++j)
      for (int k = 0; k < 5; ++k) CRE(rl, k, g, nx, j) = zero, CIM(rl, k, g, nx, j) = zero;
}

/* src/resstat3d.f90:37-60: sqrt(sum |r|^2 / dtl^2 / (nx ny)); the saved
   totres of the reference is reset to zero at the end of each call
   (src/resstat3d.f90:98), so each call's sum starts from zero */
double a3_resstat(const A3Grid* g, const double* res, const double* dtl) {
  double totres = 0.0;
  for (int j = 1; j <= g->ny; ++j)
    for (int i = 1; i <= g->nx; ++i) {
      double s = 0.0;
      for (int k = 0; k < 5; ++k) {
        const double a = CRE(res, k, g, i, j), b = CIM(res, k, g, i, j);
        s = s + (a * a - b * (-b));
      }
      const double d = dtl[IX(g, i, j)];
      totres = totres + s / (d * d);
    }
  totres = sqrt(totres / (double)((long)g->nx * g->ny));
  return totres;
}

/* src/itrbc3d.f90:35-205 for the supported boundary conditions */
void a3_itrbc(const A3Grid* g, double* vl) {
  const int nx = g->nx, ny = g->ny;
  if (g->yper) {
    for (int i = 1; i <= nx; ++i)
      for (int k = 0; k < 10; ++k) vl[k + 10 * IX(g, i, ny)] = vl[k + 10 * IX(g, i, 1)];
  } else {
    if (g->navier) {
      for (int i = 1; i <= nx; ++i)
        for (int pt = 0; pt < 2; ++pt) {
#define BW(k) g->bump[10 * (i - 1) + 2 * (k) + pt] /* u1w u2w u3w tw twp */
          for (int k = 1; k <= 3; ++k) VR(k, 1) = g->wall == 3 ? BW(k - 1) : zero;
          if (g->wall == 1) VR(0, 1) = -(gc2 * VR(0, 2) + gc3 * VR(0, 3) + gc4 * VR(0, 4) + gc5 * VR(0, 5)) / gc1;
          if (g->wall == 2) VR(0, 1) = two * VR(0, 2) - VR(0, 3);
          if (g->wall == 3) VR(0, 1) = 4.0 * VR(0, 2) - 6.0 * VR(0, 3) + 4.0 * VR(0, 4) - VR(0, 5);
          if (g->wallt == 0) VR(4, 1) = g->wall == 3 ? BW(3) : zero;
          if (g->wallt == 1) {
            if (g->wall == 3)
              VR(4, 1) = (BW(4) - (gc2 * VR(4, 2) + gc3 * VR(4, 3) + gc4 * VR(4, 4) + gc5 * VR(4, 5))) / gc1;
            else
              VR(4, 1) = -(gc2 * VR(4, 2) + gc3 * VR(4, 3) + gc4 * VR(4, 4) + gc5 * VR(4, 5)) / gc1;
          }
#undef BW
        }
    }
    if (g->top == 0)
      for (int i = 1; i <= nx; ++i)
        for (int k = 0; k < 10; ++k) vl[k + 10 * IX(g, i, ny)] = zero;
    if (g->top == 1) /* src/itrbc3d.f90:145-196: v = t */
      for (int i = 1; i <= nx; ++i) a3_top_target(g, i, vl + 10 * IX(g, i, ny));
  }
  if (g->xper)
    for (int j = 1; j <= ny; ++j)
      for (int k = 0; k < 10; ++k) vl[k + 10 * IX(g, nx, j)] = vl[k + 10 * IX(g, 1, j)];
#undef VR
#undef RV
}

/* --------------------------------------------------------------------- LHS */

/* complex mat(k,a,b,i,j): (re, im) */
#define MRE(k, a, b, p) mat[2 * ((long)(k - 1) + 5 * (a - 1) + 25 * (b - 1) + 125 * (p))]
#define MIM(k, a, b, p) mat[2 * ((long)(k - 1) + 5 * (a - 1) + 25 * (b - 1) + 125 * (p)) + 1]

/* One block row of the xi/eta LHS: slot[k] and first/second-derivative
   coefficients per slot; `combined` selects the boundary-row form in which
   the diagonal slot is formed as dtl*(a X + rcalcd alfa (Dh + i Dhi))
   (src/lhsbt2f3d.f90:44-50) instead of adding the D terms afterwards
   (src/lhs1f3d.f90:60-124). */
static void lhs_row(const A3Grid* g, const A3Ops* o, const double* dtl, int dir, long p, const double ak[5],
                    const double bk[5], int combined, int damp, double* mat) {
  const double* X = (dir == 1 ? o->Ah : o->Bh) + 25 * p;
  const double* V = (dir == 1 ? o->Vh11 : o->Vh22) + 6 * p;
  const double* AB = o->ABhi + 6 * p;
  const double ab1 = AB[dir == 1 ? 0 : 2], ab2 = AB[dir == 1 ? 1 : 3];
  const double* Dh = o->Dh + 25 * p;
  const double* Dhi = o->Dhi + 25 * p;
  const double d = dtl[p], alfa = g->alfa;
  const int calcd = dir == 1;
  const double rcalcd = calcd ? one : zero;
  for (int k = 1; k <= 5; ++k) {
    for (int a = 1; a <= 5; ++a)
      for (int b = 1; b <= 5; ++b) {
        const double x = X[(a - 1) + 5 * (b - 1)];
        if (combined && k == 3) {
          const double re = ak[k - 1] * x + rcalcd * alfa * Dh[(a - 1) + 5 * (b - 1)];
          const double im = zero + rcalcd * alfa * Dhi[(a - 1) + 5 * (b - 1)];
          MRE(k, a, b, p) = d * re;
          MIM(k, a, b, p) = d * im;
        } else {
          MRE(k, a, b, p) = ak[k - 1] * d * x;
          MIM(k, a, b, p) = zero;
        }
      }
    /* \hat{A}_i / \hat{B}_i terms: c_k = i a_k */
    const double w = ak[k - 1] * d;
    MIM(k, 2, 4, p) = MIM(k, 2, 4, p) - w * ab1;
    MIM(k, 3, 4, p) = MIM(k, 3, 4, p) - w * ab2;
    MIM(k, 4, 2, p) = MIM(k, 4, 2, p) - w * ab1;
    MIM(k, 4, 3, p) = MIM(k, 4, 3, p) - w * ab2;
  }
  if (calcd && !combined)
    for (int a = 1; a <= 5; ++a)
      for (int b = 1; b <= 5; ++b) {
        MRE(3, a, b, p) = MRE(3, a, b, p) + alfa * d * Dh[(a - 1) + 5 * (b - 1)];
        MIM(3, a, b, p) = MIM(3, a, b, p) + alfa * d * Dhi[(a - 1) + 5 * (b - 1)];
      }
  for (int k = 1; k <= 5; ++k) {
    const double w = bk[k - 1] * d;
    MRE(k, 2, 2, p) = MRE(k, 2, 2, p) - w * V[0];
    MRE(k, 2, 3, p) = MRE(k, 2, 3, p) - w * V[4];
    MRE(k, 3, 2, p) = MRE(k, 3, 2, p) - w * V[5];
    MRE(k, 3, 3, p) = MRE(k, 3, 3, p) - w * V[1];
    MRE(k, 4, 4, p) = MRE(k, 4, 4, p) - w * V[2];
    MRE(k, 5, 5, p) = MRE(k, 5, 5, p) - w * V[3];
  }
  for (int a = 1; a <= 5; ++a) MRE(3, a, a, p) = MRE(3, a, a, p) + one;
  /* implicit damping: damp 0 the fourth-order band fb1..fb5
     (src/lhs1f3d.f90:168-200, src/lhs2f3d.f90:171-203), 2 the second-order
     rows 2 and ny-1 of lhsbt2f3D in slots 2..4 (src/lhsbt2f3d.f90:277-298),
     1 none (rows 1 and ny) */
  if (g->eps_e != zero && damp != 1) {
    const double fb[5] = {1.000000000000000E+00, -4.000000000000000E+00, 6.000000000000000E+00,
                          -4.000000000000000E+00, 1.000000000000000E+00}; /* src/stencil.f90:137-141 */
    const double sb[5] = {zero, -one, two, -one, zero};
    for (int k = 1; k <= 5; ++k) {
      if (damp == 2 && (k == 1 || k == 5)) continue;
      const double c = damp == 0 ? fb[k - 1] : sb[k - 1];
      for (int a = 1; a <= 5; ++a) MRE(k, a, a, p) = MRE(k, a, a, p) + alfa * d * g->eps_e * g->buff[p] * c;
    }
  }
  /* sponge of the eta LHS (calcd false there; src/lhs2f3d.f90:207-224,
     src/lhsbt2f3d.f90:147-167): mat(3,a,a) + alfa dtl spg, or
     alfa dtl (spg + spg2) for ispg >= 2 */
  if (!calcd && g->ispg >= 1) {
    const double sp = g->ispg == 1 ? g->spg[p] : g->spg[p] + g->spg2[p];
    for (int a = 1; a <= 5; ++a) MRE(3, a, a, p) = MRE(3, a, a, p) + alfa * d * sp;
  }
}

/* src/lhs1f3d.f90 / src/lhs2f3d.f90, then the boundary rows of
   src/lhsbt2f3d.f90 and the boundary conditions of src/lhsbc1f3d.f90 /
   src/lhsbc2f3d.f90 */
int a3_lhs(const A3Grid* g, const A3Ops* o, const double* dtl, int dir, double* mat) {
  const int nx = g->nx, ny = g->ny;
  const double h = dir == 1 ? g->dxi : g->deta, alfa = g->alfa;
  const double hinv = one / h, hsinv = one / (h * h);
  const int per = dir == 1 ? g->xper : g->yper;
  double ak[5], bk[5];
  /* interior rows: slots 1..5 <-> columns -2..+2 */
  const double gi[5] = {ga1, ga2, zero, ga3, ga4}, di[5] = {da1, da2, da3, da4, da5};
  for (int k = 0; k < 5; ++k) ak[k] = alfa * gi[k] / h, bk[k] = alfa * di[k] / (h * h);
  OMP_FOR
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) lhs_row(g, o, dtl, dir, IX(g, i, j), ak, bk, 0, 0, mat);
  if (!per) {
    if (dir == 1) return 1; /* non-periodic xi sweep: not supported by this oracle */
    /* boundary rows j = 1, 2, ny-1, ny (src/lhsbt2f3d.f90:36-600) */
    const double g1[5] = {gc1, gc2, gc3, gc4, gc5}, d1[5] = {dd1, dd2, dd3, dd4, dd5};
    const double g2[5] = {gb1, gb2, gb3, gb4, gb5}, d2[5] = {db1, db2, db3, db4, db5};
    const int s1[5] = {3, 4, 5, 1, 2}, s2[5] = {2, 3, 4, 5, 1};
    const int sN1[5] = {4, 3, 2, 1, 5}, sN[5] = {3, 2, 1, 5, 4}; /* slot of coefficient t (1..5) */
    for (int i = 1; i <= nx; ++i) {
      for (int t = 0; t < 5; ++t) ak[s1[t] - 1] = alfa * g1[t] * hinv, bk[s1[t] - 1] = alfa * d1[t] * hsinv;
      lhs_row(g, o, dtl, dir, IX(g, i, 1), ak, bk, 1, 1, mat);
      for (int t = 0; t < 5; ++t) ak[s2[t] - 1] = alfa * g2[t] * hinv, bk[s2[t] - 1] = alfa * d2[t] * hsinv;
      lhs_row(g, o, dtl, dir, IX(g, i, 2), ak, bk, 1, 2, mat);
      for (int t = 0; t < 5; ++t) ak[sN1[t] - 1] = -(alfa * g2[t] * hinv), bk[sN1[t] - 1] = alfa * d2[t] * hsinv;
      lhs_row(g, o, dtl, dir, IX(g, i, ny - 1), ak, bk, 1, 2, mat);
      for (int t = 0; t < 5; ++t) ak[sN[t] - 1] = -(alfa * g1[t] * hinv), bk[sN[t] - 1] = alfa * d1[t] * hsinv;
      lhs_row(g, o, dtl, dir, IX(g, i, ny), ak, bk, 1, 1, mat);
    }
  }
  /* boundary conditions of the wall (j = 1) and top (j = ny) rows */
  if (!g->yper && g->navier) {
    for (int i = 1; i <= nx; ++i) {
      const long p = IX(g, i, 1);
      if (dir == 1) { /* src/lhsbc1f3d.f90:24-45: identity rows */
        for (int a = 1; a <= 5; ++a)
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MRE(k, a, b, p) = zero, MIM(k, a, b, p) = zero;
        for (int a = 1; a <= 5; ++a) MRE(3, a, a, p) = one;
      } else { /* src/lhsbc2f3d.f90:24-66 */
        const int sl[5] = {3, 4, 5, 1, 2};
        const double gcs[5] = {gc1, gc2, gc3, gc4, gc5};
        if (g->wall == 1) {
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MRE(k, 1, b, p) = zero, MIM(k, 1, b, p) = zero;
          for (int t = 0; t < 5; ++t) MRE(sl[t], 1, 1, p) = -gcs[t];
        }
        if (g->wall == 3) { /* third-order extrapolation, src/lhsbc2f3d.f90:41-48 */
          const double ex3[5] = {-one, 4.0, -6.0, 4.0, -one};
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MRE(k, 1, b, p) = zero, MIM(k, 1, b, p) = zero;
          for (int t = 0; t < 5; ++t) MRE(sl[t], 1, 1, p) = ex3[t];
        }
        for (int a = 2; a <= 4; ++a)
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MRE(k, a, b, p) = zero, MIM(k, a, b, p) = zero;
        for (int a = 2; a <= 4; ++a) MRE(3, a, a, p) = one;
        if (g->wallt == 0 || g->wallt == 1) {
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MRE(k, 5, b, p) = zero, MIM(k, 5, b, p) = zero;
          if (g->wallt == 0) MRE(3, 5, 5, p) = one;
          else
            for (int t = 0; t < 5; ++t) MRE(sl[t], 5, 5, p) = -gcs[t];
        }
      }
    }
  }
  if (!g->yper && (g->top == 0 || g->top == 1))
    for (int i = 1; i <= nx; ++i) {
      const long p = IX(g, i, ny);
      for (int a = 1; a <= 5; ++a)
        for (int k = 1; k <= 5; ++k)
          for (int b = 1; b <= 5; ++b) MRE(k, a, b, p) = zero, MIM(k, a, b, p) = zero;
      for (int a = 1; a <= 5; ++a) MRE(3, a, a, p) = one;
    }
  return 0;
}

/* rtb3D, src/impdrv3d.f90:471-501: r = 4/3 vold - 1/3 v2old - v - 2/3 dtl r */
void a3_rtb(const A3Grid* g, double* r, const double* v, const double* vold, const double* v2old, const double* dtl) {
  const double onept33 = 1.3333333333333333333e+0, pt33 = 3.3333333333333333333e-1,
               pt66 = 6.6666666666666666666e-1;  /* src/global.f90:13-18 */
  OMP_FOR
  for (int j = 1; j <= g->ny; ++j)
    for (int i = 1; i <= g->nx; ++i)
      for (int k = 0; k < 10; ++k) {
        const long e = k + 10 * IX(g, i, j);
        r[e] = onept33 * vold[e] - pt33 * v2old[e] - v[e] - pt66 * dtl[IX(g, i, j)] * r[e];
      }
}

/* -------------------------------------------------------------------- step */

/* src/impdrv3d.f90:130-356 with impl = 1, iLHS = 1, USE_CPENTA1BC semantics
   for the xi sweep (the corrected boundary solve) */
double a3_step(const A3Grid* g, const A3Ops* o, const double* dtl, int niter, double* v, double* vold, double* r,
               double* matx, double* maty, double* perx, double* per2x, double* pery, double* per2y,
               int* factored) {
  const int nx = g->nx, ny = g->ny;
  const long n10 = 10L * nx * ny;
  double totres = 0.0;
  memcpy(vold, v, n10 * sizeof(double));
  a3_itrbc(g, v);
  for (int iter = 1; iter <= niter; ++iter) {
    a3_lrhs(g, o, v, r);
    a3_rbe(g, r, v, vold, dtl);
    a3_rhsbc(g, r, v);
    totres = a3_resstat(g, r, dtl);
    if (!*factored) {
      a3_lhs(g, o, dtl, 1, matx);
      if (g->xper) orc_cpenta_p(2, nx, ny, matx, r, perx, per2x, 0, ORC_COMPAT_PERIODIC_SLOT);
      else orc_cpenta_bc(2, nx, ny, matx, r, 0, 0);
      a3_lhs(g, o, dtl, 2, maty);
      if (g->yper) orc_cpenta_p(1, ny, nx, maty, r, pery, per2y, 0, ORC_COMPAT_PERIODIC_SLOT);
      else orc_cpenta_bc(1, ny, nx, maty, r, 0, 0);
      *factored = 1;
    }
    if (g->xper) orc_cpenta_p(2, nx, ny, matx, r, perx, per2x, 1, ORC_COMPAT_PERIODIC_SLOT);
    else orc_cpenta_bc(2, nx, ny, matx, r, 1, 0);
    if (g->yper) orc_cpenta_p(1, ny, nx, maty, r, pery, per2y, 1, ORC_COMPAT_PERIODIC_SLOT);
    else orc_cpenta_bc(1, ny, nx, maty, r, 1, 0);
    OMP_FOR
    for (long e = 0; e < n10; ++e) v[e] = v[e] + r[e];
    a3_itrbc(g, v);
  }
  return totres;
}

/* One step of the time schemes of src/impdrv3d.f90:130-356 (iLHS = 1):
   impl 1 backward Euler (alfa = g->alfa); impl 2 two-step backward, which is
   backward Euler while lstep = 0 and then rtb3D with alfa = 2/3, the LHS
   factored again at the first step with lstep = 1 (:134-143,179-193,228-231);
   impl 3 midpoint, the RHS operator at (v + vold)/2 with rbe3D and alfa =
   1/2 (:195-199).  vold and v2old carry over between steps; w is scratch;
   *alfa_fac is the alfa of the current factors (any value outside
   {1, 2/3, 1/2, g->alfa} before the first step). */
double a3_step_impl(const A3Grid* g, const A3Ops* o, const double* dtl, int niter, int impl, int lstep, double* v,
                    double* vold, double* v2old, double* w, double* r, double* matx, double* maty, double* perx,
                    double* per2x, double* pery, double* per2y, double* alfa_fac) {
  const int nx = g->nx, ny = g->ny;
  const long n10 = 10L * nx * ny;
  const double pt66 = 6.6666666666666666666e-1, pt5 = 0.5;
  A3Grid gl = *g;
  double totres = 0.0;
  if (impl == 2 && lstep > 0) memcpy(v2old, vold, n10 * sizeof(double));
  memcpy(vold, v, n10 * sizeof(double));
  a3_itrbc(g, v);
  for (int iter = 1; iter <= niter; ++iter) {
    const int rtb = impl == 2 && lstep > 0;
    gl.alfa = impl == 3 ? pt5 : rtb ? pt66 : (impl == 2 ? 1.0 : g->alfa);
    if (impl == 3) {
      OMP_FOR
      for (long e = 0; e < n10; ++e) w[e] = pt5 * (v[e] + vold[e]);
      a3_lrhs(&gl, o, w, r);
    } else {
      a3_lrhs(&gl, o, v, r);
    }
    if (rtb) a3_rtb(&gl, r, v, vold, v2old, dtl);
    else a3_rbe(&gl, r, v, vold, dtl);
    a3_rhsbc(&gl, r, v);
    totres = a3_resstat(&gl, r, dtl);
    if (*alfa_fac != gl.alfa) {
      a3_lhs(&gl, o, dtl, 1, matx);
      if (gl.xper) orc_cpenta_p(2, nx, ny, matx, r, perx, per2x, 0, ORC_COMPAT_PERIODIC_SLOT);
      else orc_cpenta_bc(2, nx, ny, matx, r, 0, 0);
      a3_lhs(&gl, o, dtl, 2, maty);
      if (gl.yper) orc_cpenta_p(1, ny, nx, maty, r, pery, per2y, 0, ORC_COMPAT_PERIODIC_SLOT);
      else orc_cpenta_bc(1, ny, nx, maty, r, 0, 0);
      *alfa_fac = gl.alfa;
    }
    if (gl.xper) orc_cpenta_p(2, nx, ny, matx, r, perx, per2x, 1, ORC_COMPAT_PERIODIC_SLOT);
    else orc_cpenta_bc(2, nx, ny, matx, r, 1, 0);
    if (gl.yper) orc_cpenta_p(1, ny, nx, maty, r, pery, per2y, 1, ORC_COMPAT_PERIODIC_SLOT);
    else orc_cpenta_bc(1, ny, nx, maty, r, 1, 0);
    OMP_FOR
    for (long e = 0; e < n10; ++e) v[e] = v[e] + r[e];
    a3_itrbc(g, v);
  }
  return totres;
}
