/*
 * CPU oracle for the nonlinear two-dimensional implicit ADI step.
 * TEST INFRASTRUCTURE ONLY (see impdrv2d_oracle.h for scope and citations).
 * Built with -ffp-contract=off: every expression is evaluated left to right
 * with separate roundings, as the reference Fortran on x86-64; x**2 is x*x
 * and x**y (real y) is pow, as gfortran compiles them.
 */
#include "impdrv2d_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle_common.h"
#include "penta_oracle.h"

#define G(a2) (&(a2)->g)

/* ---------------------------------------------------------------- genmtrx */

/* src/genmtrx.f90 with linear = 0, general = true, mattyp = 0, idamp = 0,
   kzl = 0: the nonlinear RHS and the operators of the LHS. */
/* smoother, src/smoother.f90 without symmetry planes: rl += eps_e buff D(vl)
   over the nc interleaved components of each point, the eta pass first (rows
   2 and ny-1 second order, 3 and ny-2 fourth order, 4..ny-3 sixth order),
   then the xi pass with the same pattern over i (no periodic wrap). */
static void a2_smoother(const A3Grid* g, int nc, double* rl, const double* vl) {
  const int nx = g->nx, ny = g->ny;
  const double fa1 = -1.666666666666667E-01, fa2 = 2.000000000000000E+00, fa3 = -6.500000000000000E+00,
               fa4 = 9.333333333333333E+00, fa5 = -6.500000000000000E+00, fa6 = 2.000000000000000E+00,
               fa7 = -1.666666666666667E-01; /* src/stencil.f90:145-151 */
  for (int pass = 0; pass < 2; ++pass) {
    const int n = pass == 0 ? ny : nx;
    for (int l = 1; l <= (pass == 0 ? nx : ny); ++l)
      for (int c = 2; c <= n - 1; ++c) {
        const int i = pass == 0 ? l : c, j = pass == 0 ? c : l;
        const long st = pass == 0 ? (long)nc * nx : nc;
        const long p = IX(g, i, j);
        const double eb = g->eps_e * g->buff[p];
        for (int k = 0; k < nc; ++k) {
          const double* V = vl + k + nc * p;
#define VS(d) V[(long)(d) * st]
          double s;
          if (c == 2 || c == n - 1) s = -1.0 * VS(-1) + 2.0 * VS(0) - 1.0 * VS(1);
          else if (c == 3 || c == n - 2) s = VS(-2) - 4.0 * VS(-1) + 6.0 * VS(0) - 4.0 * VS(1) + 1.0 * VS(2);
          else s = fa1 * VS(-3) + fa2 * VS(-2) + fa3 * VS(-1) + fa4 * VS(0) + fa5 * VS(1) + fa6 * VS(2) + fa7 * VS(3);
#undef VS
          rl[k + nc * p] = rl[k + nc * p] + eb * s;
        }
      }
  }
}

int a2_genmtrx(const A2Grid* a2, const double* vl, A3Ops* o, double* rl) {
  const A3Grid* g = G(a2);
  const int nx = g->nx, ny = g->ny;
  const long np = (long)nx * ny;
  double* g1v = (double*)calloc(5 * np, sizeof(double));
  double* g2v = (double*)calloc(5 * np, sizeof(double));
  double* g11v = (double*)calloc(5 * np, sizeof(double));
  double* g12v = (double*)calloc(5 * np, sizeof(double));
  double* g22v = (double*)calloc(5 * np, sizeof(double));
  if (!g1v || !g2v || !g11v || !g12v || !g22v) return 3;
  a3_deriv1(g, 5, vl, g1v, g2v);                /* genmtrx.f90:72 */
  a3_deriv2(g, 5, vl, g1v, g11v, g12v, g22v);   /* genmtrx.f90:77 */
  if (g->navier && (g->wallt == 1 || g->wallt == 2))  /* gradbc.f90:15 */
    for (int i = 1; i <= nx; ++i) FV(g2v, 5, 4, g, i, 1) = zero;
  const double gamma = g->gamma, gamma1 = g->gamma1, Ma = g->Ma, Re = g->Re, Pr = g->Pr;
  OMP_FOR
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const long p = IX(g, i, j);
      const double m1 = g->m1[p], m2 = g->m2[p], n1 = g->n1[p], n2 = g->n2[p];
      const double m11 = g->m11[p], m12 = g->m12[p], m22 = g->m22[p], n11 = g->n11[p], n12 = g->n12[p],
                   n22 = g->n22[p];
      const double m1m1 = m1 * m1, m1m2 = m1 * m2, m2m2 = m2 * m2, n1n1 = n1 * n1, n1n2 = n1 * n2, n2n2 = n2 * n2;
      const double m1n1 = m1 * n1, m1n2 = m1 * n2, m2n1 = m2 * n1, m2n2 = m2 * n2;
      double g1vl[5], g2vl[5], g11vl[5], g12vl[5], g22vl[5];
      for (int k = 0; k < 5; ++k) { /* genmtrx.f90:116-136 */
        const double a1 = FV(g1v, 5, k, g, i, j), b1 = FV(g2v, 5, k, g, i, j);
        const double a11 = FV(g11v, 5, k, g, i, j), a12 = FV(g12v, 5, k, g, i, j), a22 = FV(g22v, 5, k, g, i, j);
        g11vl[k] = a11 * m1m1 + two * a12 * m1n1 + a22 * n1n1 + a1 * m11 + b1 * n11;
        g12vl[k] = a11 * m1m2 + a12 * (m1n2 + m2n1) + a22 * n1n2 + a1 * m12 + b1 * n12;
        g22vl[k] = a11 * m2m2 + two * a12 * m2n2 + a22 * n2n2 + a1 * m22 + b1 * n22;
        g1vl[k] = a1 * m1 + b1 * n1;
        g2vl[k] = a1 * m2 + b1 * n2;
      }
      /* genmtrx.f90:152-228 */
      double fact = one / (gamma * (Ma * Ma));
      double fact1 = one / Re;
      double fact2 = gamma / (Pr * Re);
      double fact3 = gamma * gamma1 * (Ma * Ma) / Re;
      /* u3 = v(4) enters no term of the two-dimensional equations */
      const double rho = FV(vl, 5, 0, g, i, j), u1 = FV(vl, 5, 1, g, i, j), u2 = FV(vl, 5, 2, g, i, j),
                   t = FV(vl, 5, 4, g, i, j);
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
      double gp[3];
      gp[0] = fact * (grho[0] * t + rho * gt[0]);
      gp[1] = fact * (grho[1] * t + rho * gt[1]);
      gp[2] = fact * (grho[2] * t + rho * gt[2]);
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
      /* nonlinear RHS, genmtrx.f90:282-312 */
      double* R = rl + 5 * p;
      R[0] = rho * divu + grho[0] * u1 + grho[1] * u2;
      R[1] = u1 * gu[0][0] + u2 * gu[0][1] + rhoinv * gp[0] -
             fact1 * (g1lm * divu + lm * g1divu + two * (g1mu * S[0][0] + g2mu * S[0][1] + mu * S1jj)) * rhoinv;
      R[2] = u1 * gu[1][0] + u2 * gu[1][1] + rhoinv * gp[1] -
             fact1 * (g2lm * divu + lm * g2divu + two * (g1mu * S[1][0] + g2mu * S[1][1] + mu * S2jj)) * rhoinv;
      R[3] = u1 * gu[2][0] + u2 * gu[2][1] - fact1 * (two * (g1mu * S[2][0] + g2mu * S[2][1] + mu * S3jj)) * rhoinv;
      R[4] = u1 * gt[0] + u2 * gt[1] + gamma1 * t * divu -
             rhoinv * (fact2 * (g1con * gt[0] + g2con * gt[1] + con * Lapt) +
                       fact3 * (lm * (divu * divu) +
                                two * mu *
                                    (S[0][0] * S[0][0] + S[0][1] * S[0][1] + S[0][2] * S[0][2] + S[1][0] * S[1][0] +
                                     S[1][1] * S[1][1] + S[1][2] * S[1][2] + S[2][0] * S[2][0] + S[2][1] * S[2][1])));
      double A[5][5] = {{0}}, B[5][5] = {{0}}, D[5][5] = {{0}}, Vij[4];
      double gmsinv;
      /* A, genmtrx.f90:458-503 */
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
      /* B, genmtrx.f90:525-575 */
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
      /* Vij, genmtrx.f90:586-600 */
      fact1 = one / Re;
      fact2 = gamma / (Pr * Re);
      Vij[0] = fact1 * rhoinv * (lm + two * mu);
      Vij[1] = fact1 * rhoinv * mu;
      Vij[2] = fact2 * rhoinv * con;
      Vij[3] = fact1 * rhoinv * (lm + mu);
      /* \hat{A}, \hat{B}, genmtrx.f90:602-700 */
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
      /* D, genmtrx.f90:702-836 (linear = 0) */
      D[0][0] = divu; D[0][1] = grho[0]; D[0][2] = grho[1]; D[0][3] = grho[2]; D[0][4] = zero;
      fact1 = rhoinv / Re;
      gmsinv = one / (gamma * (Ma * Ma));
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
      fact2 = gamma * gamma1 * (Ma * Ma) * rhoinv / Re;
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
      for (int a = 0; a < 5; ++a)
        for (int b = 0; b < 5; ++b) o->Dh[a + 5 * b + 25 * p] = D[a][b];
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
    }
  free(g1v); free(g2v); free(g11v); free(g12v); free(g22v);
  if (rl && g->ispg == 2) /* the sponge towards the free stream, genmtrx.f90:436-446 */
    for (long p = 0; p < np; ++p) {
      const double sp = g->spg[p] + g->spg2[p];
      rl[0 + 5 * p] = rl[0 + 5 * p] + sp * (vl[0 + 5 * p] - one);
      for (int k = 1; k <= 3; ++k) rl[k + 5 * p] = rl[k + 5 * p] + sp * (vl[k + 5 * p]);
      rl[4 + 5 * p] = rl[4 + 5 * p] + sp * (vl[4 + 5 * p] - one);
    }
  if (rl && g->eps_e != zero) a2_smoother(g, 5, rl, vl); /* genmtrx.f90:1008 */
  return 0;
}

/* rbe, src/impdrv.f90:482-505: r = vold - v - dtl r */
void a2_rbe(const A2Grid* a2, double* r, const double* v, const double* vold, const double* dtl) {
  const A3Grid* g = G(a2);
  for (int j = 1; j <= g->ny; ++j)
    for (int i = 1; i <= g->nx; ++i)
      for (int k = 0; k < 5; ++k) {
        const long e = k + 5 * IX(g, i, j);
        r[e] = vold[e] - v[e] - dtl[IX(g, i, j)] * r[e];
      }
}

/* ------------------------------------------------------- Riemann far field */

/* vn, vt, extrapolated state and the invariants of boundary node i,
   src/reimann.f90:60-72 (shared by Reimann, ReimannRHS, ReimannLHS) */
typedef struct {
  double vn, vint[5], R1, R2, rho, p, vt_in;
  int inflow;
} RmState;

static RmState rm_state(const A2Grid* a2, int i, const double* vb, const double* vb1, const double* vb2) {
  const A3Grid* g = G(a2);
  const int nx = g->nx;
  const double bn1 = a2->bnt[i - 1], bn2 = a2->bnt[nx + i - 1];
  const double gamma = g->gamma, gamma1 = g->gamma1, Ma = g->Ma;
  RmState s;
  s.vn = bn1 * vb[1] + bn2 * vb[2];
  for (int k = 0; k < 5; ++k) s.vint[k] = two * vb1[k] - vb2[k];
  const double cb = sqrt(a2->tbt[i - 1]) / Ma;
  s.R1 = bn1 * a2->ubt[i - 1] + bn2 * a2->vbt[i - 1] - two * cb / gamma1;
  const double c = sqrt(s.vint[4]) / Ma;
  s.R2 = bn1 * s.vint[1] + bn2 * s.vint[2] + two * c / gamma1;
  s.inflow = s.vn <= zero;
  if (s.inflow) {
    s.rho = a2->rhobt[i - 1];
    s.p = a2->rhobt[i - 1] * a2->tbt[i - 1] / (gamma * (Ma * Ma));  /* pbt, src/potential.f90:29 */
    s.vt_in = bn2 * a2->ubt[i - 1] - bn1 * a2->vbt[i - 1];
  } else {
    s.rho = s.vint[0];
    s.p = s.vint[0] * s.vint[4] / (gamma * (Ma * Ma));
    s.vt_in = bn2 * s.vint[1] - bn1 * s.vint[2];
  }
  return s;
}

/* the boundary state the invariants give, src/reimann.f90:104-150 */
static void rm_values(const A2Grid* a2, int i, const RmState* s, double out[5]) {
  const A3Grid* g = G(a2);
  const int nx = g->nx;
  const double bn1 = a2->bnt[i - 1], bn2 = a2->bnt[nx + i - 1];
  const double gamma = g->gamma, gamma1 = g->gamma1, Ma = g->Ma;
  const double vn = pt5 * (s->R1 + s->R2), vt = s->vt_in;
  const double gq = gamma1 / four, dR = s->R2 - s->R1;
  out[0] = pow(pow(s->rho, gamma) / (gamma * s->p) * (gq * gq) * (dR * dR), one / gamma1);
  out[1] = (-(bn1 * vn) - bn2 * vt) / (-(bn1 * bn1) - bn2 * bn2);
  out[2] = (-(bn2 * vn) + bn1 * vt) / (-(bn1 * bn1) - bn2 * bn2);
  out[3] = s->inflow ? a2->wbt[i - 1] : s->vint[3];
  const double q = Ma * gamma1 / four * dR;
  out[4] = q * q;
}

/* ------------------------------------------------------------------ BCs */

/* src/rhsbc.f90:256-370 (nonlinear branch) */
void a2_rhsbc(const A2Grid* a2, double* rl, const double* vl) {
  const A3Grid* g = G(a2);
  const int nx = g->nx, ny = g->ny;
#define VR(k, ii, jj) vl[(k) + 5 * IX(g, ii, jj)]
#define RV(k, ii, jj) rl[(k) + 5 * IX(g, ii, jj)]
  if (g->yper) {
    for (int i = 1; i <= nx; ++i)
      for (int k = 0; k < 5; ++k) RV(k, i, ny) = zero;
  } else {
    if (g->navier) {
      for (int i = 1; i <= nx; ++i) {
        for (int k = 1; k <= 3; ++k) RV(k, i, 1) = zero;
        if (g->wall == 1)
          RV(0, i, 1) = gc1 * VR(0, i, 1) + gc2 * VR(0, i, 2) + gc3 * VR(0, i, 3) + gc4 * VR(0, i, 4) +
                        gc5 * VR(0, i, 5);
        if (g->wall == 3)
          RV(0, i, 1) = VR(0, i, 1) - (4.0 * VR(0, i, 2) - 6.0 * VR(0, i, 3) + 4.0 * VR(0, i, 4) - VR(0, i, 5));
        if (g->wallt == 0) {
          const double tt = tan(a2->theta);
          RV(4, i, 1) = VR(4, i, 1) - (one + pt5 * g->gamma1 * (g->Ma * g->Ma) * (one + tt * tt) * sqrt(g->Pr));
        }
        if (g->wallt == 1)
          RV(4, i, 1) = gc1 * VR(4, i, 1) + gc2 * VR(4, i, 2) + gc3 * VR(4, i, 3) + gc4 * VR(4, i, 4) +
                        gc5 * VR(4, i, 5);
      }
    }
    if (g->Ma > one) {
      for (int i = 1; i <= nx; ++i)
        for (int k = 0; k < 5; ++k) RV(k, i, ny) = zero;
    } else if (g->top == 0) {
      /* ReimannRHS, src/reimann.f90:162-236: r = v - boundary state */
      for (int i = 1; i <= nx; ++i) {
        const RmState s = rm_state(a2, i, &VR(0, i, ny), &VR(0, i, ny - 1), &VR(0, i, ny - 2));
        double b[5];
        rm_values(a2, i, &s, b);
        for (int k = 0; k < 5; ++k) RV(k, i, ny) = VR(k, i, ny) - b[k];
      }
    }
  }
  if (g->xper)
    for (int j = 1; j <= ny; ++j)
      for (int k = 0; k < 5; ++k) RV(k, nx, j) = zero;
}

/* src/itrbc.f90:623-760 (nonlinear branch) */
void a2_itrbc(const A2Grid* a2, double* vl) {
  const A3Grid* g = G(a2);
  const int nx = g->nx, ny = g->ny;
  if (g->yper) {
    for (int i = 1; i <= nx; ++i)
      for (int k = 0; k < 5; ++k) VR(k, i, ny) = VR(k, i, 1);
  } else {
    if (g->navier) {
      for (int i = 1; i <= nx; ++i) {
        for (int k = 1; k <= 3; ++k) VR(k, i, 1) = zero;
        if (g->wall == 1) VR(0, i, 1) = -(gc2 * VR(0, i, 2) + gc3 * VR(0, i, 3) + gc4 * VR(0, i, 4) + gc5 * VR(0, i, 5)) / gc1;
        if (g->wall == 3) VR(0, i, 1) = 4.0 * VR(0, i, 2) - 6.0 * VR(0, i, 3) + 4.0 * VR(0, i, 4) - VR(0, i, 5);
        if (g->wallt == 0) {
          const double tt = tan(a2->theta);
          VR(4, i, 1) = one + pt5 * g->gamma1 * (g->Ma * g->Ma) * (one + tt * tt) * sqrt(g->Pr);
        }
        if (g->wallt == 1)
          VR(4, i, 1) = -(gc2 * VR(4, i, 2) + gc3 * VR(4, i, 3) + gc4 * VR(4, i, 4) + gc5 * VR(4, i, 5)) / gc1;
      }
    }
    if (g->Ma > one) {
      for (int i = 1; i <= nx; ++i) {
        VR(0, i, ny) = one; VR(1, i, ny) = one; VR(2, i, ny) = zero; VR(3, i, ny) = zero; VR(4, i, ny) = one;
      }
    } else if (g->top == 0) {
      /* Reimann, src/reimann.f90:2-156 */
      for (int i = 1; i <= nx; ++i) {
        const RmState s = rm_state(a2, i, &VR(0, i, ny), &VR(0, i, ny - 1), &VR(0, i, ny - 2));
        double b[5];
        rm_values(a2, i, &s, b);
        for (int k = 0; k < 5; ++k) VR(k, i, ny) = b[k];
      }
    } else if (g->top == 3) {
      /* the held quiescent top, src/itrbc.f90 (nonlinear, top = 3) */
      for (int i = 1; i <= nx; ++i) {
        VR(0, i, ny) = one; VR(1, i, ny) = zero; VR(2, i, ny) = zero; VR(3, i, ny) = zero; VR(4, i, ny) = one;
      }
    }
  }
  if (g->xper)
    for (int j = 1; j <= ny; ++j)
      for (int k = 0; k < 5; ++k) VR(k, nx, j) = VR(k, 1, j);
#undef VR
#undef RV
}

/* src/resstat.f90:37-60 (its saved totres is reset at the end of each call) */
double a2_resstat(const A2Grid* a2, const double* res, const double* dtl) {
  const A3Grid* g = G(a2);
  double totres = 0.0;
  for (int j = 1; j <= g->ny; ++j)
    for (int i = 1; i <= g->nx; ++i) {
      const double* r = res + 5 * IX(g, i, j);
      const double d = dtl[IX(g, i, j)];
      const double resnod = (r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3] + r[4] * r[4]) / (d * d);
      totres = totres + resnod;
    }
  totres = sqrt(totres / (double)((long)g->nx * g->ny));
  return totres;
}

/* -------------------------------------------------------------------- LHS */

#define MT(k, a, b, p) mat[(long)(k - 1) + 5 * (a - 1) + 25 * (b - 1) + 125 * (p)]

/* A 5x5 block in some storage: entry (a, b) at p[(a-1) sa + (b-1) sb]. */
typedef struct { double* p; long sa, sb; } Blk;
#define RB(k, a, b) (rb[(k) - 1].p[(long)((a) - 1) * rb[(k) - 1].sa + (long)((b) - 1) * rb[(k) - 1].sb])

/* ReimannLHS, src/reimann.f90:238-401: the blocks of row ny at columns
   ny-2, ny-1, ny (rb[0], rb[1], rb[2]); entries not set are left as they are */
static void rm_lhs_blk(const A2Grid* a2, int i, const double* vb, const double* vb1, const double* vb2,
                       const Blk rb[3]) {
  const A3Grid* g = G(a2);
  const int nx = g->nx;
  const double bn1 = a2->bnt[i - 1], bn2 = a2->bnt[nx + i - 1];
  const double gamma = g->gamma, gamma1 = g->gamma1, Ma = g->Ma;
  const RmState s = rm_state(a2, i, vb, vb1, vb2);
  const double dR = s.R2 - s.R1, gq = gamma1 / four;
  const double sq = sqrt(s.vint[4]);
  const double bb = bn1 * bn1 + bn2 * bn2;
  double fact, fact1, fact2;
  /* m2 = 2 F (slot 2), m3 = -F (slot 1) for the row's coefficients F */
#define PUT(a, b, F) (RB(2, a, b) = two * (F), RB(1, a, b) = -(F))
  if (s.inflow) {
    fact = pow(pow(s.rho, gamma) / (gamma * s.p) * (gq * gq), one / gamma1) * two / gamma1 *
           pow(dR, (two - gamma1) / gamma1);
    RB(3, 1, 1) = -one;
    PUT(1, 2, fact * bn1);
    PUT(1, 3, fact * bn2);
    PUT(1, 5, fact / (gamma1 * Ma * sq));
    fact = pt5 * bn1 / bb;
    RB(3, 2, 2) = -one;
    PUT(2, 2, fact * bn1);
    PUT(2, 3, fact * bn2);
    PUT(2, 5, fact / (gamma1 * Ma * sq));
    fact = pt5 * bn2 / bb;
    RB(3, 3, 3) = -one;
    PUT(3, 2, fact * bn1);
    PUT(3, 3, fact * bn2);
    PUT(3, 5, fact / (gamma1 * Ma * sq));
    RB(3, 4, 4) = -one;
    fact = (Ma * gamma1 / four) * (Ma * gamma1 / four) * two * dR;
    RB(3, 5, 5) = -one;
    PUT(5, 2, fact * bn1);
    PUT(5, 3, fact * bn2);
    PUT(5, 5, fact / (gamma1 * Ma * sq));
  } else {
    const double rg = pow(s.rho, gamma) / (gamma * s.p);
    fact1 = pow(rg, one / gamma1) * pow(gq, two / gamma1) * (two / gamma1) * pow(dR, (two - gamma1) / gamma1);
    fact2 = pow(gq * dR, two / gamma1) * one / (gamma * gamma1) * pow(rg, (two - gamma) / gamma1);
    const double fr = fact2 * pow(s.rho, gamma + 1) / (gamma * (Ma * Ma) * (s.p * s.p));
    RB(3, 1, 1) = -one;
    PUT(1, 2, fact1 * bn1 + gamma1 * pow(s.rho, gamma1) / s.p);
    PUT(1, 3, fact1 * bn2);
    PUT(1, 5, fact1 / (gamma1 * Ma * sq) - fr);
    fact1 = pt5 * bn1 / bb;
    fact2 = bn2 / bb;
    RB(3, 2, 2) = -one;
    PUT(2, 2, fact1 * bn1 + fact2 * bn2);
    PUT(2, 3, fact1 * bn2 - fact2 * bn1);
    PUT(2, 5, fact1 / (gamma1 * Ma * sq));
    fact1 = pt5 * bn2 / bb;
    fact2 = bn1 / bb;
    RB(3, 3, 3) = -one;
    PUT(3, 2, fact1 * bn1 - fact2 * bn2);
    PUT(3, 3, fact1 * bn2 + fact2 * bn1);
    PUT(3, 5, fact1 / (gamma1 * Ma * sq));
    RB(3, 4, 4) = -one;
    RB(2, 4, 4) = two;
    RB(1, 4, 4) = -one;
    fact = (Ma * gamma1 / four) * (Ma * gamma1 / four) * two * dR;
    RB(3, 5, 5) = -one;
    PUT(5, 2, fact * bn1);
    PUT(5, 3, fact * bn2);
    PUT(5, 5, fact / (gamma1 * Ma * sq));
  }
#undef PUT
}

/* the same into slots 3, 2, 1 (columns ny, ny-1, ny-2) of row ny's
   pentadiagonal record */
static void rm_lhs(const A2Grid* a2, int i, const double* vb, const double* vb1, const double* vb2, double* mat,
                   long p) {
  const Blk rb[3] = {{&MT(1, 1, 1, p), 5, 25}, {&MT(2, 1, 1, p), 5, 25}, {&MT(3, 1, 1, p), 5, 25}};
  rm_lhs_blk(a2, i, vb, vb1, vb2, rb);
}

/* lhs1f / lhs2f (src/lhsf.f90:7-162, 164-329), the eta boundary rows
   (src/lhsbt2f.f90:28-400), and the boundary conditions
   (src/lhsbc1f.f90:230-605, src/lhsbc2f.f90:193-330). */
int a2_lhs(const A2Grid* a2, const A3Ops* o, const double* dtl, const double* vl, int dir, double* mat) {
  const A3Grid* g = G(a2);
  const int nx = g->nx, ny = g->ny;
  const double alfa = g->alfa;
  if (dir == 1 && !g->xper) return 1;
  if (g->yper) return 1;
  const double h = dir == 1 ? g->dxi : g->deta;
  const double ak[5] = {alfa * ga1 / h, alfa * ga2 / h, alfa * zero / h, alfa * ga3 / h, alfa * ga4 / h};
  const double bk[5] = {alfa * da1 / (h * h), alfa * da2 / (h * h), alfa * da3 / (h * h), alfa * da4 / (h * h),
                        alfa * da5 / (h * h)};
  OMP_FOR
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const long p = IX(g, i, j);
      const double d = dtl[p];
      const double* X = (dir == 1 ? o->Ah : o->Bh) + 25 * p;
      const double* V = (dir == 1 ? o->Vh11 : o->Vh22) + 6 * p;
      for (int a = 1; a <= 5; ++a)
        for (int b = 1; b <= 5; ++b)
          for (int k = 1; k <= 5; ++k) MT(k, a, b, p) = ak[k - 1] * d * X[(a - 1) + 5 * (b - 1)];
      if (dir == 1)
        for (int a = 1; a <= 5; ++a)
          for (int b = 1; b <= 5; ++b)
            MT(3, a, b, p) = MT(3, a, b, p) + alfa * d * o->Dh[(a - 1) + 5 * (b - 1) + 25 * p];
      for (int k = 1; k <= 5; ++k) {
        MT(k, 2, 2, p) = MT(k, 2, 2, p) - bk[k - 1] * d * V[0];
        MT(k, 2, 3, p) = MT(k, 2, 3, p) - bk[k - 1] * d * V[4];
        MT(k, 3, 2, p) = MT(k, 3, 2, p) - bk[k - 1] * d * V[5];
        MT(k, 3, 3, p) = MT(k, 3, 3, p) - bk[k - 1] * d * V[1];
        MT(k, 4, 4, p) = MT(k, 4, 4, p) - bk[k - 1] * d * V[2];
        MT(k, 5, 5, p) = MT(k, 5, 5, p) - bk[k - 1] * d * V[3];
      }
      for (int a = 1; a <= 5; ++a) MT(3, a, a, p) = MT(3, a, a, p) + one;
      /* implicit damping (src/lhsf.f90:113-145, 262-294) and, in the eta
         LHS, the sponge (src/lhsf.f90:296-312) */
      if (g->eps_e != zero) {
        const double fb[5] = {1.000000000000000E+00, -4.000000000000000E+00, 6.000000000000000E+00,
                              -4.000000000000000E+00, 1.000000000000000E+00};
        for (int k = 1; k <= 5; ++k)
          for (int a = 1; a <= 5; ++a) MT(k, a, a, p) = MT(k, a, a, p) + alfa * d * g->eps_e * g->buff[p] * fb[k - 1];
      }
      if (dir == 2 && g->ispg == 2)
        for (int a = 1; a <= 5; ++a) MT(3, a, a, p) = MT(3, a, a, p) + alfa * d * (g->spg[p] + g->spg2[p]);
    }
  if (dir == 2) {
    /* rows 1, 2, ny-1, ny: coefficient t at slot s[t], src/lhsbt2f.f90 */
    const double detainv = one / g->deta, detasinv = one / (g->deta * g->deta);
    const double gcs[5] = {gc1, gc2, gc3, gc4, gc5}, gbs[5] = {gb1, gb2, gb3, gb4, gb5};
    const double dds[5] = {dd1, dd2, dd3, dd4, dd5}, dbs[5] = {db1, db2, db3, db4, db5};
    const int s1[5] = {3, 4, 5, 1, 2}, s2[5] = {2, 3, 4, 5, 1}, sN1[5] = {4, 3, 2, 1, 5}, sN[5] = {3, 2, 1, 5, 4};
    for (int i = 1; i <= nx; ++i)
      for (int r = 0; r < 4; ++r) {
        const int j = r == 0 ? 1 : r == 1 ? 2 : r == 2 ? ny - 1 : ny;
        const int* sl = r == 0 ? s1 : r == 1 ? s2 : r == 2 ? sN1 : sN;
        const double* gcf = (r == 0 || r == 3) ? gcs : gbs;
        const double* dcf = (r == 0 || r == 3) ? dds : dbs;
        const double sg = r >= 2 ? -one : one;
        const long p = IX(g, i, j);
        const double d = dtl[p];
        const double* X = o->Bh + 25 * p;
        const double* V = o->Vh22 + 6 * p;
        for (int a = 1; a <= 5; ++a)
          for (int b = 1; b <= 5; ++b)
            for (int t = 0; t < 5; ++t) {
              const double v = alfa * d * gcf[t] * detainv * X[(a - 1) + 5 * (b - 1)];
              MT(sl[t], a, b, p) = sg < zero ? -v : v;
            }
        for (int t = 0; t < 5; ++t) {
          const int k = sl[t];
          const double w = alfa * d * dcf[t] * detasinv;
          MT(k, 2, 2, p) = MT(k, 2, 2, p) - w * V[0];
          MT(k, 2, 3, p) = MT(k, 2, 3, p) - w * V[4];
          MT(k, 3, 2, p) = MT(k, 3, 2, p) - w * V[5];
          MT(k, 3, 3, p) = MT(k, 3, 3, p) - w * V[1];
          MT(k, 4, 4, p) = MT(k, 4, 4, p) - w * V[2];
          MT(k, 5, 5, p) = MT(k, 5, 5, p) - w * V[3];
        }
        for (int a = 1; a <= 5; ++a) MT(3, a, a, p) = MT(3, a, a, p) + one;
        /* sponge: lhsbt2f declares spgl(ny,nx) for the (nx,ny) array it is
           given, so row j of line i reads element (j-1) + (i-1) ny of it
           (src/lhsbt2f.f90:18,94-108) */
        if (g->ispg == 2) {
          const long q = (long)(j - 1) + (long)(i - 1) * ny;
          for (int a = 1; a <= 5; ++a) MT(3, a, a, p) = MT(3, a, a, p) + alfa * d * (g->spg[q] + g->spg2[q]);
        }
        /* damping of rows 2 and ny-1 in slots 2..4 (src/lhsbt2f.f90:193-213) */
        if (g->eps_e != zero && (r == 1 || r == 2)) {
          const double sb[3] = {-one, two, -one};
          for (int k = 2; k <= 4; ++k)
            for (int a = 1; a <= 5; ++a)
              MT(k, a, a, p) = MT(k, a, a, p) + alfa * d * g->eps_e * g->buff[p] * sb[k - 2];
        }
      }
  }
  /* boundary conditions */
  for (int i = 1; i <= nx; ++i) {
    if (g->navier) {
      const long p = IX(g, i, 1);
      if (dir == 1) {
        /* src/lhsbc1f.f90:238-265 */
        if (g->wall == 1 || g->wall == 2 || g->wall == 3) {
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MT(k, 1, b, p) = zero;
          MT(3, 1, 1, p) = one;
        }
        for (int a = 2; a <= 4; ++a)
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MT(k, a, b, p) = zero;
        for (int a = 2; a <= 4; ++a) MT(3, a, a, p) = one;
        if (g->wallt == 0 || g->wallt == 1) {
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MT(k, 5, b, p) = zero;
          MT(3, 5, 5, p) = one;
        }
      } else {
        /* src/lhsbc2f.f90:197-279 */
        const int sl[5] = {3, 4, 5, 1, 2};
        const double gcs[5] = {gc1, gc2, gc3, gc4, gc5}, ex3[5] = {-one, 4.0, -6.0, 4.0, -one};
        if (g->wall == 1 || g->wall == 3) {
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MT(k, 1, b, p) = zero;
          for (int t = 0; t < 5; ++t) MT(sl[t], 1, 1, p) = g->wall == 1 ? -gcs[t] : ex3[t];
        }
        for (int a = 2; a <= 4; ++a)
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MT(k, a, b, p) = zero;
        for (int a = 2; a <= 4; ++a) MT(3, a, a, p) = one;
        if (g->wallt == 0) {
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MT(k, 5, b, p) = zero;
          MT(3, 5, 5, p) = -one;
        }
        if (g->wallt == 1) {
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MT(k, 5, b, p) = zero;
          for (int t = 0; t < 5; ++t) MT(sl[t], 5, 5, p) = -gcs[t];
        }
      }
    }
    const long p = IX(g, i, ny);
    if (dir == 1) {
      /* src/lhsbc1f.f90:594-605: identity rows (top 0) */
      if (g->top == 0) {
        for (int a = 1; a <= 5; ++a)
          for (int k = 1; k <= 5; ++k)
            for (int b = 1; b <= 5; ++b) MT(k, a, b, p) = zero;
        for (int a = 1; a <= 5; ++a) MT(3, a, a, p) = one;
      }
    } else if (g->Ma < one && g->top == 0) {
      /* src/lhsbc2f.f90:284-291 */
      for (int a = 1; a <= 5; ++a)
        for (int k = 1; k <= 5; ++k)
          for (int b = 1; b <= 5; ++b) MT(k, a, b, p) = zero;
      rm_lhs(a2, i, vl + 5 * IX(g, i, ny), vl + 5 * IX(g, i, ny - 1), vl + 5 * IX(g, i, ny - 2), mat, p);
    } else if (g->Ma < one && g->top == 3) {
      /* src/lhsbc2f.f90:332-339: identity row (the xi LHS keeps its band row,
         src/lhsbc1f.f90:596 acts for top 0 only; the RHS row is left as rbe
         gives it, src/rhsbc.f90:350-356) */
      for (int a = 1; a <= 5; ++a)
        for (int k = 1; k <= 5; ++k)
          for (int b = 1; b <= 5; ++b) MT(k, a, b, p) = zero;
      for (int a = 1; a <= 5; ++a) MT(3, a, a, p) = one;
    }
  }
  return 0;
}
#undef MT

/* -------------------------------------------------------------------- step */

/* src/impdrv.f90:171-400 with linear = 0, impl = 1, iLHS = 1 */
double a2_step(const A2Grid* a2, int niter, double* v, double* vold, double* r, A3Ops* ops, double* dtl,
               double* mat, double* per, double* cfl) {
  const A3Grid* g = G(a2);
  const int nx = g->nx, ny = g->ny;
  const long n5 = 5L * nx * ny;
  double totres = 0.0;
  const double c = a3_set_time_step(g, v, dtl);  /* impdrv.f90:176 */
  if (cfl) *cfl = c;
  memcpy(vold, v, n5 * sizeof(double));
  a2_itrbc(a2, v);
  for (int iter = 1; iter <= niter; ++iter) {
    a2_genmtrx(a2, v, ops, r);
    a2_rbe(a2, r, v, vold, dtl);
    a2_rhsbc(a2, r, v);
    totres = a2_resstat(a2, r, dtl);
    a2_lhs(a2, ops, dtl, v, 1, mat);
    orc_penta_p(2, nx, ny, mat, r, per, ORC_COMPAT_PERIODIC_SLOT);
    a2_lhs(a2, ops, dtl, v, 2, mat);
    orc_penta_bc(1, ny, nx, mat, r);
    OMP_FOR
    for (long e = 0; e < n5; ++e) v[e] = v[e] + r[e];
    a2_itrbc(a2, v);
  }
  return totres;
}

/* ----------------------------------------------- second-order LHS (iLHS = 0) */

/* Block of row t (1..n) at column c of line iv in the block-tridiagonal
   storage: mat(3,5,5,...) slot c-t+2 or one of the boundary blocks
   bc(14,5,5,nlines), in the block table of src/nsolve2bc.f90:40-420 (the
   same table as oracle/tri_oracle.c). */
static Blk tri_blk(double* mat3, double* bc, long rec, int iv, int t, int c, int n) {
  static const int tab[6][5] = {{2, 3, -1, -2, -3}, {1, 2, 3, -4, -5}, {-7, 1, 2, 3, -6},
                                {-8, 1, 2, 3, -9}, {-10, -11, 1, 2, 3}, {-12, -13, -14, 1, 2}};
  int src = 0;
  if (t <= 3) src = tab[t - 1][c - 1];
  else if (t >= n - 2) src = tab[t - (n - 2) + 3][c - (n - 4)];
  else src = c - t + 2;
  Blk b;
  if (src > 0) b.p = mat3 + (src - 1) + 75 * rec, b.sa = 3, b.sb = 15;
  else b.p = bc + (-src - 1) + 350L * iv, b.sa = 14, b.sb = 70;
  return b;
}
#define EB(B, a, b) ((B).p[(long)((a) - 1) * (B).sa + (long)((b) - 1) * (B).sb])

/* The second-order LHS of the xi (dir 1: lhs1, src/lhs.f90:7-137, with the
   nonlinear lhsbc1 rows, src/lhsbc1.f90) or eta direction (dir 2: lhs2,
   src/lhs.f90:140-277, lhsbt2, src/lhsbt2.f90, and the nonlinear lhsbc2
   rows, src/lhsbc2.f90) in the reference's block-tridiagonal storage:
   dir 1 mat3(3,5,5,nx,ny) (lines over j; a periodic xi leaves bc zero,
   src/lhsbt1.f90), dir 2 mat3(3,5,5,nx,ny) with bc(14,5,5,nx) (lines over
   i).  Expression order follows the reference (Fortran left to right). */
int a2_lhs2(const A2Grid* a2, const A3Ops* o, const double* dtl, const double* vl, int dir, double* mat3,
            double* bc) {
  const A3Grid* g = G(a2);
  const int nx = g->nx, ny = g->ny;
  const double alfa = g->alfa;
  if ((dir == 1 && !g->xper) || g->yper || ny < 8) return 1;
  const double h = dir == 1 ? g->dxi : g->deta;
  const double a1 = -alfa * pt5 / h, a2c = alfa * zero, a3 = alfa * pt5 / h;
  const double b1 = alfa / (h * h), b2 = -alfa * two / (h * h), b3 = alfa / (h * h);
  const double ak[3] = {a1, a2c, a3}, bk[3] = {b1, b2, b3};
  memset(bc, 0, sizeof(double) * 350 * (size_t)(dir == 1 ? ny : nx));
  /* band, src/lhs.f90:44-104 (lhs1) and :180-240 (lhs2) */
  OMP_FOR
  for (int j = 1; j <= ny; ++j)
    for (int i = 1; i <= nx; ++i) {
      const long p = IX(g, i, j);
      const double d = dtl[p];
      const double* X = (dir == 1 ? o->Ah : o->Bh) + 25 * p;
      const double* V = (dir == 1 ? o->Vh11 : o->Vh22) + 6 * p;
      double* m = mat3 + 75 * p;
#define M3(k, a, b) m[(k - 1) + 3 * (a - 1) + 15 * (b - 1)]
      for (int a = 1; a <= 5; ++a)
        for (int b = 1; b <= 5; ++b)
          for (int k = 1; k <= 3; ++k) M3(k, a, b) = ak[k - 1] * d * X[(a - 1) + 5 * (b - 1)];
      if (dir == 1)
        for (int a = 1; a <= 5; ++a)
          for (int b = 1; b <= 5; ++b) M3(2, a, b) = M3(2, a, b) + alfa * d * o->Dh[(a - 1) + 5 * (b - 1) + 25 * p];
      for (int k = 1; k <= 3; ++k) {
        M3(k, 2, 2) = M3(k, 2, 2) - bk[k - 1] * d * V[0];
        M3(k, 2, 3) = M3(k, 2, 3) - bk[k - 1] * d * V[4];
        M3(k, 3, 2) = M3(k, 3, 2) - bk[k - 1] * d * V[5];
        M3(k, 3, 3) = M3(k, 3, 3) - bk[k - 1] * d * V[1];
        M3(k, 4, 4) = M3(k, 4, 4) - bk[k - 1] * d * V[2];
        M3(k, 5, 5) = M3(k, 5, 5) - bk[k - 1] * d * V[3];
      }
      for (int a = 1; a <= 5; ++a) M3(2, a, a) = M3(2, a, a) + one;
      /* second-order damping (eps_i = 4 eps_e) and, in the eta LHS, the
         sponge (src/lhs.f90:23-27,89-103 and 229-250) */
      if (g->eps_e != zero) {
        const double eps_i = 4.0 * g->eps_e;
        const double ck[3] = {-alfa * eps_i, alfa * two * eps_i, -alfa * eps_i};
        for (int k = 1; k <= 3; ++k)
          for (int a = 1; a <= 5; ++a) M3(k, a, a) = M3(k, a, a) + ck[k - 1] * d * g->buff[p];
      }
      if (dir == 2 && g->ispg == 2)
        for (int a = 1; a <= 5; ++a) M3(2, a, a) = M3(2, a, a) + alfa * d * (g->spg[p] + g->spg2[p]);
#undef M3
    }
  if (dir == 2) {
    /* boundary rows, src/lhsbt2.f90:28-520: row j, the stencil over columns
       c0..c0+4, first (g) and second (d) derivative coefficients, sign */
    const double detainv = one / g->deta, detasinv = one / (g->deta * g->deta);
    const double gcs[5] = {gc1, gc2, gc3, gc4, gc5}, gbs[5] = {gb1, gb2, gb3, gb4, gb5};
    const double gas[5] = {ga1, ga2, zero, ga3, ga4};
    const double dds[5] = {dd1, dd2, dd3, dd4, dd5}, dbs[5] = {db1, db2, db3, db4, db5};
    const double das[5] = {da1, da2, da3, da4, da5};
    for (int i = 1; i <= nx; ++i)
      for (int r = 0; r < 6; ++r) {
        const int j = r < 3 ? r + 1 : ny - 5 + r;
        const int c0 = r < 3 ? 1 : ny - 4;
        /* coefficient of column c0 + t */
        double gk[5], dk[5];
        double sg = one;
        for (int t = 0; t < 5; ++t) {
          if (r == 0) gk[t] = gcs[t], dk[t] = dds[t];
          else if (r == 1) gk[t] = gbs[t], dk[t] = dbs[t];
          else if (r == 2 || r == 3) gk[t] = gas[t], dk[t] = das[t];
          else if (r == 4) gk[t] = gbs[4 - t], dk[t] = dbs[4 - t], sg = -one;
          else gk[t] = gcs[4 - t], dk[t] = dds[4 - t], sg = -one;
        }
        const long p = IX(g, i, j);
        const double d = dtl[p];
        const double* X = o->Bh + 25 * p;
        const double* V = o->Vh22 + 6 * p;
        const long rec = (long)(i - 1) + (long)nx * (j - 1);
        for (int t = 0; t < 5; ++t) {
          const int c = c0 + t;
          const Blk B = tri_blk(mat3, bc, rec, i - 1, j, c, ny);
          for (int a = 1; a <= 5; ++a)
            for (int b = 1; b <= 5; ++b) {
              /* the central rows 3 and ny-2 set their diagonal block to a
                 literal zero before the viscous terms */
              const double v = alfa * d * gk[t] * detainv * X[(a - 1) + 5 * (b - 1)];
              EB(B, a, b) = (r == 2 || r == 3) && t == 2 ? zero : sg < zero ? -v : v;
            }
          const double w = alfa * d * dk[t] * detasinv;
          EB(B, 2, 2) = EB(B, 2, 2) - w * V[0];
          EB(B, 2, 3) = EB(B, 2, 3) - w * V[4];
          EB(B, 3, 2) = EB(B, 3, 2) - w * V[5];
          EB(B, 3, 3) = EB(B, 3, 3) - w * V[1];
          EB(B, 4, 4) = EB(B, 4, 4) - w * V[2];
          EB(B, 5, 5) = EB(B, 5, 5) - w * V[3];
        }
        /* the far-end rows have no block at column j+1 beyond ny; rows 1
           and ny keep mat(1) / mat(3) of the band zero */
        if (r == 0)
          for (int a = 1; a <= 5; ++a)
            for (int b = 1; b <= 5; ++b) mat3[0 + 3 * (a - 1) + 15 * (b - 1) + 75 * rec] = zero;
        if (r == 5)
          for (int a = 1; a <= 5; ++a)
            for (int b = 1; b <= 5; ++b) mat3[2 + 3 * (a - 1) + 15 * (b - 1) + 75 * rec] = zero;
        for (int a = 1; a <= 5; ++a) mat3[1 + 3 * (a - 1) + 15 * (a - 1) + 75 * rec] += one;
        /* sponge through the transposed spgl(ny,nx) view, then the damping
           of rows 2, ny-1 (-1, 2, -1) and 3, ny-2 (fb1..fb5)
           (src/lhsbt2.f90:96-110,170-205,266-310,374-420,482-525,579-595) */
        if (g->ispg == 2) {
          const long q = (long)(j - 1) + (long)(i - 1) * ny;
          for (int a = 1; a <= 5; ++a)
            mat3[1 + 3 * (a - 1) + 15 * (a - 1) + 75 * rec] += alfa * d * (g->spg[q] + g->spg2[q]);
        }
        if (g->eps_e != zero && r >= 1 && r <= 4) {
          const double fb[5] = {1.000000000000000E+00, -4.000000000000000E+00, 6.000000000000000E+00,
                                -4.000000000000000E+00, 1.000000000000000E+00};
          const double sb[3] = {-one, two, -one};
          const int wide = r == 2 || r == 3;
          for (int t = 0; t < (wide ? 5 : 3); ++t) {
            const int c = wide ? j - 2 + t : j - 1 + t;
            const Blk B = tri_blk(mat3, bc, rec, i - 1, j, c, ny);
            const double cf = wide ? fb[t] : sb[t];
            for (int a = 1; a <= 5; ++a) EB(B, a, a) = EB(B, a, a) + alfa * d * g->eps_e * g->buff[p] * cf;
          }
        }
      }
  }
  /* boundary conditions (nonlinear branches) */
  for (int i = 1; i <= nx; ++i) {
    const long rw = (long)(i - 1), rt = (long)(i - 1) + (long)nx * (ny - 1);
    double* mw = mat3 + 75 * rw;
    double* mt = mat3 + 75 * rt;
#define MW(k, a, b) mw[(k - 1) + 3 * (a - 1) + 15 * (b - 1)]
#define MTT(k, a, b) mt[(k - 1) + 3 * (a - 1) + 15 * (b - 1)]
#define BCI(jb, a, b) bc[(jb - 1) + 14 * (a - 1) + 70 * (b - 1) + 350L * (i - 1)]
    if (g->navier) {
      if (dir == 1) {
        /* src/lhsbc1.f90 (nonlinear): identity rows at the wall */
        if (g->wall == 1 || g->wall == 2 || g->wall == 3) {
          for (int k = 1; k <= 3; ++k)
            for (int b = 1; b <= 5; ++b) MW(k, 1, b) = zero;
          MW(2, 1, 1) = one;
        }
        for (int a = 2; a <= 4; ++a) {
          for (int k = 1; k <= 3; ++k)
            for (int b = 1; b <= 5; ++b) MW(k, a, b) = zero;
          MW(2, a, a) = one;
        }
        if (g->wallt == 0 || g->wallt == 1) {
          for (int k = 1; k <= 3; ++k)
            for (int b = 1; b <= 5; ++b) MW(k, 5, b) = zero;
          MW(2, 5, 5) = one;
        }
      } else {
        /* src/lhsbc2.f90 (nonlinear) */
        if (g->wall == 1) {
          for (int k = 1; k <= 3; ++k)
            for (int b = 1; b <= 5; ++b) MW(k, 1, b) = zero;
          for (int jb = 1; jb <= 3; ++jb)
            for (int b = 1; b <= 5; ++b) BCI(jb, 1, b) = zero;
          MW(2, 1, 1) = -gc1;
          MW(3, 1, 1) = -gc2;
          BCI(1, 1, 1) = -gc3;
          BCI(2, 1, 1) = -gc4;
          BCI(3, 1, 1) = -gc5;
        }
        if (g->wall == 3) {  /* bc(1:3,1,:,:) is not cleared, src/lhsbc2.f90 */
          for (int k = 1; k <= 3; ++k)
            for (int b = 1; b <= 5; ++b) MW(k, 1, b) = zero;
          MW(2, 1, 1) = -one;
          MW(3, 1, 1) = 4.0;
          BCI(1, 1, 1) = -6.0;
          BCI(2, 1, 1) = 4.0;
          BCI(3, 1, 1) = -one;
        }
        for (int a = 2; a <= 4; ++a) {
          for (int k = 1; k <= 3; ++k)
            for (int b = 1; b <= 5; ++b) MW(k, a, b) = zero;
          for (int jb = 1; jb <= 3; ++jb)
            for (int b = 1; b <= 5; ++b) BCI(jb, a, b) = zero;
          MW(2, a, a) = one;
        }
        if (g->wallt == 0 || g->wallt == 1) {
          for (int k = 1; k <= 3; ++k)
            for (int b = 1; b <= 5; ++b) MW(k, 5, b) = zero;
          for (int jb = 1; jb <= 3; ++jb)
            for (int b = 1; b <= 5; ++b) BCI(jb, 5, b) = zero;
        }
        if (g->wallt == 0) MW(2, 5, 5) = -one;
        if (g->wallt == 1) {
          MW(2, 5, 5) = -gc1;
          MW(3, 5, 5) = -gc2;
          BCI(1, 5, 5) = -gc3;
          BCI(2, 5, 5) = -gc4;
          BCI(3, 5, 5) = -gc5;
        }
      }
    }
    if (dir == 1) {
      if (g->top == 0) {  /* src/lhsbc1.f90 (nonlinear), top identity rows */
        for (int k = 1; k <= 3; ++k)
          for (int a = 1; a <= 5; ++a)
            for (int b = 1; b <= 5; ++b) MTT(k, a, b) = zero;
        for (int a = 1; a <= 5; ++a) MTT(2, a, a) = one;
      }
    } else if (g->Ma >= one || g->top == 0) {
      for (int k = 1; k <= 3; ++k)
        for (int a = 1; a <= 5; ++a)
          for (int b = 1; b <= 5; ++b) MTT(k, a, b) = zero;
      for (int jb = 12; jb <= 14; ++jb)
        for (int a = 1; a <= 5; ++a)
          for (int b = 1; b <= 5; ++b) BCI(jb, a, b) = zero;
      if (g->Ma < one) {
        /* ReimannLHS on (mat(2), mat(1), bc(14)) of row ny */
        const Blk rb[3] = {{&BCI(14, 1, 1), 14, 70}, {&MTT(1, 1, 1), 3, 15}, {&MTT(2, 1, 1), 3, 15}};
        rm_lhs_blk(a2, i, vl + 5 * IX(g, i, ny), vl + 5 * IX(g, i, ny - 1), vl + 5 * IX(g, i, ny - 2), rb);
      } else {
        for (int a = 1; a <= 5; ++a) MTT(2, a, a) = one;
      }
    }
#undef MW
#undef MTT
#undef BCI
  }
  return 0;
}
#undef EB

/* src/impdrv.f90:171-400 with linear = 0, impl = 1, iLHS = 0: the
   second-order LHS and the block-tridiagonal solves solve2p (xi) and
   solve1bc (eta), src/impdrv.f90:307-344.  mat3 (3,5,5,nx,ny) and bc
   (14,5,5,nx) are scratch. */
double a2_step2(const A2Grid* a2, int niter, double* v, double* vold, double* r, A3Ops* ops, double* dtl,
                double* mat3, double* bc, double* cfl) {
  const A3Grid* g = G(a2);
  const int nx = g->nx, ny = g->ny;
  const long n5 = 5L * nx * ny;
  double totres = 0.0;
  const double c = a3_set_time_step(g, v, dtl);
  if (cfl) *cfl = c;
  memcpy(vold, v, n5 * sizeof(double));
  a2_itrbc(a2, v);
  for (int iter = 1; iter <= niter; ++iter) {
    a2_genmtrx(a2, v, ops, r);
    a2_rbe(a2, r, v, vold, dtl);
    a2_rhsbc(a2, r, v);
    totres = a2_resstat(a2, r, dtl);
    a2_lhs2(a2, ops, dtl, v, 1, mat3, bc);
    orc_tri_p(2, nx, ny, mat3, r);
    a2_lhs2(a2, ops, dtl, v, 2, mat3, bc);
    orc_tri_bc(1, ny, nx, mat3, r, bc);
    OMP_FOR
    for (long e = 0; e < n5; ++e) v[e] = v[e] + r[e];
    a2_itrbc(a2, v);
  }
  return totres;
}

/* ------------------------------------------------------------ time schemes */

/* rtb, src/impdrv.f90:511-539: the two-step backward right-hand side
   r = onept33 vold - pt33 v2old - v - pt66 dtl r */
void a2_rtb(const A2Grid* a2, double* r, const double* v, const double* vold, const double* v2old,
            const double* dtl) {
  const A3Grid* g = G(a2);
  const double onept33 = 1.3333333333333333333, pt33 = 3.3333333333333333333e-1, pt66 = 6.6666666666666666666e-1;
  for (int j = 1; j <= g->ny; ++j)
    for (int i = 1; i <= g->nx; ++i)
      for (int k = 0; k < 5; ++k) {
        const long e = k + 5 * IX(g, i, j);
        r[e] = onept33 * vold[e] - pt33 * v2old[e] - v[e] - pt66 * dtl[IX(g, i, j)] * r[e];
      }
}

/* One step of src/impdrv.f90:172-402 (linear = 0) with the time scheme impl
   (src/impdrv.f90:186-198, 245-279) and the LHS order ilhs
   (src/impdrv.f90:307-332):
     impl 1  backward Euler with the grid's alfa;
     impl 2  two-step backward: backward Euler (alfa = 1) while lstep = 0,
             afterwards v2old = vold and rtb with alfa = pt66;
     impl 3  midpoint: genmtrx on pt5 (v + vold) (the operators of the LHS
             too), rbe, alfa = pt5.
   ilhs 1 uses the fourth-order LHS and the pentadiagonal solvers, 0 the
   second-order LHS and the block-tridiagonal solvers.  v2old and w
   (5,nx,ny) are needed for impl 2 and 3; mat(5,5,5,nx,ny) + per for ilhs 1,
   mat3(3,5,5,nx,ny) + bc(14,5,5,nx) for ilhs 0. */
double a2_step_impl(const A2Grid* a2, int ilhs, int impl, long lstep, int niter, double* v, double* vold,
                    double* v2old, double* w, double* r, A3Ops* ops, double* dtl, double* mat, double* per,
                    double* mat3, double* bc, double* cfl) {
  const A3Grid* g = G(a2);
  const int nx = g->nx, ny = g->ny;
  const long n5 = 5L * nx * ny;
  const int rtb = impl == 2 && lstep > 0;
  A2Grid al = *a2;
  al.g.alfa = impl == 3 ? pt5 : rtb ? 6.6666666666666666666e-1 : (impl == 2 ? one : g->alfa);
  double totres = 0.0;
  const double c = a3_set_time_step(g, v, dtl);
  if (cfl) *cfl = c;
  if (rtb) memcpy(v2old, vold, n5 * sizeof(double));
  memcpy(vold, v, n5 * sizeof(double));
  a2_itrbc(a2, v);
  for (int iter = 1; iter <= niter; ++iter) {
    if (impl == 3) {
      OMP_FOR
      for (long e = 0; e < n5; ++e) w[e] = pt5 * (v[e] + vold[e]);
      a2_genmtrx(&al, w, ops, r);
    } else {
      a2_genmtrx(&al, v, ops, r);
    }
    if (rtb) a2_rtb(&al, r, v, vold, v2old, dtl);
    else a2_rbe(&al, r, v, vold, dtl);
    a2_rhsbc(&al, r, v);
    totres = a2_resstat(&al, r, dtl);
    if (ilhs == 0) {
      a2_lhs2(&al, ops, dtl, v, 1, mat3, bc);
      orc_tri_p(2, nx, ny, mat3, r);
      a2_lhs2(&al, ops, dtl, v, 2, mat3, bc);
      orc_tri_bc(1, ny, nx, mat3, r, bc);
    } else {
      a2_lhs(&al, ops, dtl, v, 1, mat);
      orc_penta_p(2, nx, ny, mat, r, per, ORC_COMPAT_PERIODIC_SLOT);
      a2_lhs(&al, ops, dtl, v, 2, mat);
      orc_penta_bc(1, ny, nx, mat, r);
    }
    OMP_FOR
    for (long e = 0; e < n5; ++e) v[e] = v[e] + r[e];
    a2_itrbc(a2, v);
  }
  return totres;
}
