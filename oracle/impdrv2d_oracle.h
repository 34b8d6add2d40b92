/*
 * CPU oracle for the nonlinear two-dimensional implicit ADI step of LNS3D
 * (src/impdrv.f90 with linear = 0, impl = 1, iLHS = 1).  TEST
 * INFRASTRUCTURE ONLY: the checker for the GPU step, never the product path.
 *
 * Restated routines (each function cites the lines it follows):
 *   derivatives      src/grad.f90, src/grad2.f90, src/gradbc.f90 (the same
 *                    stencils as the complex ones, a3_deriv1/a3_deriv2)
 *   RHS, operators   src/genmtrx.f90 (linear = 0: RHS :282-312, A :458-503,
 *                    B :525-575, D :702-836, V :586-600, hats :602-700)
 *   time step        src/temporal.f90 set_time_step on the state
 *   BCs              src/rhsbc.f90 (nonlinear branch :256-370),
 *                    src/itrbc.f90 (nonlinear branch :623-760),
 *                    src/reimann.f90 (Reimann, ReimannRHS, ReimannLHS)
 *   residual         src/resstat.f90:37-60
 *   LHS              src/lhsf.f90 (lhs1f, lhs2f), src/lhsbt2f.f90,
 *                    src/lhsbc1f.f90 (:230-605), src/lhsbc2f.f90 (:193-330)
 *   step driver      src/impdrv.f90:171-400
 *
 * Supported options (the others are rejected): xper with yper false; a
 * viscous wall at j = 1 (wall 0, 1 or 3; wallt 0 or 1); the far field at
 * j = ny by Riemann invariants (top 0, Ma < 1) or held (Ma > 1); constant
 * viscosity; no sponge, damper or smoother; general metric transform.
 *
 * Layouts are the reference's (Fortran column-major): v(5,nx,ny),
 * mat(5,5,5,nx,ny), Ah(5,5,nx,ny), Vh(6,nx,ny), metrics (nx,ny), and the
 * top boundary arrays bnt(nx,2), rhobt(nx) ... (src/gengrid.f90:141-142,
 * src/potential.f90:17-30).
 */
#pragma once
#include "adi3d_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  A3Grid g;               /* grid, deck (kz = omega = 0 unused) and metrics */
  double theta;           /* isothermal wall recovery temperature angle (wallt 0) */
  const double* bnt;      /* (nx,2) unit normal of the top boundary */
  const double *rhobt, *ubt, *vbt, *wbt, *tbt;  /* top.pot (nx) */
} A2Grid;

/* r = RHS of the nonlinear equations, and the operators Ah Bh Dh Vh11 Vh12
   Vh22 of the LHS (genmtrx(v, zero, r)) */
int a2_genmtrx(const A2Grid* g, const double* v, A3Ops* ops, double* r);
void a2_rbe(const A2Grid* g, double* r, const double* v, const double* vold, const double* dtl);
void a2_rhsbc(const A2Grid* g, double* r, const double* v);
void a2_itrbc(const A2Grid* g, double* v);
double a2_resstat(const A2Grid* g, const double* r, const double* dtl);
/* LHS of the xi (dir 1) or eta (dir 2) sweep, real mat(5,5,5,nx,ny) */
int a2_lhs(const A2Grid* g, const A3Ops* ops, const double* dtl, const double* v, int dir, double* mat);
/* One implicit step of niter correctors on v (5,nx,ny): set_time_step on v,
   vold = v, itrBC, then per corrector genmtrx, rbe, rhsBC, resstat, the xi
   LHS and penta2p, the eta LHS and penta1bc, v += r, itrBC.  ops, dtl, r,
   vold, mat, per, per2 are scratch ((5,5,nx,ny) x3, (6,nx,ny) x3, (nx,ny),
   (5,nx,ny) x2, (5,5,5,nx,ny), (2,5,5,nx,ny)).  Returns totres of the last
   corrector; *cfl the step's CFL number. */
double a2_step(const A2Grid* g, int niter, double* v, double* vold, double* r, A3Ops* ops, double* dtl,
               double* mat, double* per, double* cfl);
/* The second-order path (iLHS = 0): LHS in the block-tridiagonal storage
   mat3(3,5,5,nx,ny) + bc(14,5,5,nx) (src/lhs.f90, src/lhsbt2.f90,
   src/lhsbc1.f90, src/lhsbc2.f90), and its step with solve2p / solve1bc. */
int a2_lhs2(const A2Grid* g, const A3Ops* ops, const double* dtl, const double* v, int dir, double* mat3, double* bc);
double a2_step2(const A2Grid* g, int niter, double* v, double* vold, double* r, A3Ops* ops, double* dtl,
                double* mat3, double* bc, double* cfl);
/* rtb (src/impdrv.f90:511-539) and one step with the time scheme impl 1/2/3
   (src/impdrv.f90:186-279) and the LHS order ilhs 1/0; lstep counts the
   steps before this one. */
void a2_rtb(const A2Grid* g, double* r, const double* v, const double* vold, const double* v2old, const double* dtl);
double a2_step_impl(const A2Grid* g, int ilhs, int impl, long lstep, int niter, double* v, double* vold,
                    double* v2old, double* w, double* r, A3Ops* ops, double* dtl, double* mat, double* per,
                    double* mat3, double* bc, double* cfl);

#ifdef __cplusplus
}
#endif
