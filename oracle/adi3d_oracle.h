/*
 * CPU oracle for the linearised single-Fourier-mode implicit ADI step of
 * LNS3D (src/impdrv3d.f90).  TEST INFRASTRUCTURE ONLY: the checker for the
 * GPU step, never the product path.
 *
 * Restated routines (each function cites the lines it follows):
 *   derivatives      src/cgrad.f90, src/cgrad2.f90, src/grad.f90, src/grad2.f90,
 *                    src/cgradbc.f90, src/gradbc.f90, src/stencil.f90
 *   operators        src/genmtrx.f90 (linear = 1 branch), src/getmat.f90 (mattyp 0)
 *   time step        src/temporal.f90 set_time_step
 *   RHS              src/lrhs3d.f90, rbe3D (src/impdrv3d.f90:444-469)
 *   BCs              src/rhsbc3d.f90, src/itrbc3d.f90
 *   residual         src/resstat3d.f90
 *   LHS              src/lhs1f3d.f90, src/lhs2f3d.f90, src/lhsbt2f3d.f90,
 *                    src/lhsbc1f3d.f90, src/lhsbc2f3d.f90
 *   step driver      src/impdrv3d.f90:130-356 (impl = 1, iLHS = 1)
 *
 * Supported options (the others are rejected): optx, opty in {0, -1, other};
 * xper (the x sweep is periodic) or not; yper false with a viscous wall at
 * j = 1 (wall 1 or 2, wallt 0 or 1) and a zero-disturbance top (top 0);
 * no sponge, smoother, damper, symmetry or Carpenter closures; constant
 * viscosity (mattyp 0); general (curvilinear) metric transform.
 *
 * Layouts are the reference's (Fortran column-major): v(5,nx,ny) complex as
 * interleaved (re, im), vm(5,nx,ny) real, Ah(5,5,nx,ny), Vh(6,nx,ny),
 * ABhi(6,nx,ny), metrics (nx,ny), mat(5,5,5,nx,ny) complex.
 */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nx, ny;
  double dxi, deta;
  double Ma, Re, Pr, gamma, gamma1;
  double omega, kz;       /* frequency and spanwise wavenumber (beta) */
  double alfa;            /* 1 for backward Euler */
  double cflmax, dtmax;
  int loctime;            /* 0 global time step, 1 local */
  int xper, yper, navier, wall, wallt, top, optx, opty;
  /* metrics (nx,ny): m1 m2 n1 n2 m11 m12 m22 n11 n12 n22 */
  const double *m1, *m2, *n1, *n2, *m11, *m12, *m22, *n11, *n12, *n22;
  /* sponge (src/lrhs3d.f90:220-240, src/lhs2f3d.f90:207-224): ispg 0 none,
     1 spg, > 4 spg + spg2 (2..4 not restated); spg, spg2 (nx,ny) */
  int ispg;
  const double *spg, *spg2;
  /* explicit smoother and implicit damping (src/smoother3d.f90,
     src/lhs1f3d.f90:168-200, src/lhs2f3d.f90:171-203, src/lhsbt2f3d.f90:
     277-298, 431-452): eps_e and buff(nx,ny); eps_e = 0 turns both off */
  double eps_e;
  const double* buff;
  /* inflow sponges (src/lrhs3d.f90:242-280): the mean flow vm(5,nx,ny), the
     x coordinates x(nx,ny), x0 and (ispg 3) wamp(nx); the eigenfunction
     sponge (ispg 4, src/sponge.f90:536-607): its target cvic, complex
     (5,nx,ny) */
  const double *vm, *xc, *wamp;
  double x0;
  const double* cvic;
  /* the bump wall (wall = 3, src/rhsbc3d.f90:45-104, src/itrbc3d.f90:46-121):
     u1w, u2w, u3w, tw, twp of src/genbump.f90, complex (5,nx) */
  const double* bump;
} A3Grid;

/* Frozen operators of the linear step (outputs of genmtrx(vm, kz, vm)). */
typedef struct {
  double *Ah, *Bh, *Dh, *Dhi;        /* (5,5,nx,ny) */
  double *Vh11, *Vh12, *Vh22, *ABhi; /* (6,nx,ny) */
} A3Ops;

/* first and second derivatives of v(ncomp,nx,ny) (real doubles; a complex
   field is passed as ncomp = 10 interleaved components) */
int a3_deriv1(const A3Grid* g, int ncomp, const double* v, double* g1v, double* g2v);
int a3_deriv2(const A3Grid* g, int ncomp, const double* v, const double* g1v, double* g11v, double* g12v,
              double* g22v);
/* operators from the mean flow vm(5,nx,ny) */
int a3_genmtrx(const A3Grid* g, const double* vm, A3Ops* ops);
/* local / global time step from the mean flow; returns the CFL number */
double a3_set_time_step(const A3Grid* g, const double* vm, double* dtl);
/* r = L(v) (lrhs3D), then r = vold - v - dtl r (rbe3D) */
int a3_lrhs(const A3Grid* g, const A3Ops* ops, const double* v, double* r);
/* the inflow sponge's target at (i, j), complex (5) as 10 doubles */
void a3_inflow_target(const A3Grid* g, int i, int j, double t[10]);
/* the forced top boundary's wave at (i, ny) (top = 1) */
void a3_top_target(const A3Grid* g, int i, double t[10]);
void a3_rbe(const A3Grid* g, double* r, const double* v, const double* vold, const double* dtl);
void a3_rhsbc(const A3Grid* g, double* r, const double* v);
double a3_resstat(const A3Grid* g, const double* r, const double* dtl);
void a3_itrbc(const A3Grid* g, double* v);
/* LHS of the xi (dir 1) or eta (dir 2) sweep, complex mat(5,5,5,nx,ny) */
int a3_lhs(const A3Grid* g, const A3Ops* ops, const double* dtl, int dir, double* mat);
/* One implicit step (impl 1, niter correctors): v, vold complex (5,nx,ny).
   matx, maty (and perx/per2x when xper) hold the factors: they are formed
   and factored when *factored == 0, and reused afterwards.  r is scratch.
   Returns totres of the last corrector. */
double a3_step(const A3Grid* g, const A3Ops* ops, const double* dtl, int niter, double* v, double* vold,
               double* r, double* matx, double* maty, double* perx, double* per2x, double* pery, double* per2y,
               int* factored);
/* rtb3D (src/impdrv3d.f90:471-501) and one step of the time schemes impl
   1, 2, 3 (see adi3d_oracle.c); vold, v2old persist across steps */
void a3_rtb(const A3Grid* g, double* r, const double* v, const double* vold, const double* v2old, const double* dtl);
double a3_step_impl(const A3Grid* g, const A3Ops* o, const double* dtl, int niter, int impl, int lstep, double* v,
                    double* vold, double* v2old, double* w, double* r, double* matx, double* maty, double* perx,
                    double* per2x, double* pery, double* per2y, double* alfa_fac);

#ifdef __cplusplus
}
#endif
