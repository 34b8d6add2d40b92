/*
 * lns3d_gb300 -- C ABI of the GB300 (sm_103a) implicit ADI line solvers.
 *
 * Each entry point is the drop-in for one reference Fortran solver of the
 * LNS3D implicit step and keeps its argument order, sizes and array layouts
 * (Fortran column-major, complex as interleaved (re, im) doubles, i.e.
 * complex*16).  A Fortran host binds them through iso_c_binding with VALUE
 * integer arguments and assumed-size arrays.
 *
 * Two forms per solver:
 *   lns_<name>      host pointers: the arrays are staged to the GPU, solved
 *                   and copied back; synchronous, like the Fortran call.
 *   lns_<name>_dev  device pointers: enqueued on `stream` (a cudaStream_t,
 *                   NULL for the legacy default stream); asynchronous.
 *
 * Block size: nblk must be 5 (ndof, src/global.f90).  Lines need n >= 7
 * rows (the boundary-closure rows 1, 2, n-4..n must be distinct; the
 * reference itself has no such check and silently mis-solves shorter lines).
 *
 * Return value: LNS_OK, or an LNS_ERR_* code; lns_last_error() describes the
 * last failure of the calling thread.  The reference has no error return; it
 * produces Inf/NaN on a zero pivot, which the GPU path reports as
 * LNS_ERR_PIVOT (the arrays then hold the same non-finite values).
 */
#ifndef LNS3D_GB300_H
#define LNS3D_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LNS_OK 0
#define LNS_ERR_ARG 1      /* invalid size, nblk != 5, bad code or flag */
#define LNS_ERR_CUDA 2     /* CUDA runtime failure (message in lns_last_error) */
#define LNS_ERR_PIVOT 3    /* a pivot became zero or non-finite */
#define LNS_ERR_NOMEM 4    /* device allocation failed */

/* Last error message of the calling thread ("" if none). */
const char* lns_last_error(void);
/* Library version string. */
const char* lns_version(void);

/* ---------------------------------------------------------------------------
 * Real block-pentadiagonal solves with the 4th-order boundary-closure rows,
 * single pass (factor + solve).  mat is scratch on return (its content is
 * unspecified, as in the reference); rhs returns the solution.
 */
/* replaces src/penta2bc.f:2  penta2bc(n, nsys, nblk, mat(5,nblk,nblk,n,nsys), rhs(nblk,n,nsys)) */
int lns_penta2bc(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs);
int lns_penta2bc_dev(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs, void* stream);
/* replaces src/penta1bc.f:2  penta1bc(nsys, n, nblk, mat(5,nblk,nblk,nsys,n), rhs(nblk,nsys,n)) */
int lns_penta1bc(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs);
int lns_penta1bc_dev(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs, void* stream);

/* ---------------------------------------------------------------------------
 * Complex boundary-closure solves with the LU / solve split.
 * code 0: factor mat in place (multipliers stored where entries are
 * eliminated, as the reference); 1: solve rhs with a factored mat; 2: both.
 * The solve phase applies the row n-3 -> n-1 update that the reference
 * mis-indexes (src/cpenta1bc.f:675, src/cpenta2bc.f:676), i.e. it solves the
 * factored system exactly.
 */
/* replaces src/cpenta2bc.f:2  cpenta2bc(n, nsys, nblk, mat, rhs, code) */
int lns_cpenta2bc(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs, int32_t code);
int lns_cpenta2bc_dev(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs, int32_t code,
                      void* stream);
/* replaces src/cpenta1bc.f:2  cpenta1bc(nsys, n, nblk, mat, rhs, code) */
int lns_cpenta1bc(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs, int32_t code);
int lns_cpenta1bc_dev(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs, int32_t code,
                      void* stream);

/* ---------------------------------------------------------------------------
 * Periodic solves.  np = n + 1 rows per line, n unknowns; on return row np
 * of rhs repeats row 1 (src/penta2p.f:749-751).  per(2,nblk,nblk,np,nsys)
 * ("2" solvers; (2,nblk,nblk,nsys,np) for the "1" solvers) receives the fill
 * of columns n-1, n.  Real solvers: single pass, per is scratch and per2 --
 * the reference's (6,nblk,nblk,nsys) scratch -- is not touched.  Complex
 * solvers: code as for the boundary solvers, and per and
 * per2(np-2:np-1,nblk,nblk,np,nsys) (or (...,nsys,np)) hold the factored
 * fill between a code 0 and a code 1 call, in the reference's format.
 *
 * By default the factorisation reproduces the reference exactly, including
 * its placement of one fill block at row n-5 (src/penta2p.f:278,339 and the
 * same statements in penta1p.f, cpenta1p.f, cpenta2p.f), which makes the
 * reference solve a slightly different system whose error decays with the
 * line length.  lns_set_periodic_exact(1) switches every later periodic
 * factorisation of the process to the exact LU; lns_set_periodic_exact(0)
 * restores the reference behaviour.
 */
int lns_set_periodic_exact(int32_t on);
/* replaces src/penta2p.f:2  penta2p(np, nsys, nblk, mat, rhs, per, per2) */
int lns_penta2p(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per, double* per2);
int lns_penta2p_dev(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per,
                    double* per2, void* stream);
/* replaces src/penta1p.f:2  penta1p(nsys, np, nblk, mat, rhs, per, per2) */
int lns_penta1p(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per, double* per2);
int lns_penta1p_dev(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per,
                    double* per2, void* stream);
/* replaces src/cpenta2p.f:2  cpenta2p(np, nsys, nblk, mat, rhs, per, per2, code) */
int lns_cpenta2p(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per, double* per2,
                 int32_t code);
int lns_cpenta2p_dev(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per,
                     double* per2, int32_t code, void* stream);
/* replaces src/cpenta1p.f:2  cpenta1p(nsys, np, nblk, mat, rhs, per, per2, code) */
int lns_cpenta1p(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per, double* per2,
                 int32_t code);
int lns_cpenta1p_dev(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per,
                     double* per2, int32_t code, void* stream);

/* ---------------------------------------------------------------------------
 * Mixed-precision solves (no reference counterpart: the reference solves in
 * FP64 only).  The LU factors are computed and applied in FP32 -- the FP64
 * rate of the GB300 is 1/64 of its FP32 rate -- and `refine` steps of
 * iterative refinement, x += LU32^-1 (b - A x) with the residual formed in
 * FP64 from the untouched mat, restore FP64 accuracy for well-conditioned
 * lines (two steps reach FP64 rounding on the isolated-solve workload);
 * refine = 0 gives the FP32 interior solve of the mixed ADI step.
 * mat is read only.  code 0 writes the FP32 factors to `work`; code 1
 * solves rhs in place with the factors in `work` (mat must still hold the
 * matrix that was factored); code 2 does both.  `work` is a device buffer of
 * lns_mixed_workspace_bytes(rows, nsys, is_complex, periodic) bytes (rows =
 * n, or np for periodic lines), owned by the caller and kept between the
 * code 0 and code 1 calls.  Periodic mixed solves always use the exact LU.
 */
size_t lns_mixed_workspace_bytes(int32_t rows, int32_t nsys, int32_t is_complex, int32_t periodic);
int lns_cpenta2bc_mixed_dev(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs, int32_t code,
                            int32_t refine, void* work, void* stream);
int lns_cpenta1bc_mixed_dev(int32_t nsys, int32_t n, int32_t nblk, const double* mat, double* rhs, int32_t code,
                            int32_t refine, void* work, void* stream);
int lns_cpenta2p_mixed_dev(int32_t np, int32_t nsys, int32_t nblk, const double* mat, double* rhs, int32_t code,
                           int32_t refine, void* work, void* stream);
int lns_cpenta1p_mixed_dev(int32_t nsys, int32_t np, int32_t nblk, const double* mat, double* rhs, int32_t code,
                           int32_t refine, void* work, void* stream);
/* real boundary solves, factor + solve in one call */
int lns_penta2bc_mixed_dev(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs, int32_t refine,
                           void* work, void* stream);
int lns_penta1bc_mixed_dev(int32_t nsys, int32_t n, int32_t nblk, const double* mat, double* rhs, int32_t refine,
                           void* work, void* stream);
/* host-pointer form of cpenta2bc_mixed (factor + solve), staged internally */
int lns_cpenta2bc_mixed(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs, int32_t refine);

/* ---------------------------------------------------------------------------
 * Block-tridiagonal line solves of the second-order implicit path (iLHS = 0
 * of src/impdrv.f90:307-344), real FP64, factor and right-hand side in one
 * pass as the reference does:
 *   lns_solve2bc  replaces solve2bc(n,nsys,nblk,mat,rhs,bc),   src/nsolve2bc.f90:2
 *   lns_solve1bc  replaces solve1bc(nsys,n,nblk,mat,rhs,bc),   src/nsolve1bc.f90:2
 *   lns_solve2p   replaces solve2p(np,nsys,nblk,mat,rhs,per,per2), src/nsolve2p.f90:2
 *   lns_solve1p   replaces solve1p(nsys,np,nblk,mat,rhs,per,per2), src/nsolve1p.f90:2
 * mat(3,nblk,nblk,n,nsys) ("2") or (3,nblk,nblk,nsys,n) ("1"): slot 1, 2, 3
 * = columns i-1, i, i+1; bc(14,nblk,nblk,nsys): the blocks the second-order
 * boundary rows add (rows 1..3 and n-2..n reach five columns,
 * src/nsolve2bc.f90:40-420); periodic lines have np = n+1 rows, row np
 * repeats row 1, and per, per2 are the reference's fill scratch (not used:
 * the GPU keeps its fill in the workspace).  nblk must be 5; n >= 8 (np >= 9).
 * The solution replaces rhs; mat and bc are read only.  The host forms
 * stage through library-owned device buffers; the _dev forms take device
 * pointers and a device workspace of lns_tri_workspace_bytes(rows, nsys,
 * periodic) bytes (rows = n, or np for periodic lines).
 */
size_t lns_tri_workspace_bytes(int32_t rows, int32_t nsys, int32_t periodic);
int lns_solve2bc(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* bc);
int lns_solve1bc(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs, double* bc);
int lns_solve2p(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per, double* per2);
int lns_solve1p(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per, double* per2);
int lns_solve2bc_dev(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs, const double* bc,
                     void* work, void* stream);
int lns_solve1bc_dev(int32_t nsys, int32_t n, int32_t nblk, const double* mat, double* rhs, const double* bc,
                     void* work, void* stream);
int lns_solve2p_dev(int32_t np, int32_t nsys, int32_t nblk, const double* mat, double* rhs, void* work,
                    void* stream);
int lns_solve1p_dev(int32_t nsys, int32_t np, int32_t nblk, const double* mat, double* rhs, void* work,
                    void* stream);

/* ---------------------------------------------------------------------------
 * The nonlinear two-dimensional implicit ADI step (src/impdrv.f90:171-400
 * with linear = 0, impl = 1, 2 or 3, iLHS = 1 or 0) as one device-resident context, FP64
 * throughout.  Per step: set_time_step on the state, vold = v, itrBC; per
 * corrector genmtrx(v, 0, r) (the nonlinear RHS and the operators), rbe,
 * rhsBC, resstat, lhs1f + lhsbc1f and penta2p (xi), lhs2f + lhsbt2f +
 * lhsbc2f and penta1bc (eta), v = v + r, itrBC.  The LHS is formed and
 * factored every corrector, as the reference does for the nonlinear
 * equations.
 * Supported options: a periodic xi direction (xper 1, penta2p), or a non-
 * periodic one (xper 0, penta2bc along xi, the one-sided closure rows of
 * src/lhsbt1f.f90) below Ma 1 with a Riemann far field (left 0, right 0;
 * src/reimann.f90 on bnl / bnr and left.pot / right.pot) or a symmetry plane
 * (left 2) on the left and first-order extrapolation of the right plane over
 * the viscous layer (extrap, nbl, update_nbl: src/itrbc.f90:849-886,
 * src/rhsbc.f90:461-476, src/lhsbc1f.f90:819-859); yper = 0, a viscous wall
 * at j = 1 (navier 1, wall 0, 1 or 3, wallt 0 or 1) and the Riemann far
 * field at j = ny (top 0; held free stream when Ma > 1) or the held
 * quiescent top (top 3, row ny held at (1, 0, 0, 0, 1), fourth-order LHS
 * only); constant viscosity; the sponge and the smoother as below; no
 * damper.  Arrays are Fortran-ordered: v(5,nx,ny), metrics(nx,ny,10),
 * bnt(nx,2) (src/gengrid.f90:141-142), pot(5,nx) = the rho u v w T rows of
 * top.pot (src/potential.f90:22-26).
 */
typedef struct {
  int32_t nx, ny;
  double dxi, deta;
  double Ma, Re, Pr, gamma;
  double gamma1;             /* the reference's gamma1 module variable: 0.4 as src/init.f90:28
                                sets it (not gamma - 1, which differs in the last bit); 0 means
                                gamma - 1 */
  double alfa, cflmax, dtmax;
  double theta;              /* isothermal-wall recovery angle (wallt 0, src/itrbc.f90:683-686) */
  int32_t loctime, xper, yper, navier, wall, wallt, top, optx, opty;
  int32_t lhs_order;         /* 0 or 4: the fourth-order LHS with pentadiagonal solves (iLHS = 1);
                                2: the second-order LHS (src/lhs.f90, src/lhsbt2.f90, src/lhsbc1.f90,
                                src/lhsbc2.f90) with the block-tridiagonal solves solve2p (xi) and
                                solve1bc (eta) (iLHS = 0, src/impdrv.f90:307-344); needs ny >= 8 */
  int32_t impl;              /* time scheme (src/impdrv.f90:186-279): 1 (or 0) backward Euler with
                                alfa; 2 two-step backward, backward Euler at alfa = 1 for the
                                context's first step and rtb at alfa = 2/3 after it; 3 midpoint,
                                genmtrx on (v + vold)/2 with alfa = 1/2.  Steps are counted from
                                the context's creation (a fresh run, lstep = 0). */
  int32_t ispg;              /* 0, or 2: the sponge towards the free stream, r += (spg + spg2)
                                (v - (1,0,0,0,1)) (src/genmtrx.f90:436-446) and alfa dtl
                                (spg + spg2) on the eta LHS diagonal (src/lhsf.f90:296-312,
                                src/lhsbt2f.f90, whose boundary rows read the array through a
                                transposed (ny,nx) view, kept here); lns_upload_sponge2d */
  double eps_e;              /* explicit smoother at the end of genmtrx (src/smoother.f90) and
                                implicit damping of both LHS (src/lhsf.f90:113-145, 262-294,
                                src/lhsbt2f.f90:193-213) weighted by buff (ones until
                                lns_upload_buffer2d); with lhs_order 2 the second-order damping
                                of src/lhs.f90 and src/lhsbt2.f90. */
  int32_t left, right;       /* xi planes when xper = 0: left 0 (Riemann), 2 (symmetry plane by
                                extrapolation, src/itrbc.f90:776-798) or 7 (symmetry plane by
                                mirrored stencils and LHS rows, src/grad.f90:155-250,
                                src/lhsbs1f.f90, v = 0 on it); right 0 (Riemann), 7 or 8 (the
                                initial condition held, src/rhsbc.f90:478-480);
                                ignored when xper = 1 */
  int32_t extrap;            /* -1 off, 0 or 1: the right plane extrapolated from its neighbours
                                over rows 1..nbl (the viscous layer) */
  int32_t nbl;               /* rows of the viscous layer before the first itrBC (the &extras
                                namelist's nbl, default 0); 0 <= nbl <= ny */
  int32_t update_nbl;        /* 1: every itrBC sets nbl to the first row whose u at column nx-1
                                exceeds 0.99 (src/itrbc.f90:849-857); a state with no such row
                                fails the step with LNS_ERR_ARG, where the reference stops */
} lns_params2d;

typedef struct lns_ctx2d lns_ctx2d;

/* replaces the allocations of src/impdrv.f90:30-138 */
int lns_ctx2d_create(const lns_params2d* params, lns_ctx2d** ctx);
int lns_ctx2d_destroy(lns_ctx2d* ctx);
size_t lns_ctx2d_bytes(const lns_ctx2d* ctx);
/* metrics(nx,ny,10): m1 m2 n1 n2 m11 m12 m22 n11 n12 n22 (metric.dat) */
int lns_upload_metrics2d(lns_ctx2d* ctx, const double* metrics);
/* far field of the top boundary: unit normal bnt(nx,2) and top.pot (5,nx) */
int lns_upload_top2d(lns_ctx2d* ctx, const double* bnt, const double* pot);
/* far field of a xi plane (xper = 0): side 1 = left (bnl(ny,2), left.pot
 * (5,ny)), 2 = right (bnr(ny,2), right.pot (5,ny)); the unit outward
 * normals of src/gengrid.f90:145-155 and the rho u v w T rows of
 * src/potential.f90:36-72.  Needed before the first step for a Riemann
 * plane (left 0, right 0). */
int lns_upload_side2d(lns_ctx2d* ctx, int32_t side, const double* bn, const double* pot);
/* The sponge arrays spg(nx,ny), spg2(nx,ny) (src/sponge.f90) when ispg = 2;
 * needed before the first step. */
int lns_upload_sponge2d(lns_ctx2d* ctx, const double* spg, const double* spg2);
/* The smoother weight buff(nx,ny) (src/buffer.f90, ibuff > 0) when eps_e != 0. */
int lns_upload_buffer2d(lns_ctx2d* ctx, const double* buff);
/* itrBC on a device state (the call before the step loop, src/impdrv.f90:160) */
int lns_itrbc2d_dev(lns_ctx2d* ctx, double* v, void* stream);
/* nsteps steps on the host state v(5,nx,ny) in place; totres[nsteps] (may be
 * NULL) gets resstat's value of the last corrector of each step */
int lns_step2d(lns_ctx2d* ctx, double* v, int32_t nsteps, int32_t niter, double* totres);
int lns_step2d_dev(lns_ctx2d* ctx, double* v, int32_t nsteps, int32_t niter, double* totres_dev, void* stream);
/* Inspection (device arrays): set_time_step(v), then
 * r = rhsBC(rbe(genmtrx(v, 0, r))) (src/genmtrx.f90, src/impdrv.f90:482,
 * src/rhsbc.f90) with *totres_dev = resstat(r); the operators stay in the
 * context for lns_lhs2d_dev and lns_get_field2d. */
int lns_rhs2d_dev(lns_ctx2d* ctx, const double* v, const double* vold, double* r, double* totres_dev, void* stream);
/* LHS of the xi (dir 1: src/lhsf.f90:7 + src/lhsbc1f.f90) or eta sweep
 * (dir 2: src/lhsf.f90:164 + src/lhsbt2f.f90 + src/lhsbc2f.f90 with
 * ReimannLHS, src/reimann.f90:238) from the context's operators, into the
 * device array mat(5,5,5,nx,ny).  With lhs_order = 2 the second-order LHS
 * (src/lhs.f90, src/lhsbt2.f90, src/lhsbc{1,2}.f90): its mat(3,5,5,..) and
 * bc(14,5,5,..) blocks placed in the pentadiagonal slots of their columns,
 * zero blocks elsewhere */
int lns_lhs2d_dev(lns_ctx2d* ctx, int32_t dir, const double* v, double* mat, void* stream);
/* host copy of 0 Ah, 1 Bh, 2 Dh (5,5,nx,ny), 3 Vh11, 4 Vh12, 5 Vh22
 * (6,nx,ny), 6 dtl (nx,ny) */
int lns_get_field2d(lns_ctx2d* ctx, int32_t which, double* out);

/* lns_cpenta2bc_mixed_dev with code 2 (factor + solve) that allocates no
 * device memory and takes no workspace.  No counterpart in the reference.
 * It is for callers that hold no device buffer to lend as scratch and must
 * not have the library call cudaMalloc during a solve -- for example a host
 * whose device memory is handed out by its own pool allocator (a library
 * allocation would fail or fragment the pool), or one that keeps cudaMalloc,
 * which may wait for work already queued on the device, out of its
 * time-critical loop.
 * Scratch is one fixed array of LNS_STATIC_WORKSPACE_BYTES in the library's
 * device image.  Problems whose scratch, lns_mixed_workspace_bytes(n, nsys,
 * 1, 0), exceeds it (about 29 900 rows x lines) are rejected with
 * LNS_ERR_ARG and a message giving both sizes.  Nothing in the scratch needs
 * to start at zero.  The first call on a device looks up the array's address
 * (once per device); make that first call before any stream capture.  The
 * address is kept for the rest of the process: after cudaDeviceReset (or
 * anything else that destroys the device's primary context) this entry
 * point must not be called again in that process.  All
 * calls on a device share the one array, so calls that overlap in time -- on
 * different streams or from different host threads -- race and corrupt each
 * other's results: keep them ordered (one stream, or events). */
#define LNS_STATIC_WORKSPACE_BYTES (32u << 20)
int lns_cpenta2bc_mixed_static_dev(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs,
                                   int32_t refine, void* stream);

/* ---------------------------------------------------------------------------
 * The linearised single-Fourier-mode implicit ADI step (src/impdrv3d.f90,
 * impl = 1, iLHS = 1) as one device-resident context.
 *
 * The reference keeps its state in modules (src/global.f90,
 * src/local2d.f90, src/local3d.f90) and reads it from the input deck
 * (src/input.f90); here a context owns the metrics, the frozen operators,
 * the time step, the factored xi and eta LHS and the scratch fields on one
 * device.  Sequence of a run (src/lns3d.f90:140-160, src/impdrv3d.f90):
 *   lns_ctx3d_create        deck values, device buffers
 *   lns_upload_metrics3d    metric.dat arrays
 *   lns_upload_mean3d       mean flow: genmtrx(vm, kz, vm) and set_time_step
 *                           on the GPU; the next step factors the LHS again
 *   lns_step3d / _dev       nsteps implicit steps of niter correctors
 * Supported options: xper = 1 (periodic xi sweep, cpenta2p), yper = 0 with a
 * viscous wall at j = 1 (navier = 1, wall 1, 2 or 3 (the bump), wallt 0 or 1) and a
 * zero-disturbance top (top = 0) or a top forced by an incoming acoustic
 * wave (top = 1, lns_upload_inflow3d); optx, opty any; constant viscosity
 * (mattyp 0); the sponges (ispg) and the smoother (eps_e) below; no damper
 * and no filter.  Other options return LNS_ERR_ARG.
 *
 * precision LNS_FP64 follows the reference arithmetic (complex*16
 * throughout).  LNS_MIXED keeps the RHS, the residual and the update in
 * FP64 and forms, factors and applies both LHS in FP32 (complex*8): the
 * sweeps compute the correction only, so the converged state is the FP64
 * one while each step differs from the FP64 step by FP32 rounding of the
 * correction.  No reference counterpart.
 *
 * All arrays are Fortran-ordered: v(5,nx,ny) complex*16 as interleaved
 * doubles, vm(5,nx,ny), metrics(nx,ny,10).
 */
#define LNS_FP64 0
#define LNS_MIXED 1

typedef struct {
  int32_t nx, ny;            /* grid points; with xper, point nx repeats point 1 */
  double dxi, deta;          /* computational spacings (src/gengrid.f90: 1/(nx-1), 1/(ny-1)) */
  double Ma, Re, Pr, gamma;  /* src/input.f90 deck values */
  double gamma1;             /* the reference's gamma1 (0.4, src/init.f90:28); 0 means gamma - 1 */
  double omega, beta;        /* temporal frequency and spanwise wavenumber kz = 2 pi / Lz */
  double alfa;               /* implicitness, 1 for backward Euler (impl = 1) */
  double cflmax, dtmax;      /* src/temporal.f90 time-step control */
  int32_t loctime;           /* 0 global time step, 1 local time step */
  int32_t xper, yper, navier, wall, wallt, top, optx, opty;
  int32_t precision;         /* LNS_FP64 or LNS_MIXED */
  int32_t impl;              /* time scheme (src/impdrv3d.f90:130-199): 1 (or 0)
                                backward Euler with alfa; 2 two-step backward,
                                backward Euler for the context's first step and
                                rtb3D with alfa = 2/3 after it; 3 midpoint, the
                                operator at (v + vold)/2 with alfa = 1/2.  Steps
                                are counted from the context's creation (a fresh
                                run, lstep = 0).  Batches and servers take 1. */
  int32_t ispg;              /* sponge (src/lrhs3d.f90:220-280, src/sponge.f90:536-607,
                                src/lhs2f3d.f90:207-224, src/lhsbt2f3d.f90:147-167): 0 none;
                                1 r += spg v and alfa dtl spg on the diagonal of the eta LHS;
                                > 4 the same with spg + spg2; 2, 3 r += spg v + spg2 (v - t)
                                towards the decaying inflow wave t (lns_upload_inflow3d; 3
                                scales it by wamp(i)); 4 r += (spg + spg2)(v - cvic)
                                (lns_upload_sponge_target3d).  2-4 put alfa dtl (spg + spg2)
                                on the LHS diagonal.  Batches and servers take 0. */
  double eps_e;              /* explicit smoother (src/smoother3d.f90, at the end of lrhs3D)
                                and implicit damping of both LHS (src/lhs1f3d.f90:168-200,
                                src/lhs2f3d.f90:171-203, src/lhsbt2f3d.f90:277-298,
                                431-452) with the weight buff(nx,ny): ones (the reference's
                                ibuff = 0) until lns_upload_buffer3d.  0 turns both off.
                                Beside a symmetry plane (left or right 7) both take its
                                mirrored stencils.  Batches and servers take 0. */
  int32_t left, right;       /* the xi boundaries when xper = 0 (src/itrbc3d.f90:203-414,
                                src/rhsbc3d.f90:167-324, src/lhsbc1f3d.f90:412-448,
                                src/lhsbc2f3d.f90:146-174): left 0 zero disturbance, 1 an
                                incoming acoustic wave exp(-a (x - x0)) exp(i kk x) formed from
                                the mean flow (lns_upload_inflow3d), 4 the eigenfunction inflow
                                (lns_upload_profile3d), 5 the undamped acoustic wave exp(i kk x)
                                (lns_upload_inflow3d), 7 a symmetry plane; right 0 zero
                                disturbance, 4 the eigenfunction outflow (with left 4), 5 the
                                acoustic wave, 7 a symmetry plane, 8 the held initial
                                condition.  The acoustic planes take x as the reference does,
                                x(j,1) and x(j,nx) of the (nx,ny) grid, the point (j-1) and
                                (j-1) + nx (nx-1) (src/itrbc3d.f90:331, 395); right 5 needs
                                ny >= nx, which keeps that point inside the grid.  A symmetry plane
                                (src/cgrad.f90:193-266, src/lhsbs1f3d.f90) mirrors the field,
                                v changing sign, into the stencils of its three nearest points
                                and the xi LHS rows of its two (the smoother and the implicit
                                damping included); it needs ny <= nx (those rows read ABhi
                                through the reference's
                                (6,ny,nx) view of the (6,nx,ny) array, src/lhsbs1f3d.f90:17,
                                which the GPU reproduces and which leaves the array when ny > nx).
                                Ignored with xper = 1.  Batches and servers take xper = 1. */
} lns_params3d;

typedef struct lns_ctx3d lns_ctx3d;

/* Allocates the context on the current device.  replaces the allocations of
 * src/impdrv3d.f90:46-99 and the deck of src/input.f90 */
int lns_ctx3d_create(const lns_params3d* params, lns_ctx3d** ctx);
int lns_ctx3d_destroy(lns_ctx3d* ctx);
/* Device bytes the context holds (excluding what the caller owns). */
size_t lns_ctx3d_bytes(const lns_ctx3d* ctx);
/* metrics(nx,ny,10) on the host: m1 m2 n1 n2 m11 m12 m22 n11 n12 n22
 * (src/gengrid.f90:82-131, metric.dat) */
int lns_upload_metrics3d(lns_ctx3d* ctx, const double* metrics);
/* The sponge coefficients spg(nx,ny) and, for ispg > 4, spg2(nx,ny), as the
 * host's sponge setup (src/sponge.f90) leaves them; needed before the first
 * step when ispg != 0; invalidates the factored LHS. */
int lns_upload_sponge3d(lns_ctx3d* ctx, const double* spg, const double* spg2);
/* ispg 2, 3, top 1, left 1 or 5, right 5: the x coordinates x(nx,ny), the station x0 and the
 * amplitudes wamp(nx) (NULL: ones, the reference's default; ispg 3 needs
 * them) of the inflow sponge's wave (src/lrhs3d.f90:242-268) and of the
 * forced top boundary's incoming acoustic wave (top 1: v = t and r = -(v - t)
 * on row ny, src/itrbc3d.f90:145-196, src/rhsbc3d.f90:129-160); the waves
 * are formed on the device from these and the mean flow. */
int lns_upload_inflow3d(lns_ctx3d* ctx, const double* x, const double* wamp, double x0);
/* ispg 4: the eigenfunction target cvic, complex (5,nx,ny) as interleaved
 * doubles (src/sponge.f90:558-579). */
int lns_upload_sponge_target3d(lns_ctx3d* ctx, const double* cvic);
/* wall 3 (the bump, src/genbump.f90): u1w, u2w, u3w, tw, twp, complex (5,nx)
 * as interleaved doubles; the wall row holds these velocities, rho by
 * third-order extrapolation, T = tw (wallt 0) or the gc closure equal to twp
 * (wallt 1) (src/itrbc3d.f90:46-121, src/rhsbc3d.f90:45-104,
 * src/lhsbc2f3d.f90:41-48).  Needed before the first step. */
/* The eigenfunction of the xi planes (left 4, and right 4), the inflow.dat
 * profile that src/gendist.f90:40-47 reads: prof(10,ny) = rho, u, v, w, T as
 * (re, im) pairs per row, held at column 1 (src/itrbc3d.f90:247-320,
 * src/rhsbc3d.f90:207-243); with right 4, column nx holds
 * prof * exp(i lalpha x(nx,j)) (src/itrbc3d.f90:357-381), xr(ny) = x(nx,:)
 * and lalpha the inflow namelist's complex wavenumber (may be NULL / 0 with
 * right != 4).  Needed before the first step with left 4. */
int lns_upload_profile3d(lns_ctx3d* ctx, const double* prof, const double* xr, double lalpha_re, double lalpha_im);
int lns_upload_bump3d(lns_ctx3d* ctx, const double* bump);
/* The smoother weight buff(nx,ny) of the host's buffer setup (src/buffer.f90,
 * ibuff > 0); only for eps_e != 0; invalidates the factored LHS. */
int lns_upload_buffer3d(lns_ctx3d* ctx, const double* buff);
/* vm(5,nx,ny) on the host: builds the frozen operators (src/genmtrx.f90,
 * linear = 1, called as genmtrx(vm, kz, vm) at src/lns3d.f90:149) and the
 * time step (src/temporal.f90:12-130, called at src/impdrv3d.f90:54);
 * *cfl (may be NULL) returns the CFL number of that time step.  Invalidates
 * the stored LHS factors. */
int lns_upload_mean3d(lns_ctx3d* ctx, const double* vm, double* cfl);
/* nsteps implicit steps on the host disturbance v(5,nx,ny) (in place);
 * totres[nsteps] (may be NULL) receives resstat3D's residual of the last
 * corrector of each step.  replaces the body of src/impdrv3d.f90:130-356:
 * vold = v, itrBC3D, then niter times lrhs3D, rbe3D, rhsBC3D, resstat3D,
 * the xi sweep cpenta2p (LHS lhs1f3D + lhsbc1f3D factored at the first
 * step of the context), the eta sweep cpenta1bc (lhs2f3D + lhsbt2f3D +
 * lhsbc2f3D), v = v + r, itrBC3D. */
int lns_step3d(lns_ctx3d* ctx, double* v, int32_t nsteps, int32_t niter, double* totres);
/* Device form: v is a device array; totres_dev (may be NULL) a device array
 * of nsteps doubles; enqueued on `stream`.  The first call after
 * lns_upload_mean3d factors the LHS and waits for the pivot check. */
int lns_step3d_dev(lns_ctx3d* ctx, double* v, int32_t nsteps, int32_t niter, double* totres_dev, void* stream);
/* itrBC3D on a device state: the call before the step loop (src/impdrv3d.f90:125-126) */
int lns_itrbc3d_dev(lns_ctx3d* ctx, double* v, void* stream);

/* Inspection (device arrays, enqueued on `stream`), for parity checks.
 * r = rhsBC3D(rbe3D(lrhs3D(v), v, vold)) (src/lrhs3d.f90:2,
 * src/impdrv3d.f90:444, src/rhsbc3d.f90:2) in FP64, and *totres_dev =
 * resstat3D(r) (src/resstat3d.f90:2) when totres_dev is not NULL. */
int lns_rhs3d_dev(lns_ctx3d* ctx, const double* v, const double* vold, double* r, double* totres_dev, void* stream);
/* The unfactored LHS of the xi (dir 1: src/lhs1f3d.f90 + src/lhsbc1f3d.f90)
 * or eta sweep (dir 2: src/lhs2f3d.f90 + src/lhsbt2f3d.f90 +
 * src/lhsbc2f3d.f90) into the complex*16 device array mat(5,5,5,nx,ny). */
int lns_lhs3d_dev(lns_ctx3d* ctx, int32_t dir, double* mat, void* stream);
/* Line mode of the FP64 periodic sweeps, no reference counterpart.  With
 * on = 1 (the default for a context used alone) the lines advance both
 * recurrences two rows per step where their row count allows it (periodic
 * lines with an odd band: nx even for xi, ny even for a periodic eta; eta
 * lines with boundary-closure rows: ny even) and the direction has at most
 * twice as many lines as the GPU has SMs (more lines fill the FP64 pipes
 * row by row): one row of each pair is combined with its neighbour's blocks
 * once, at factoring time, which changes the solution by rounding only.  on = 0 keeps every line row by
 * row, as the contexts of a batch or a server always are.  Takes effect at
 * the next factorisation (the next step).  LNS_ERR_ARG for on not 0 or 1. */
int lns_ctx3d_set_row_pairs(lns_ctx3d* ctx, int32_t on);
/* Phase timing, no reference counterpart.  lns_ctx3d_profile(ctx, 1) makes
 * every later corrector record CUDA events on its stream (and resets the
 * record); lns_ctx3d_profile_read waits for them and returns the summed
 * milliseconds of LNS_PROFILE_SEGMENTS segments in ms[]: 0 RHS, 1 xi
 * scaling, 2 xi forward recurrence, 3 xi backward recurrence, 4 xi border
 * (the periodic lines' border unknowns and correction; empty for a
 * non-periodic xi), 5 eta scaling, 6 eta forward, 7 eta backward (with a
 * periodic eta's border), 8 update; and the number of correctors in
 * *ncorr.  Clears the record. */
#define LNS_PROFILE_SEGMENTS 9
int lns_ctx3d_profile(lns_ctx3d* ctx, int32_t on);
int lns_ctx3d_profile_read(lns_ctx3d* ctx, double* ms, int32_t* ncorr);
/* Copy of a frozen field to the host in the reference layout:
 * 0 Ah, 1 Bh, 2 Dh, 3 Dhi (5,5,nx,ny); 4 Vh11, 5 Vh12, 6 Vh22, 7 ABhi
 * (6,nx,ny); 8 dtl (nx,ny). */
int lns_get_field3d(lns_ctx3d* ctx, int32_t which, double* out);

/* ---------------------------------------------------------------------------
 * The linearised two-dimensional implicit step (src/impdrv.f90:171-400 with
 * linear = 1: src/lrhs.f90 about the frozen operators of genmtrx(vm, 0, vm),
 * src/lns3d.f90:149; rbe/rtb, rhsBC, resstat, lhs1f/lhs2f with their
 * boundary rows, penta2p or penta2bc, penta1p or penta1bc, v += r, itrBC).
 * With the spanwise wavenumber and the frequency zero these are the
 * single-mode step's routines on real fields, so the context runs a
 * single-mode context at beta = omega = 0 (the options it supports, FP64)
 * and converts the state: v(5,nx,ny) is real here.  Sequence:
 *   lns_lin2d_create(params with beta = omega = 0)   deck values; xper = 1, or xper = 0 with
 *                                                    left 0 (zero disturbance), 1 (nonreflecting)
 *                                                    or 7 (symmetry plane: the mirrored stencils,
 *                                                    and v = 0 and r = 0 for the second velocity
 *                                                    component, src/itrbc.f90:525-527) and right
 *                                                    0 or 1 (nonreflecting)
 *   lns_lin2d_set_nbl                                the &extras namelist's nbl (default 0): the
 *                                                    nonreflecting planes tie the density to the
 *                                                    outgoing characteristic on rows j > nbl
 *                                                    (src/itrbc.f90:340-342, src/rhsbc.f90:195)
 *   lns_upload_metrics_lin2d, lns_upload_mean_lin2d  metric.dat, mean.dat
 *   lns_itrbc_lin2d_dev                              the itrBC before the loop (src/impdrv.f90:160)
 *   lns_step_lin2d / _dev                            nsteps steps of niter correctors
 */
typedef struct lns_lin2d lns_lin2d;
int lns_lin2d_create(const lns_params3d* params, lns_lin2d** ctx);
int lns_lin2d_destroy(lns_lin2d* ctx);
size_t lns_lin2d_bytes(const lns_lin2d* ctx);
int lns_lin2d_set_nbl(lns_lin2d* ctx, int32_t nbl);
int lns_upload_metrics_lin2d(lns_lin2d* ctx, const double* metrics);
int lns_upload_mean_lin2d(lns_lin2d* ctx, const double* vm, double* cfl);
int lns_itrbc_lin2d_dev(lns_lin2d* ctx, double* v, void* stream);
/* host copy of the frozen time step dtl(nx,ny) (set_time_step on the mean flow) */
int lns_get_dtl_lin2d(lns_lin2d* ctx, double* dtl);
/* v(5,nx,ny) real on the host, in place; totres[nsteps] (may be NULL) gets
 * resstat's value of the last corrector of each step */
int lns_step_lin2d(lns_lin2d* ctx, double* v, int32_t nsteps, int32_t niter, double* totres);
int lns_step_lin2d_dev(lns_lin2d* ctx, double* v, int32_t nsteps, int32_t niter, double* totres_dev, void* stream);

/* ---------------------------------------------------------------------------
 * Batches of linearised problems (no reference counterpart: the reference
 * runs one problem per process).  A batch holds nprob independent problems
 * -- each with its own deck (grid size, beta, omega, ...), metrics, mean
 * flow and disturbance -- and advances all of them together: every phase of
 * the step (RHS, scaling, recurrences, fill, update) is one launch for all
 * problems, whose blocks look up their problem and local block in a work
 * table, and the whole step is captured once as a CUDA graph and replayed.
 * Each problem's result is identical to a lns_ctx3d run of the same problem
 * (the same kernels on the same data).  All problems share the precision.
 */
typedef struct lns_batch3d lns_batch3d;
/* params[nprob]: the deck of each problem */
int lns_batch3d_create(int32_t nprob, const lns_params3d* params, lns_batch3d** batch);
int lns_batch3d_destroy(lns_batch3d* batch);
size_t lns_batch3d_bytes(const lns_batch3d* batch);
/* metrics (nx,ny,10), mean flow vm(5,nx,ny) and disturbance v(5,nx,ny)
 * complex of problem prob (host arrays) */
int lns_batch3d_upload(lns_batch3d* batch, int32_t prob, const double* metrics, const double* vm, const double* v);
/* Picks the lines per CTA of the recurrences (1, 2 or 4) by timing a few
 * steps of each; the problems' states are restored afterwards. */
int lns_batch3d_tune(lns_batch3d* batch, int32_t niter, int32_t* lines_per_cta);
/* Steps every problem until its residual (resstat3D, the last corrector of
 * a step) is <= tol (tol > 0), or max_steps steps.  A problem stops on the
 * device in the step whose residual reaches tol: its state stays the one
 * whose residual met the tolerance, whatever check_every (how often the host
 * reads the residuals) and the other problems are.  steps[prob] = that step
 * (-1 if none), final_res[prob] = the last residual measured. */
int lns_batch3d_run(lns_batch3d* batch, int32_t max_steps, int32_t niter, double tol, int32_t check_every,
                    int32_t* steps, double* final_res);
int lns_batch3d_get_state(lns_batch3d* batch, int32_t prob, double* v);

/* ---------------------------------------------------------------------------
 * Serving (no reference counterpart).  A server keeps every admitted
 * request's operators, factors and state resident on the device and
 * advances all of them as one batch; requests that arrive while others are
 * running are admitted at the next tick when a slot and device memory
 * (budget_bytes) are free, and leave the batch when their residual reaches
 * their tolerance (the state is then the one that met it, as in
 * lns_batch3d_run) or after max_steps steps.  A request's result is
 * independent of the other requests in the batch.  Not thread-safe: one
 * host thread drives a server.
 */
#define LNS_REQ_QUEUED 1
#define LNS_REQ_RUNNING 2
#define LNS_REQ_DONE 3      /* converged: residual <= tol */
#define LNS_REQ_STOPPED 4   /* max_steps reached first */
#define LNS_REQ_FAILED 5    /* could not be admitted (allocation or upload failed), or its
                               result could not be read back */
typedef struct lns_server3d lns_server3d;
int lns_server3d_create(size_t budget_bytes, int32_t max_slots, int32_t precision, int32_t niter,
                        lns_server3d** server);
int lns_server3d_destroy(lns_server3d* server);
/* copies the request's host arrays (as lns_batch3d_upload); *id names it */
int lns_server3d_submit(lns_server3d* server, const lns_params3d* params, const double* metrics, const double* vm,
                        const double* v, double tol, int32_t max_steps, int64_t* id);
/* admits what fits, runs up to nsteps batched steps (fewer when a running
 * request has fewer left before its max_steps, so that none runs past it),
 * retires finished requests */
int lns_server3d_tick(lns_server3d* server, int32_t nsteps, int32_t* running, int32_t* queued);
/* state LNS_REQ_*, the step that met tol (or steps run), the last residual,
 * and the seconds from submission to completion (-1 while unfinished) */
int lns_server3d_poll(lns_server3d* server, int64_t id, int32_t* state, int32_t* steps, double* res,
                      double* latency_s);
/* the finished request's state v(5,nx,ny) complex; forgets the request.  A
 * failed request returns LNS_ERR_ARG and is forgotten too. */
int lns_server3d_fetch(lns_server3d* server, int64_t id, double* v);
size_t lns_server3d_bytes_in_use(const lns_server3d* server);
/* How many times the server has captured its step as a CUDA graph (a
 * diagnostic, no reference counterpart).  The batched kernels are
 * persistent grids over work tables in device memory, so requests joining
 * and leaving rewrite the tables and leave the captured step in place; it is
 * captured again only when a table outgrows its buffer or the stencil width
 * of the running requests changes. */
int32_t lns_server3d_graph_captures(const lns_server3d* server);

#ifdef __cplusplus
}
#endif

#endif /* LNS3D_GB300_H */
