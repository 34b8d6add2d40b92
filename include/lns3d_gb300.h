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
/* Measured FP64 fused multiply-add rate of the current device in TFLOP/s
 * (a short DFMA stream on every SM); the denominator of the FP64 roofline
 * that the line solvers are reported against.  No reference counterpart.
 * Returns a negative value on failure. */
double lns_probe_fp64_tflops(void);

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

#ifdef __cplusplus
}
#endif

#endif /* LNS3D_GB300_H */
