/*
 * CPU oracle for the LNS3D block-pentadiagonal line solvers.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA
 * kernels in lns3d_gb300/csrc; only tests/, __graft_entry__.smoke() and the
 * cpu_baseline leg of bench.py may load it.  The product path never calls it.
 *
 * It restates, as one generic right-looking block elimination, the eight
 * reference solvers
 *   src/penta1bc.f:2  src/penta2bc.f:2  src/penta1p.f:2  src/penta2p.f:2
 *   src/cpenta1bc.f:2 src/cpenta2bc.f:2 src/cpenta1p.f:2 src/cpenta2p.f:2
 * and is pinned bit-for-bit against those sources translated mechanically by
 * oracle/f77sub2c.py (oracle/_ref/libref_penta.so).
 *
 * Array layouts are the reference's (Fortran column-major, 1-based in the
 * comments, 0-based in C):
 *   layout 2 ("penta2*"): mat(5,5,5,n,nsys)  rhs(5,n,nsys)   lines batched over the 2nd index
 *   layout 1 ("penta1*"): mat(5,5,5,nsys,n)  rhs(5,nsys,n)   lines batched over the 1st index
 *   mat(k,m,q,i,iv): slot k (1..5 <-> column offset -2..+2 with the boundary
 *   wrap of src/lhsbt1f.f90:43-48,102-107,199-204), block row m, block column q.
 *   Periodic fill: per(2,5,5,np,nsys) / per(2,5,5,nsys,np); complex
 *   per2(np-2:np-1,5,5,np,nsys) / (np-2:np-1,5,5,nsys,np); the real periodic
 *   solvers' per2(6,5,5,nsys) is scratch.
 * Complex numbers are interleaved (re, im) doubles, as Fortran complex*16.
 */
#pragma once
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reproduce the reference periodic solvers' fill placement at row n-5
 * (src/penta2p.f:278,339; src/penta1p.f and src/cpenta{1,2}p.f at the same
 * statements): the column-(n-1) fill of pivot row n-5 is added to slot 4
 * (column n-2) of row n-3 instead of slot 5.  On by default for parity with
 * the reference; without it the oracle is the exact LU of the periodic matrix. */
#define ORC_COMPAT_PERIODIC_SLOT 1
/* Reproduce, serially and in line order, the complex boundary solvers' solve
 * phase at row n-3 (src/cpenta1bc.f:675, src/cpenta2bc.f:676): the row n-1
 * update is replaced by an update of rhs at transposed indices.  Off by
 * default (the reference races under OpenMP and may index out of bounds). */
#define ORC_COMPAT_CBC_RHS 2

/* Out-of-bounds accesses skipped by ORC_COMPAT_CBC_RHS since load. */
long orc_oob_count(void);

/* Real boundary-closure solve (penta1bc / penta2bc). n >= 7. */
int orc_penta_bc(int layout, int n, int nsys, double* mat, double* rhs);
/* Real periodic solve (penta1p / penta2p) on np = n+1 rows; row np = row 1. */
int orc_penta_p(int layout, int np, int nsys, double* mat, double* rhs,
                double* per, int flags);
/* Complex boundary-closure solve (cpenta1bc / cpenta2bc); code 0 LU, 1 solve, 2 both. */
int orc_cpenta_bc(int layout, int n, int nsys, double* mat, double* rhs, int code, int flags);
/* Complex periodic solve (cpenta1p / cpenta2p); code 0 LU, 1 solve, 2 both. */
int orc_cpenta_p(int layout, int np, int nsys, double* mat, double* rhs,
                 double* per, double* per2, int code, int flags);

/* Block-tridiagonal solves of the second-order path (tri_oracle.c):
 * solve1bc / solve2bc (src/nsolve{1,2}bc.f90) with the boundary blocks
 * bc(14,5,5,nsys), n >= 8; solve1p / solve2p (src/nsolve{1,2}p.f90) on
 * np = n+1 rows, row np = row 1.  mat(3,5,5,...) is read only. */
int orc_tri_bc(int layout, int n, int nsys, const double* mat, double* rhs, const double* bc);
int orc_tri_p(int layout, int np, int nsys, const double* mat, double* rhs);

#ifdef __cplusplus
}
#endif
