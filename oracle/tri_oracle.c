/*
 * CPU oracle for the LNS3D block-tridiagonal line solvers of the
 * second-order implicit path (iLHS = 0): src/nsolve1bc.f90:2 (solve1bc),
 * src/nsolve2bc.f90:2 (solve2bc), src/nsolve1p.f90:2 (solve1p),
 * src/nsolve2p.f90:2 (solve2p).  TEST INFRASTRUCTURE ONLY: the checker for
 * the CUDA path, never the product path.
 *
 * A block-tridiagonal line, with the boundary-closure blocks that the
 * second-order boundary rows add (bc(14,5,5,nsys)), is a block-pentadiagonal
 * line whose other blocks are zero, and the reference eliminates it in the
 * same order as its pentadiagonal solvers (pivot row ascending, pivot column
 * ascending; division for the in-block step, a reciprocal for the rows
 * below).  So each line is copied into the pentadiagonal storage and solved
 * by the pentadiagonal restatement (penta_oracle.c); updates by the zero
 * blocks add exact zeros.  Where the reference keeps a block (its mat slot
 * or bc index, src/nsolve2bc.f90:40-420):
 *   row 1      columns 1..5   mat(2) mat(3) bc(1) bc(2) bc(3)
 *   row 2      columns 1..5   mat(1) mat(2) mat(3) bc(4) bc(5)
 *   row 3      columns 1..5   bc(7) mat(1) mat(2) mat(3) bc(6)
 *   rows 4..n-3               mat(1) mat(2) mat(3) at columns i-1, i, i+1
 *   row n-2    columns n-4..n bc(8) mat(1) mat(2) mat(3) bc(9)
 *   row n-1    columns n-4..n bc(10) bc(11) mat(1) mat(2) mat(3)
 *   row n      columns n-4..n bc(12) bc(13) bc(14) mat(1) mat(2)
 * Periodic lines (np = n+1 rows, src/nsolve2p.f90:36-100): mat(1) of row 1
 * is column n and mat(3) of row n is column 1; the reference's fill
 * (per: column n of rows 1..n-2, per2: row n, rolling) is the pentadiagonal
 * solver's fill restricted to those blocks.
 * Layouts: 2 ("solve2*") mat(3,5,5,n,nsys) rhs(5,n,nsys); 1 ("solve1*")
 * mat(3,5,5,nsys,n) rhs(5,nsys,n); bc(14,5,5,nsys) in both.
 */
#include <stdlib.h>
#include <string.h>

#include "penta_oracle.h"

static long tri_rec(int layout, int rows, int nsys, int t, int iv) {
  return layout == 2 ? (long)(t - 1) + (long)rows * iv : (long)iv + (long)nsys * (t - 1);
}

/* penta slot (1..5) of column c in row t of a boundary-closure line
   (inverse of the boundary layout, src/lhsbt1f.f90:43-48,102-107,199-204) */
static int penta_slot_bc(int t, int c, int n) {
  if (t == 1) { static const int s[6] = {0, 3, 4, 5, 1, 2}; return s[c]; }
  if (t == 2) { static const int s[6] = {0, 2, 3, 4, 5, 1}; return s[c]; }
  if (t == n - 1) { static const int s[5] = {5, 1, 2, 3, 4}; return s[c - (n - 4)]; }
  if (t == n) { static const int s[5] = {4, 5, 1, 2, 3}; return s[c - (n - 4)]; }
  return c - t + 3;
}

static void put(double* prec, int slot, const double* blk, long bstride) {
  for (int m = 0; m < 5; ++m)
    for (int q = 0; q < 5; ++q) prec[(slot - 1) + 5 * (m + 5 * q)] = blk[bstride * (m + 5 * q)];
}

int orc_tri_bc(int layout, int n, int nsys, const double* tmat, double* rhs, const double* bc) {
  if (n < 8 || nsys < 1 || (layout != 1 && layout != 2)) return 1;
  double* pm = (double*)calloc((size_t)125 * n * nsys, sizeof(double));
  if (!pm) return 2;
  for (int iv = 0; iv < nsys; ++iv) {
    const double* b = bc + 350L * iv;
    for (int t = 1; t <= n; ++t) {
      const long r = tri_rec(layout, n, nsys, t, iv);
      double* pr = pm + 125 * r;
      const double* tr = tmat + 75 * r;
      /* (column, source block) per the table above: mat slot k at tr + k-1
         (stride 3), bc index j at b + j-1 (stride 14) */
      int cols[5], cnt = 0;
      const double* src[5];
      long strd[5];
      const int nb = t == 1 || t == 2 || t == 3 || t >= n - 2 ? 5 : 3;
      /* kind: 'm' mat slot, 'b' bc index */
      static const char kind1[5] = {'m', 'm', 'b', 'b', 'b'}, kind2[5] = {'m', 'm', 'm', 'b', 'b'},
                        kind3[5] = {'b', 'm', 'm', 'm', 'b'}, kindA[5] = {'b', 'm', 'm', 'm', 'b'},
                        kindB[5] = {'b', 'b', 'm', 'm', 'm'}, kindC[5] = {'b', 'b', 'b', 'm', 'm'};
      static const int idx1[5] = {2, 3, 1, 2, 3}, idx2[5] = {1, 2, 3, 4, 5}, idx3[5] = {7, 1, 2, 3, 6},
                       idxA[5] = {8, 1, 2, 3, 9}, idxB[5] = {10, 11, 1, 2, 3}, idxC[5] = {12, 13, 14, 1, 2};
      const char* kind = 0;
      const int* idx = 0;
      int c0 = 1;
      if (t == 1) kind = kind1, idx = idx1;
      else if (t == 2) kind = kind2, idx = idx2;
      else if (t == 3) kind = kind3, idx = idx3;
      else if (t == n - 2) kind = kindA, idx = idxA, c0 = n - 4;
      else if (t == n - 1) kind = kindB, idx = idxB, c0 = n - 4;
      else if (t == n) kind = kindC, idx = idxC, c0 = n - 4;
      if (nb == 5) {
        for (int a = 0; a < 5; ++a) {
          cols[cnt] = c0 + a;
          src[cnt] = kind[a] == 'm' ? tr + idx[a] - 1 : b + idx[a] - 1;
          strd[cnt] = kind[a] == 'm' ? 3L : 14L;
          ++cnt;
        }
      } else {
        for (int k = 1; k <= 3; ++k) {
          cols[cnt] = t + k - 2;
          src[cnt] = tr + k - 1;
          strd[cnt] = 3L;
          ++cnt;
        }
      }
      for (int a = 0; a < cnt; ++a) put(pr, penta_slot_bc(t, cols[a], n), src[a], strd[a]);
    }
  }
  const int rc = orc_penta_bc(layout, n, nsys, pm, rhs);
  free(pm);
  return rc;
}

int orc_tri_p(int layout, int np, int nsys, const double* tmat, double* rhs) {
  const int n = np - 1;
  if (n < 8 || nsys < 1 || (layout != 1 && layout != 2)) return 1;
  double* pm = (double*)calloc((size_t)125 * np * nsys, sizeof(double));
  double* per = (double*)calloc((size_t)50 * np * nsys, sizeof(double));
  if (!pm || !per) {
    free(pm);
    free(per);
    return 2;
  }
  for (int iv = 0; iv < nsys; ++iv)
    for (int t = 1; t <= n; ++t) {
      const long r = tri_rec(layout, np, nsys, t, iv);
      for (int k = 1; k <= 3; ++k) put(pm + 125 * r, k + 1, tmat + 75 * r + (k - 1), 3L);
    }
  const int rc = orc_penta_p(layout, np, nsys, pm, rhs, per, 0);
  free(pm);
  free(per);
  return rc;
}
