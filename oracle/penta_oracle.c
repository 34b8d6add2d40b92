/*
 * CPU oracle for the LNS3D block-pentadiagonal line solvers.
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA kernels, never the
 * product path (see penta_oracle.h for layouts and citations).
 *
 * Build without FP contraction (oracle/Makefile: -ffp-contract=off) so that
 * each a + b*c rounds twice, as the reference Fortran does on x86-64.
 */
#include "penta_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

static long g_oob = 0;
long orc_oob_count(void) { return g_oob; }
static void orc_oob_note(void) { ++g_oob; }

/* ---------------------------------------------------------------- real */
#define T double
#define S(x) x##_r
#define ADD(a, b) ((a) + (b))
#define SUB(a, b) ((a) - (b))
#define MUL(a, b) ((a) * (b))
#define DIV(a, b) ((a) / (b))
#define NEG(a) (-(a))
#define ONE 1.0
#include "penta_engine.inc"
#undef T
#undef S
#undef ADD
#undef SUB
#undef MUL
#undef DIV
#undef NEG
#undef ONE

/* ------------------------------------------------------------- complex */
typedef struct { double re, im; } ocx;
static inline ocx cx_add(ocx a, ocx b) { ocx z = {a.re + b.re, a.im + b.im}; return z; }
static inline ocx cx_sub(ocx a, ocx b) { ocx z = {a.re - b.re, a.im - b.im}; return z; }
/* Fortran complex multiply without NaN recovery: (ac - bd, ad + bc). */
static inline ocx cx_mul(ocx a, ocx b) {
  ocx z = {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
  return z;
}
static inline ocx cx_neg(ocx a) { ocx z = {-a.re, -a.im}; return z; }
/* Complex division by Smith's range-reduced method (R. L. Smith, "Algorithm
   116: Complex division", CACM 5(8), 1962), which gfortran uses for
   complex*16 division under its default -fcx-fortran-rules. */
static inline ocx cx_div(ocx a, ocx b) {
  ocx z;
  if (fabs(b.re) < fabs(b.im)) {
    double r = b.re / b.im, d = b.re * r + b.im;
    z.re = (a.re * r + a.im) / d;
    z.im = (a.im * r - a.re) / d;
  } else {
    double r = b.im / b.re, d = b.im * r + b.re;
    z.re = (a.im * r + a.re) / d;
    z.im = (a.im - a.re * r) / d;
  }
  return z;
}
static const ocx cx_one = {1.0, 0.0};

#define T ocx
#define S(x) x##_c
#define ADD(a, b) cx_add(a, b)
#define SUB(a, b) cx_sub(a, b)
#define MUL(a, b) cx_mul(a, b)
#define DIV(a, b) cx_div(a, b)
#define NEG(a) cx_neg(a)
#define ONE cx_one
#include "penta_engine.inc"
#undef T
#undef S
#undef ADD
#undef SUB
#undef MUL
#undef DIV
#undef NEG
#undef ONE

/* ----------------------------------------------------------------- API */

/* Lines are independent: the timing build (-fopenmp) solves them in
   parallel, the parity build serially. */
#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

static int check(int layout, int n, int nsys) {
  if (layout != 1 && layout != 2) return 1;
  if (n < 7 || nsys < 0) return 2;
  return 0;
}

/* src/penta1bc.f:2, src/penta2bc.f:2 */
int orc_penta_bc(int layout, int n, int nsys, double* mat, double* rhs) {
  int e = check(layout, n, nsys);
  if (e) return e;
  for (int iv = 0; iv < nsys; ++iv) {
    Line_r L = {0, layout, n, n, nsys, iv, mat, rhs, NULL, NULL};
    factor_r(&L, 1, 0);
    forward_r(&L, 0, rhs, layout);
    backward_r(&L);
  }
  return 0;
}

/* Periodic set-up, src/penta2p.f:44-57 and src/cpenta1p.f:52-77: the
   wrapped blocks of rows 1, 2, n-1, n move into the fill storage. */
#define PERIODIC_SETUP(SFX, ZV)                                                          \
  static void setup_##SFX(Line_##SFX* L) {                                               \
    int n = L->n;                                                                        \
    for (int i = 1; i <= L->nrows; ++i)                                                  \
      for (int q = 0; q < 5; ++q)                                                        \
        for (int m = 0; m < 5; ++m) {                                                    \
          BV_##SFX a = perb_##SFX(L, 1, i), b = perb_##SFX(L, 2, i);                     \
          a.p[m * a.sm + q * a.sq] = ZV;                                                 \
          b.p[m * b.sm + q * b.sq] = ZV;                                                 \
          {                                                                              \
            BV_##SFX c = per2b_##SFX(L, n - 1, i), d = per2b_##SFX(L, n, i);             \
            c.p[m * c.sm + q * c.sq] = ZV;                                               \
            d.p[m * d.sm + q * d.sq] = ZV;                                               \
          }                                                                              \
        }                                                                                \
    for (int q = 0; q < 5; ++q)                                                          \
      for (int m = 0; m < 5; ++m) {                                                      \
        long o;                                                                          \
        BV_##SFX s;                                                                      \
        s = slot_##SFX(L, 1, 1); o = m * s.sm + q * s.sq;                                \
        { BV_##SFX t = perb_##SFX(L, 1, 1); t.p[m * t.sm + q * t.sq] = s.p[o]; }         \
        s = slot_##SFX(L, 1, 2); o = m * s.sm + q * s.sq;                                \
        { BV_##SFX t = perb_##SFX(L, 2, 1); t.p[m * t.sm + q * t.sq] = s.p[o]; }         \
        s = slot_##SFX(L, 2, 1); o = m * s.sm + q * s.sq;                                \
        { BV_##SFX t = perb_##SFX(L, 2, 2); t.p[m * t.sm + q * t.sq] = s.p[o]; }         \
        s = slot_##SFX(L, n - 1, 5); o = m * s.sm + q * s.sq;                            \
        { BV_##SFX t = per2b_##SFX(L, n - 1, 1); t.p[m * t.sm + q * t.sq] = s.p[o]; }    \
        s = slot_##SFX(L, n, 4); o = m * s.sm + q * s.sq;                                \
        { BV_##SFX t = per2b_##SFX(L, n, 1); t.p[m * t.sm + q * t.sq] = s.p[o]; }        \
        s = slot_##SFX(L, n, 5); o = m * s.sm + q * s.sq;                                \
        { BV_##SFX t = per2b_##SFX(L, n, 2); t.p[m * t.sm + q * t.sq] = s.p[o]; }        \
      }                                                                                  \
  }
PERIODIC_SETUP(r, 0.0)
static const ocx cx_zero = {0.0, 0.0};
PERIODIC_SETUP(c, cx_zero)

/* src/penta1p.f:2, src/penta2p.f:2.  The reference's per2(6,5,5,nsys) is a
   sliding scratch window; the oracle keeps the whole fill of rows n-1 and n
   in its own scratch (same values, different storage). */
int orc_penta_p(int layout, int np, int nsys, double* mat, double* rhs, double* per, int flags) {
  int n = np - 1;
  int e = check(layout, n, nsys);
  if (e) return e;
  double* p2 = (double*)calloc((size_t)50 * np * (nsys > 0 ? nsys : 1), sizeof(double));
  if (!p2) return 3;
  for (int iv = 0; iv < nsys; ++iv) {
    Line_r L = {1, layout, n, np, nsys, iv, mat, rhs, per, p2};
    setup_r(&L);
    factor_r(&L, 1, flags);
    forward_r(&L, 0, rhs, layout);
    backward_r(&L);
    double* r1 = rhsp_r(&L, 1);
    double* rn = rhsp_r(&L, np);
    for (int q = 0; q < 5; ++q) rn[q] = r1[q];
  }
  free(p2);
  return 0;
}

/* src/cpenta1bc.f:2, src/cpenta2bc.f:2 */
int orc_cpenta_bc(int layout, int n, int nsys, double* mat, double* rhs, int code, int flags) {
  int e = check(layout, n, nsys);
  if (e) return e;
  if (code < 0 || code > 2) return 4;
  ocx* M = (ocx*)mat;
  ocx* R = (ocx*)rhs;
  if (code == 0 || code == 2)
    OMP_FOR
    for (int iv = 0; iv < nsys; ++iv) {
      Line_c L = {0, layout, n, n, nsys, iv, M, R, NULL, NULL};
      factor_c(&L, 1, 0);
    }
  if (code == 1 || code == 2)
    OMP_FOR
    for (int iv = 0; iv < nsys; ++iv) {
      Line_c L = {0, layout, n, n, nsys, iv, M, R, NULL, NULL};
      forward_c(&L, flags, R, layout);
      backward_c(&L);
    }
  return 0;
}

/* src/cpenta1p.f:2, src/cpenta2p.f:2 */
int orc_cpenta_p(int layout, int np, int nsys, double* mat, double* rhs, double* per,
                 double* per2, int code, int flags) {
  int n = np - 1;
  int e = check(layout, n, nsys);
  if (e) return e;
  if (code < 0 || code > 2) return 4;
  ocx* M = (ocx*)mat;
  ocx* R = (ocx*)rhs;
  if (code == 0 || code == 2)
    OMP_FOR
    for (int iv = 0; iv < nsys; ++iv) {
      Line_c L = {1, layout, n, np, nsys, iv, M, R, (ocx*)per, (ocx*)per2};
      setup_c(&L);
      factor_c(&L, 1, flags);
    }
  if (code == 1 || code == 2)
    OMP_FOR
    for (int iv = 0; iv < nsys; ++iv) {
      Line_c L = {1, layout, n, np, nsys, iv, M, R, (ocx*)per, (ocx*)per2};
      forward_c(&L, 0, R, layout);
      backward_c(&L);
      ocx* r1 = rhsp_c(&L, 1);
      ocx* rn = rhsp_c(&L, np);
      for (int q = 0; q < 5; ++q) rn[q] = r1[q];
    }
  return 0;
}
