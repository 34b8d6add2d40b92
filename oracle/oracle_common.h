/*
 * Definitions shared by the oracle's step restatements (adi3d_oracle.c,
 * impdrv2d_oracle.c).  TEST INFRASTRUCTURE ONLY.
 */
#pragma once

/* src/stencil.f90:10-94 (the reference's coefficient table) */
/* Line and row loops are independent; the timing build (-fopenmp) runs them
   in parallel, the parity build (no -fopenmp) serially.  The residual sum
   stays serial so its order is the same in both. */
#ifdef _OPENMP
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#else
#define OMP_FOR
#endif

static const double ga1 = 8.333333333333333333333E-02, ga2 = -6.666666666666666666667E-01,
                    ga3 = 6.666666666666666666667E-01, ga4 = -8.333333333333333333333E-02;
static const double gc1 = -2.083333333333333333333E+00, gc2 = 4.000000000000000000000E+00,
                    gc3 = -3.000000000000000000000E+00, gc4 = 1.333333333333333333333E+00,
                    gc5 = -2.500000000000000000000E-01;
static const double gb1 = -2.500000000000000000000E-01, gb2 = -8.333333333333333333333E-01,
                    gb3 = 1.500000000000000000000E+00, gb4 = -5.000000000000000000000E-01,
                    gb5 = 8.333333333333333333333E-02;
static const double da1 = -8.333333333333333333333E-02, da2 = 1.333333333333333333333E+00,
                    da3 = -2.500000000000000000000E+00, da4 = 1.333333333333333333333E+00,
                    da5 = -8.333333333333333333333E-02;
static const double db1 = 9.166666666666666666667E-01, db2 = -1.666666666666666666667E+00,
                    db3 = 5.000000000000000000000E-01, db4 = 3.333333333333333333333E-01,
                    db5 = -8.333333333333333333333E-02;
static const double dd1 = 2.916666666666666666667E+00, dd2 = -8.666666666666666666667E+00,
                    dd3 = 9.500000000000000000000E+00, dd4 = -4.666666666666666666667E+00,
                    dd5 = 9.166666666666666666667E-01;
/* src/global.f90:2-15 */
static const double zero = 0.0, pt5 = 5.0000000000000000000e-1, pt66 = 6.6666666666666666666e-1,
                    one = 1.0, two = 2.0, four = 4.0;

#define IX(g, i, j) ((long)((i) - 1) + (long)(g)->nx * ((j) - 1))
#define FV(v, nc, c, g, i, j) (v)[(long)(c) + (long)(nc) * IX(g, i, j)]
