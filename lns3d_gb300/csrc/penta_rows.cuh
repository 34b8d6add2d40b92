// Block-row elimination of real block-pentadiagonal lines with boundary-
// closure rows (penta2bc / penta1bc semantics, src/penta2bc.f), for the
// solves of the nonlinear 2D step, whose LHS is formed and factored anew
// every corrector.
//
// The reference eliminates one scalar pivot at a time.  Here a CTA of 128
// threads owns one line and works on whole 5x5 blocks, so each block row
// costs a few dependent FP64 operations per stage instead of a chain of
// scalar pivots each closed by a barrier:
//   load      row t's five blocks into a window of nine block columns
//             (offsets -4..4 from the diagonal; rows 1, 2, n-1, n hold the
//             further nodes of their one-sided stencils in the free slots);
//   eliminate the blocks left of the diagonal, column by column, with the
//             normalised rows stored for the rows above
//             (row_t -= L_c [I U_c | z_c], one thread per output entry);
//   normalise the diagonal block by Gauss-Jordan without divisions: each
//             step scales the other rows by the pivot and subtracts the
//             pivot row, so a step is two dependent operations, and the
//             rows are divided by their accumulated diagonals once at the
//             end (one Newton-refined reciprocal per row);
//   store     [U_t | z_t] for the rows below and for back substitution.
// Back substitution x_t = z_t - sum_d U_t[d] x_{t+d} runs in reverse with
// one 16-lane group per unknown.  The elimination is the reference's
// unpivoted LU reordered, so results agree with the reference to rounding.
#pragma once
#include <cuda_runtime.h>

namespace lns {
namespace rows {

constexpr int kThreads = 128;   // one line per CTA
constexpr int kRec = 105;       // per row: U blocks for columns t+1..t+4 (4 x 25) and z (5)

struct Args {
  const double* mat;     // mat(5,5,5) records in the reference layout
  double* rhs;           // rhs(5) records: the right-hand side in, the solution out
  double* work;          // kRec doubles per row and line
  int n, nsys;
  long long row_stride, line_stride;  // in records
  int* status;           // set to 1 on a zero or non-finite diagonal
};

__device__ __forceinline__ int mod5(int x) { return ((x % 5) + 5) % 5; }
// first column held by row t (rows hold five consecutive columns)
__device__ __forceinline__ int lo_col(int t, int n) { return min(max(t - 2, 1), n - 4); }

// 1/d by Newton-Raphson from the single-precision reciprocal: each step
// x <- x + x (1 - d x) doubles the correct bits (24 -> 48 -> 96)
__device__ __forceinline__ double recip(double d) {
  const float f = (float)d;
  double x = (double)__frcp_rn(f);
  if (!(fabs(x) < 1e300) || x == 0.0) return 1.0 / d;  // outside single-precision range
  double e = fma(-d, x, 1.0);
  x = fma(x, e, x);
  e = fma(-d, x, 1.0);
  return fma(x, e, x);
}

__device__ __forceinline__ void cp_async8(double* dst, const double* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

struct Smem {
  double raw[2][130];          // prefetched records: 125 matrix entries (reference order) and 5 rhs
  // the row's window of block columns, W[25 o + 5 a + b] (o = column - t + 4),
  // then its right-hand side at 225; from the diagonal on (o >= 4) it is one
  // of the two Gauss-Jordan buffers
  double W[230];
  double G[230];               // the other buffer, same layout
  double ring[4][kRec];        // [U | z] of the last four rows
  double xs[4][5];             // back substitution: the last four solutions
};

// Gauss-Jordan entry (row j, column col) of [C | blocks t+1..t+4 | r] in
// the window layout
__device__ __forceinline__ int gj_at(int j, int col) {
  return col < 25 ? 25 * (4 + col / 5) + 5 * j + col % 5 : 225 + j;
}

__global__ void __launch_bounds__(kThreads) rows_bc_kernel(Args a) {
  __shared__ Smem S;
  const int iv = blockIdx.x;
  if (iv >= a.nsys) return;
  const int tid = threadIdx.x, n = a.n;
  auto rec = [&](int t) { return a.row_stride * (t - 1) + a.line_stride * iv; };
  double* work = a.work + (long long)iv * n * kRec;
  auto load_raw = [&](int t, int buf) {
    const double* gm = a.mat + 125 * rec(t);
    for (int e = tid; e < 125; e += kThreads) cp_async8(&S.raw[buf][e], gm + e);
    if (tid < 5) cp_async8(&S.raw[buf][125 + tid], a.rhs + 5 * rec(t) + tid);
    cp_commit();
  };
  // per-thread roles, fixed for the whole line.  Window entries e = tid and
  // tid + 128: block column o holds slot mod5(o - 2) + 1 of the record
  // whatever the row (column t + o - 4 has slot mod5(c - t + 2) + 1).
  const int we0 = tid, we1 = tid + kThreads;
  const int wo0 = we0 / 25, wo1 = we1 / 25;
  const int src0 = mod5(wo0 - 2) + 5 * ((we0 % 25) / 5) + 25 * (we0 % 5);
  const int src1 = we1 < 225 ? mod5(wo1 - 2) + 5 * ((we1 % 25) / 5) + 25 * (we1 % 5) : 125 + we1 - 225;
  // elimination output: block d0 (column c + d0 + 1), entry (ar, eb); r[ar] for threads 100..104
  const int d0 = tid / 25, ar = tid < 100 ? (tid % 25) / 5 : tid - 100, eb = tid % 5;
  // Gauss-Jordan entries e = tid (all threads) and tid + 128 (two threads)
  const int gj0 = tid / 26, gc0 = tid % 26, ga0 = gj_at(gj0, gc0);
  const int gj1 = 4, gc1 = 24 + tid, ga1 = tid < 2 ? gj_at(gj1, gc1) : 0;
  auto roff = [](int j, int col) { return col < 25 ? 25 * ((col - 5) / 5) + 5 * j + (col - 5) % 5 : 100 + j; };

  load_raw(1, 0);
  for (int t = 1; t <= n; ++t) {
    const int buf = (t - 1) & 1;
    cp_wait_all();
    __syncthreads();
    const int lo = lo_col(t, n), olo = lo - t + 4;  // the row holds block columns olo..olo+4
    S.W[we0] = (wo0 >= olo && wo0 <= olo + 4) ? S.raw[buf][src0] : 0.0;
    if (we1 < 230) S.W[we1] = we1 >= 225 || (wo1 >= olo && wo1 <= olo + 4) ? S.raw[buf][src1] : 0.0;
    __syncthreads();
    if (t < n) load_raw(t + 1, buf ^ 1);
    // eliminate the columns left of the diagonal, ascending
    for (int c = lo; c < t; ++c) {
      const int wc = lo_col(c, n) + 4 - c;  // row c's normalised part spans c+1..c+wc
      const double* U = S.ring[(c - 1) & 3];
      const double* L = S.W + 25 * (c - t + 4);
      if (tid < 100 ? d0 < wc : tid < 105) {
        const int at = tid < 100 ? 25 * (c + d0 + 1 - t + 4) + 5 * ar + eb : 225 + ar;
        const int ub = tid < 100 ? 25 * d0 + eb : 100;
        const int us = tid < 100 ? 5 : 1;
        double acc = S.W[at];
#pragma unroll
        for (int q = 0; q < 5; ++q) acc = fma(-L[5 * ar + q], U[ub + us * q], acc);
        S.W[at] = acc;
      }
      __syncthreads();
    }
    // Gauss-Jordan on [C | blocks t+1..t+4 | r] (zero blocks past the row's
    // reach stay zero) without divisions, ping-pong between W and G
    double* cur = S.W;
    double* nxt = S.G;
#pragma unroll 1
    for (int k = 0; k < 5; ++k) {
      const double piv = cur[gj_at(k, k)];
      if (gc0 > k) {
        const double g = cur[ga0];
        nxt[ga0] = gj0 == k ? g : fma(-cur[gj_at(gj0, k)], cur[gj_at(k, gc0)], g * piv);
      }
      if (tid < 2) {
        const double g = cur[ga1];
        nxt[ga1] = k == 4 ? g : fma(-cur[gj_at(gj1, k)], cur[gj_at(k, gc1)], g * piv);
      }
      // the diagonals of the rows already pivoted, which the step scales by
      // the pivot (their entry in the pivot row's column is zero), and the
      // pivot row's own
      if (tid < k) nxt[gj_at(tid, tid)] = cur[gj_at(tid, tid)] * piv;
      if (tid == k) nxt[gj_at(k, k)] = piv;
      double* sw = cur;
      cur = nxt;
      nxt = sw;
      __syncthreads();
    }
    // divide by the accumulated diagonals; store [U_t | z_t]
    double* R = S.ring[(t - 1) & 3];
    double* gw = work + (long long)(t - 1) * kRec;
    if (gc0 >= 5) {
      const double dj = cur[gj_at(gj0, gj0)];
      if (gc0 == 25 && !(fabs(dj) > 0.0 && isfinite(dj)) && a.status) atomicExch(a.status, 1);
      const double val = cur[ga0] * recip(dj);
      const int off = roff(gj0, gc0);
      R[off] = val;
      gw[off] = val;
    }
    if (tid < 2) {
      const double dj = cur[gj_at(gj1, gj1)];
      if (tid == 1 && !(fabs(dj) > 0.0 && isfinite(dj)) && a.status) atomicExch(a.status, 1);
      const double val = cur[ga1] * recip(dj);
      const int off = roff(gj1, gc1);
      R[off] = val;
      gw[off] = val;
    }
    __syncthreads();
  }
  // back substitution, rows n..1: the records of row t-1 prefetched during row t
  const int a5 = tid >> 4, p = tid & 15;  // unknown a5 (< 5), its 16-lane group
  auto load_rec = [&](int t, int buf) {
    const double* src = work + (long long)(t - 1) * kRec;
    for (int e = tid; e < kRec; e += kThreads) cp_async8(&S.raw[buf][e], src + e);
    cp_commit();
  };
  load_rec(n, 0);
  for (int t = n; t >= 1; --t) {
    const int buf = (n - t) & 1;
    cp_wait_all();
    __syncthreads();
    if (t > 1) load_rec(t - 1, buf ^ 1);
    const int w = lo_col(t, n) + 4 - t;
    double part = 0.0;
    if (a5 < 5) {
      for (int term = p; term < 5 * w; term += 16) {
        const int d = term / 5 + 1, q = term % 5;
        part = fma(S.raw[buf][25 * (d - 1) + 5 * a5 + q], S.xs[(t + d - 1) & 3][q], part);
      }
    }
    for (int s = 8; s > 0; s >>= 1) part += __shfl_down_sync(0xffffffffu, part, s, 16);
    __syncthreads();  // every read of xs for row t is done before row t's value replaces row t+4's
    if (a5 < 5 && p == 0) {
      const double x = S.raw[buf][100 + a5] - part;
      S.xs[(t - 1) & 3][a5] = x;
      a.rhs[5 * rec(t) + a5] = x;
    }
  }
}

}  // namespace rows
}  // namespace lns
