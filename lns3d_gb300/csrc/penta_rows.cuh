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

// ---------------------------------------------------------------------------
// Periodic lines (penta2p / penta1p semantics, src/penta2p.f): n = np - 1
// unknown rows; slot k of row t holds column t + k - 3, cyclically.  Rows
// 1..n-2 run as above with their normalised records spanning the columns
// [t+1, t+2, n-1, n] (merged where they meet), so row t's window holds
// columns t-2..t+2 and the two border columns n-1, n.  Rows n-1 and n,
// whose entries left of the band fill in column by column, are eliminated
// right-looking: after row c's record is stored, column c leaves both
// (their columns c..c+2 in a three-block ring, columns n-3..n fixed).
// With quirk set, row n-3's update of column n-1 from pivot row n-5 lands in
// column n-2, as the reference's factorisation places it (src/penta2p.f:278,
// 339); the solution's row np repeats row 1.
struct PArgs {
  const double* mat;
  double* rhs;
  double* work;          // kRec doubles per row and line
  int n, nsys;           // unknown rows (np - 1), lines
  long long row_stride, line_stride;
  int quirk;
  int* status;
};

struct PSmem {
  double raw[2][130];
  // window blocks of columns t-2, t-1, t, t+1, t+2, n-1, n (W[25 w + 5 a + b],
  // a column in two roles kept once: in block 5 or 6), r at 175
  double W[180];
  double G[180];
  double ring[4][kRec];
  double bot[2][7][25];  // rows n-1, n: columns c..c+2 at c % 3, columns n-3..n at 3..6
  double brhs[2][5];
  double xs[4][5];       // back substitution: rows t+1, t+2
  double xf[2][5];       // x_{n-1}, x_n
};

__device__ __forceinline__ int gjp_at(int j, int col) {
  return col < 25 ? 25 * (2 + col / 5) + 5 * j + col % 5 : 175 + j;
}

__global__ void __launch_bounds__(kThreads) rows_p_kernel(PArgs a) {
  __shared__ PSmem S;
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
  // slot (1..5) of row t holding column col, or 0
  auto slot_of = [&](int t, int col) {
    int k = col - t + 3;
    if (k < 1) k += n;
    if (k > n) k -= n;
    return k >= 1 && k <= 5 ? k : 0;
  };
  // the record's block s covers column target(c, s), or 0 when merged away
  auto target = [&](int c, int s) {
    if (s == 0) return c + 1 < n - 1 ? c + 1 : 0;
    if (s == 1) return c + 2 < n - 1 ? c + 2 : 0;
    return s == 2 ? n - 1 : n;
  };
  auto widx = [&](int t, int col) { return col == n - 1 ? 5 : col == n ? 6 : col - t + 2; };
  auto bidx = [&](int col) { return col >= n - 3 ? 3 + col - (n - 3) : col % 3; };
  // per-thread roles
  const int d0 = tid / 25, ar = tid < 100 ? (tid % 25) / 5 : tid - 100, eb = tid % 5;
  const int gj0 = tid / 26, gc0 = tid % 26, ga0 = gjp_at(gj0, gc0);
  const int gj1 = 4, gc1 = 24 + tid, ga1 = tid < 2 ? gjp_at(gj1, gc1) : 0;
  auto roff = [](int j, int col) { return col < 25 ? 25 * ((col - 5) / 5) + 5 * j + (col - 5) % 5 : 100 + j; };

  // rows n-1 and n start in the bottom storage
  for (int e = tid; e < 350; e += kThreads) (&S.bot[0][0][0])[e] = 0.0;
  __syncthreads();
  for (int e = tid; e < 260; e += kThreads) {
    const int b = e / 130, x = e % 130, t = n - 1 + b;
    const double val = a.mat[125 * rec(t) + (x < 125 ? x : 0)];
    if (x < 125) {
      const int k = x % 5 + 1, m = (x / 5) % 5, q = x / 25;
      int col = t + k - 3;
      if (col > n) col -= n;
      S.bot[b][bidx(col)][5 * m + q] = val;
    } else {
      S.brhs[b][x - 125] = a.rhs[5 * rec(t) + x - 125];
    }
  }

  // Gauss-Jordan of the prepared window, then [U_t | z_t] into the ring and work
  auto normalise = [&](int t) {
    double* cur = S.W;
    double* nxt = S.G;
#pragma unroll 1
    for (int k = 0; k < 5; ++k) {
      const double piv = cur[gjp_at(k, k)];
      if (gc0 > k) {
        const double g = cur[ga0];
        nxt[ga0] = gj0 == k ? g : fma(-cur[gjp_at(gj0, k)], cur[gjp_at(k, gc0)], g * piv);
      }
      if (tid < 2) {
        const double g = cur[ga1];
        nxt[ga1] = k == 4 ? g : fma(-cur[gjp_at(gj1, k)], cur[gjp_at(k, gc1)], g * piv);
      }
      if (tid < k) nxt[gjp_at(tid, tid)] = cur[gjp_at(tid, tid)] * piv;
      if (tid == k) nxt[gjp_at(k, k)] = piv;
      double* sw = cur;
      cur = nxt;
      nxt = sw;
      __syncthreads();
    }
    double* R = S.ring[(t - 1) & 3];
    double* gw = work + (long long)(t - 1) * kRec;
    if (gc0 >= 5) {
      const double dj = cur[gjp_at(gj0, gj0)];
      if (gc0 == 25 && !(fabs(dj) > 0.0 && isfinite(dj)) && a.status) atomicExch(a.status, 1);
      const double val = cur[ga0] * recip(dj);
      const int off = roff(gj0, gc0);
      R[off] = val;
      gw[off] = val;
    }
    if (tid < 2) {
      const double dj = cur[gjp_at(gj1, gj1)];
      if (tid == 1 && !(fabs(dj) > 0.0 && isfinite(dj)) && a.status) atomicExch(a.status, 1);
      const double val = cur[ga1] * recip(dj);
      const int off = roff(gj1, gc1);
      R[off] = val;
      gw[off] = val;
    }
    __syncthreads();
  };

  load_raw(1, 0);
  for (int t = 1; t <= n - 2; ++t) {
    const int buf = (t - 1) & 1;
    cp_wait_all();
    __syncthreads();
    // the window: block w covers column t + w - 2 (w < 5, cyclically) or n-1, n
    for (int e = tid; e < 180; e += kThreads) {
      double val;
      if (e < 175) {
        const int w = e / 25, ab = e % 25;
        int col = w == 5 ? n - 1 : w == 6 ? n : t + w - 2;
        if (col < 1) col += n;
        const bool own = w >= 5 || (col != n - 1 && col != n);
        const int k = own ? slot_of(t, col) : 0;
        val = k ? S.raw[buf][(k - 1) + 5 * (ab / 5) + 25 * (ab % 5)] : 0.0;
      } else {
        val = S.raw[buf][125 + e - 175];
      }
      S.W[e] = val;
    }
    __syncthreads();
    if (t < n - 2) load_raw(t + 1, buf ^ 1);
    // eliminate columns t-2, t-1
    for (int c = t - 2; c < t; ++c) {
      if (c < 1) continue;
      const double* U = S.ring[(c - 1) & 3];
      const double* L = S.W + 25 * (c - t + 2);
      int col = tid < 100 ? target(c, d0) : 1;
      if (tid < 100 && a.quirk && t == n - 3 && c == n - 5 && d0 == 2) col = n - 2;
      if (tid < 100 ? col > 0 : tid < 105) {
        const int at = tid < 100 ? 25 * widx(t, col) + 5 * ar + eb : 175 + ar;
        const int ub = tid < 100 ? 25 * d0 + eb : 100;
        const int us = tid < 100 ? 5 : 1;
        double acc = S.W[at];
#pragma unroll
        for (int q = 0; q < 5; ++q) acc = fma(-L[5 * ar + q], U[ub + us * q], acc);
        S.W[at] = acc;
      }
      __syncthreads();
    }
    normalise(t);
    // column t leaves rows n-1 and n
    {
      const double* R = S.ring[(t - 1) & 3];
      for (int o = tid; o < 210; o += kThreads) {
        const int b = o / 105, oo = o % 105;
        const double* L = S.bot[b][bidx(t)];
        if (oo < 100) {
          const int s = oo / 25, r5 = (oo % 25) / 5, c5 = oo % 5, col = target(t, s);
          if (col > 0) {
            double* dst = &S.bot[b][bidx(col)][5 * r5 + c5];
            double acc = *dst;
#pragma unroll
            for (int q = 0; q < 5; ++q) acc = fma(-L[5 * r5 + q], R[25 * s + 5 * q + c5], acc);
            *dst = acc;
          }
        } else {
          const int r5 = oo - 100;
          double acc = S.brhs[b][r5];
#pragma unroll
          for (int q = 0; q < 5; ++q) acc = fma(-L[5 * r5 + q], R[100 + q], acc);
          S.brhs[b][r5] = acc;
        }
      }
      __syncthreads();
      // column t's ring slot will hold column t + 3
      if (t < n - 3 && tid < 50) S.bot[tid / 25][t % 3][tid % 25] = 0.0;
    }
  }
  // row n-1: [C | block n | r] from the bottom storage
  for (int e = tid; e < 180; e += kThreads) {
    const int w = e / 25, ab = e % 25;
    double val = 0.0;
    if (e >= 175) val = S.brhs[0][e - 175];
    else if (w == 2) val = S.bot[0][5][ab];
    else if (w == 6) val = S.bot[0][6][ab];
    S.W[e] = val;
  }
  __syncthreads();
  normalise(n - 1);
  // row n: column n-1 leaves it, then [C | r]
  {
    const double* R = S.ring[(n - 2) & 3];
    const double* L = S.bot[1][5];
    if (tid < 30) {
      const int r5 = tid < 25 ? tid / 5 : tid - 25, c5 = tid % 5;
      double acc = tid < 25 ? S.bot[1][6][5 * r5 + c5] : S.brhs[1][r5];
#pragma unroll
      for (int q = 0; q < 5; ++q) acc = fma(-L[5 * r5 + q], tid < 25 ? R[75 + 5 * q + c5] : R[100 + q], acc);
      if (tid < 25) S.bot[1][6][5 * r5 + c5] = acc;
      else S.brhs[1][r5] = acc;
    }
    __syncthreads();
    for (int e = tid; e < 180; e += kThreads) {
      const int w = e / 25, ab = e % 25;
      double val = 0.0;
      if (e >= 175) val = S.brhs[1][e - 175];
      else if (w == 2) val = S.bot[1][6][ab];
      S.W[e] = val;
    }
    __syncthreads();
    normalise(n);
  }
  // back substitution, rows n..1
  const int a5 = tid >> 4, p = tid & 15;
  auto load_rec = [&](int t, int buf) {
    const double* src = work + (long long)(t - 1) * kRec;
    for (int e = tid; e < kRec; e += kThreads) cp_async8(&S.raw[buf][e], src + e);
    cp_commit();
  };
  auto xat = [&](int col) -> double* { return col >= n - 1 ? S.xf[col - (n - 1)] : S.xs[(col - 1) & 3]; };
  load_rec(n, 0);
  for (int t = n; t >= 1; --t) {
    const int buf = (n - t) & 1;
    cp_wait_all();
    __syncthreads();
    if (t > 1) load_rec(t - 1, buf ^ 1);
    double part = 0.0;
    if (a5 < 5) {
      for (int term = p; term < 20; term += 16) {
        const int s = term / 5, q = term % 5;
        const int col = t <= n - 2 ? target(t, s) : (t == n - 1 && s == 3 ? n : 0);
        if (col > 0) part = fma(S.raw[buf][25 * s + 5 * a5 + q], xat(col)[q], part);
      }
    }
    for (int sh = 8; sh > 0; sh >>= 1) part += __shfl_down_sync(0xffffffffu, part, sh, 16);
    __syncthreads();
    if (a5 < 5 && p == 0) {
      const double x = S.raw[buf][100 + a5] - part;
      xat(t)[a5] = x;
      a.rhs[5 * rec(t) + a5] = x;
      if (t == 1) a.rhs[5 * rec(n + 1) + a5] = x;  // the periodic image, row np
    }
  }
}

}  // namespace rows
}  // namespace lns
