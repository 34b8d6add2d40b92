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

// Gauss-Jordan on [C | four blocks | r] held in a window layout: block
// column col / 5 of the right part at DB + 25 (col / 5), the right-hand side
// at RB.  Thread roles: entry (tid / 26, tid % 26), and for threads 0 and 1
// also (4, 24 + tid); addresses fixed for the line.
template <int DB, int RB>
struct GjRoles {
  int j0, c0, a0, k0, p0, s0;  // own entry; (j0, 0); (0, c0); row stride of column c0
  int a1, k1, p1, s1;
  static __device__ __forceinline__ int at(int j, int col) {
    return col < 25 ? DB + 25 * (col / 5) + 5 * j + col % 5 : RB + j;
  }
  __device__ explicit GjRoles(int tid) {
    j0 = tid / 26;
    c0 = tid % 26;
    a0 = at(j0, c0);
    k0 = DB + 5 * j0;
    p0 = at(0, c0);
    s0 = c0 < 25 ? 5 : 1;
    const int c1 = 24 + tid;
    a1 = tid < 2 ? at(4, c1) : 0;
    k1 = DB + 20;
    p1 = tid < 2 ? at(0, c1) : 0;
    s1 = c1 < 25 ? 5 : 1;
  }
};

// Five division-free steps: each scales the other rows by the pivot and
// subtracts the pivot row; the rows already pivoted keep only their
// diagonal, scaled too.  Returns the buffer holding the result.
template <int DB, int RB>
__device__ __forceinline__ double* gauss_jordan(double* cur, double* nxt, const GjRoles<DB, RB>& g, int tid) {
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const double piv = cur[DB + 6 * k];
    if (g.c0 > k) {
      const double x = cur[g.a0];
      nxt[g.a0] = g.j0 == k ? x : fma(-cur[g.k0 + k], cur[g.p0 + g.s0 * k], x * piv);
    }
    if (tid < 2) {
      const double x = cur[g.a1];
      nxt[g.a1] = k == 4 ? x : fma(-cur[g.k1 + k], cur[g.p1 + g.s1 * k], x * piv);
    }
    if (tid < k) nxt[DB + 6 * tid] = cur[DB + 6 * tid] * piv;
    if (tid == k) nxt[DB + 6 * k] = piv;
    double* sw = cur;
    cur = nxt;
    nxt = sw;
    __syncthreads();
  }
  return cur;
}

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
  const GjRoles<100, 225> gr(tid);
  const int gj0 = gr.j0, gc0 = gr.c0, ga0 = gr.a0, gj1 = 4, gc1 = 24 + tid, ga1 = gr.a1;
  auto roff = [](int j, int col) { return col < 25 ? 25 * ((col - 5) / 5) + 5 * j + (col - 5) % 5 : 100 + j; };
  const int off0 = roff(gj0, gc0 < 5 ? 5 : gc0), off1 = roff(gj1, gc1);

  // the window of row t from its record in raw buffer (t - 1) & 1
  auto build_window = [&](int t) {
    const int buf = (t - 1) & 1;
    const int olo = lo_col(t, n) - t + 4;  // the row holds block columns olo..olo+4
    S.W[we0] = (wo0 >= olo && wo0 <= olo + 4) ? S.raw[buf][src0] : 0.0;
    if (we1 < 230) S.W[we1] = we1 >= 225 || (wo1 >= olo && wo1 <= olo + 4) ? S.raw[buf][src1] : 0.0;
  };

  // Row t's window is built in row t-1's last segment, while row t+1's
  // record is on its way: per row, the eliminations, five Gauss-Jordan
  // steps and the store, each closed by one barrier.
  load_raw(1, 0);
  cp_wait_all();
  __syncthreads();
  build_window(1);
  if (n > 1) load_raw(2, 1);
  __syncthreads();
  for (int t = 1; t <= n; ++t) {
    const int lo = lo_col(t, n);
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
    cp_wait_all();  // row t+1's record, visible after the Gauss-Jordan barriers
    double* cur = gauss_jordan(S.W, S.G, gr, tid);
    // divide by the accumulated diagonals; store [U_t | z_t]; the window of
    // row t+1 (W is free: the result is in G)
    double* R = S.ring[(t - 1) & 3];
    double* gw = work + (long long)(t - 1) * kRec;
    if (t < n) {
      build_window(t + 1);
      if (t + 1 < n) load_raw(t + 2, (t + 1) & 1);
    }
    if (gc0 >= 5) {
      const double dj = cur[100 + 6 * gj0];
      if (gc0 == 25 && !(fabs(dj) > 0.0 && isfinite(dj)) && a.status) atomicExch(a.status, 1);
      const double val = cur[ga0] * recip(dj);
      R[off0] = val;
      gw[off0] = val;
    }
    if (tid < 2) {
      const double dj = cur[100 + 6 * gj1];
      if (tid == 1 && !(fabs(dj) > 0.0 && isfinite(dj)) && a.status) atomicExch(a.status, 1);
      const double val = cur[ga1] * recip(dj);
      R[off1] = val;
      gw[off1] = val;
    }
    __syncthreads();
  }
  // back substitution, rows n..1: the records of row t-1 prefetched during row t
  const int a5 = tid >> 4, p = tid & 15;  // unknown a5 (< 5), its 16-lane group
  const int dA = p / 5 + 1, qA = p % 5, dB = (p + 16) / 5 + 1, qB = (p + 16) % 5;
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
    if (a5 < 5) {  // terms p and p + 16 of sum_d U_t[d] x_{t+d}: block dA / dB, entry qA / qB
      if (p < 5 * w) part = S.raw[buf][25 * (dA - 1) + 5 * a5 + qA] * S.xs[(t + dA - 1) & 3][qA];
      if (p + 16 < 5 * w) part = fma(S.raw[buf][25 * (dB - 1) + 5 * a5 + qB], S.xs[(t + dB - 1) & 3][qB], part);
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
  const GjRoles<50, 175> gr(tid);
  const int gj0 = gr.j0, gc0 = gr.c0, ga0 = gr.a0, gj1 = 4, gc1 = 24 + tid, ga1 = gr.a1;
  auto roff = [](int j, int col) { return col < 25 ? 25 * ((col - 5) / 5) + 5 * j + (col - 5) % 5 : 100 + j; };
  const int off0 = roff(gj0, gc0 < 5 ? 5 : gc0), off1 = roff(gj1, gc1);

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
    double* cur = gauss_jordan(S.W, S.G, gr, tid);
    double* R = S.ring[(t - 1) & 3];
    double* gw = work + (long long)(t - 1) * kRec;
    if (gc0 >= 5) {
      const double dj = cur[50 + 6 * gj0];
      if (gc0 == 25 && !(fabs(dj) > 0.0 && isfinite(dj)) && a.status) atomicExch(a.status, 1);
      const double val = cur[ga0] * recip(dj);
      R[off0] = val;
      gw[off0] = val;
    }
    if (tid < 2) {
      const double dj = cur[50 + 6 * gj1];
      if (tid == 1 && !(fabs(dj) > 0.0 && isfinite(dj)) && a.status) atomicExch(a.status, 1);
      const double val = cur[ga1] * recip(dj);
      R[off1] = val;
      gw[off1] = val;
    }
    __syncthreads();
  };

  // the window of row t from raw buffer (t - 1) & 1: block w covers column
  // t + w - 2 (w < 5, cyclically) or n-1, n
  auto build_window = [&](int t) {
    const int buf = (t - 1) & 1;
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
  };

  // as in rows_bc_kernel, row t's window is built in row t-1's last
  // segment (here beside the elimination of column t-1 from the last rows)
  load_raw(1, 0);
  cp_wait_all();
  __syncthreads();
  build_window(1);
  if (n - 2 > 1) load_raw(2, 1);
  __syncthreads();
  for (int t = 1; t <= n - 2; ++t) {
    // column t-1's ring slot in the last rows will hold column t + 2
    if (t - 1 >= 1 && t - 1 < n - 3 && tid < 50) S.bot[tid / 25][(t - 1) % 3][tid % 25] = 0.0;
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
    cp_wait_all();  // row t+1's record, visible after the Gauss-Jordan barriers
    normalise(t);
    // column t leaves rows n-1 and n; the window of row t+1 (W is free)
    {
      if (t < n - 2) {
        build_window(t + 1);
        if (t + 1 < n - 2) load_raw(t + 2, (t + 1) & 1);
      }
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
  const int sA = p / 5, qA = p % 5, qB = (p + 16) % 5;  // term p + 16 (p < 4) lies in block 3
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
    if (a5 < 5) {  // terms p and p + 16 of sum_s U_t[s] x_{target(s)}
      const int colA = t <= n - 2 ? target(t, sA) : (t == n - 1 && sA == 3 ? n : 0);
      if (colA > 0) part = S.raw[buf][25 * sA + 5 * a5 + qA] * xat(colA)[qA];
      if (p < 4) {
        const int colB = t <= n - 2 ? target(t, 3) : (t == n - 1 ? n : 0);
        if (colB > 0) part = fma(S.raw[buf][75 + 5 * a5 + qB], xat(colB)[qB], part);
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
