// Sweeps of the 3D step on factors kept in a scaled block form.
//
// The line solvers factor A = L U in the reference's storage
// (src/cpenta1bc.f:52-498, src/cpenta2p.f): per row i the stored lower
// blocks S_ic (applied as y_i += S_ic y_c), the in-block LU of the diagonal
// block D_i = L_ii U_ii, and the upper blocks T_ic (x_i -= T_ic x_c).  With
//     yh_i = U_ii^-1 y_i,   s_i = D_i^-1 r_i,
//     F_ic = -D_i^-1 S_ic U_cc,   B_ic = U_ii^-1 T_ic,
// the two triangular solves become
//     forward   yh_i = s_i - sum_c F_ic yh_c
//     backward  x_i  = yh_i - sum_c B_ic x_c
// so a row of either recurrence is two (at the boundary rows up to four)
// dense 5x5 block-vector products and nothing else: no in-block
// substitution, no division.  The products of a row are spread over 25
// lanes of a warp, lane l = m + 5 q owning entry (m, q); the sum over q is a
// gather of five shuffles.  s_i = D_i^-1 r_i and, for periodic lines, the
// fill of rows n-1, n (columns n-1, n) are independent of the recurrence and
// run as point-parallel kernels around it.
//
// Internal record of row i (125 entries, block-major, entry (m, q) of a
// block at m + 5 q):
//   block 0  D_i^-1
//   blocks 1..4 by row type (F_d: column i-d, B_d: column i+d)
//     rows 3..n-2     F1 F2 B1 B2          row 1    B3 B4 B1 B2
//     row 2           F1 B3 B1 B2          row n-1  F1 F2 B1 F3
//     row n           F1 F2 F3 F4          periodic lines: F1 F2 B1 B2 on
//                                          every row, absent blocks zero
// Periodic lines are solved bordered: with the unknowns split into the band
// rows 1..n-2 (A11, whose factors are the records of those rows) and the
// border rows n-1, n, [A11 A12; A21 A22] [x1; x2] = [b1; b2] gives
//   z = A11^-1 b1 (the two recurrences, border terms left out),
//   x2 = S^-1 (b2 - A21 z), S = A22 - A21 W, W = A11^-1 A12,
//   x1 = z - W x2,
// where W (ten columns, 50 entries per record, in the fill array), S^-1 and
// the six non-zero blocks of A21 are formed once, at factoring time.  A21
// reaches only rows 1, 2, n-3, n-2 of z, so the border needs no sum over the
// line.
// The prep kernels read the factors in one precision (TM) and write the
// internal form in the precision of the sweeps (TC), computing in FP64.
#pragma once
#include <type_traits>

#include "penta_direct.cuh"

namespace lns {
namespace chain {

struct Args {
  const void* mat;   // factored records, reference storage (prep only)
  void* chn;         // internal records
  const void* per;   // periodic fill in the reference storage (prep only)
  const void* per2;
  void* fillE;       // periodic lines: W, 50 entries per record (may alias per)
  void* rhs;
  int n;             // unknowns per line (periodic: np - 1)
  int nsys;
  long long row_stride, line_stride;
  // periodic lines: kBordCd complex doubles per line (see kBordCd)
  void* bord = nullptr;
  // FP64 periodic lines solved in row pairs: 50 entries per record (see
  // pair_prep_kernel); null for lines solved row by row
  void* pairs = nullptr;
};

// Border data of a periodic line: S^-1 (row k, column j at k + 10 j; k, j =
// m + 5 b for component m of border row n-1+b), the six blocks of A21 (rows
// n-1: columns n-3, n-2, 1; row n: columns n-2, 1, 2; entry (m, q) at
// m + 5 q), and the sixteen border blocks of the unfactored LHS, kept from
// before the factorisation until W and S are formed.
constexpr int kBordSinv = 0, kBordA21 = 100, kBordRaw = 250, kBordCd = 650;

__device__ __forceinline__ long long rec_of(const Args& a, int r, int iv) {
  return a.row_stride * (r - 1) + a.line_stride * iv;
}

// ------------------------------------------------------------------- prep
// Warp-per-record helpers (FP64 arithmetic whatever the storage type).
__device__ __forceinline__ cd ld_cd(const cd* p) { return *p; }
__device__ __forceinline__ cd ld_cd(const cf* p) { return cd{(double)p->x, (double)p->y}; }
__device__ __forceinline__ void st_t(cd* p, cd v) { *p = v; }
__device__ __forceinline__ void st_t(cf* p, cd v) { *p = cf{(float)v.x, (float)v.y}; }

// C = A * B for 5x5 blocks in shared memory (entry (m,q) at m + 5 q), lane
// l < 25 computes entry l.  `upperB` skips the zero lower part of B.
__device__ __forceinline__ cd mm5(const cd* A, const cd* B, int m, int q, bool upperB) {
  cd acc{0.0, 0.0};
#pragma unroll
  for (int k = 0; k < 5; ++k)
    if (!upperB || k <= q) acc = fmac(acc, A[m + 5 * k], B[k + 5 * q]);
  return acc;
}

constexpr int kPrepWarps = 4;
// per-warp shared memory of the prep kernels, in cd units
constexpr int kPrepSm = 7 * 25;

// Position of the block of column offset d (-4..4, d != 0) in the internal
// record of row i, or -1 when the row holds no such block.
__device__ __forceinline__ int pos_bc(int i, int n, int d) {
  if (i == 1) return d == 1 ? 3 : d == 2 ? 4 : d == 3 ? 1 : d == 4 ? 2 : -1;
  if (i == 2) return d == -1 ? 1 : d == 1 ? 3 : d == 2 ? 4 : d == 3 ? 2 : -1;
  if (i == n) return d == -1 ? 1 : d == -2 ? 2 : d == -3 ? 3 : d == -4 ? 4 : -1;
  if (i == n - 1) return d == -1 ? 1 : d == -2 ? 2 : d == 1 ? 3 : d == -3 ? 4 : -1;
  return d == -1 ? 1 : d == -2 ? 2 : d == 1 ? 3 : d == 2 ? 4 : -1;
}
__device__ __forceinline__ bool has_bc(int i, int n, int d) {
  const int c = i + d;
  if (c < 1 || c > n) return false;
  if (d < 0) return c >= (i >= n - 1 ? n - 4 : i - 2);
  return c <= (i <= 2 ? 5 : min(i + 2, n));
}
__device__ __forceinline__ int pos_p(int d) { return d == -1 ? 1 : d == -2 ? 2 : d == 1 ? 3 : d == 2 ? 4 : -1; }
__device__ __forceinline__ bool has_p(int i, int n, int d) {
  // periodic band after the fill set-up (src/cpenta2p.f:52-77): lower blocks
  // from column 1, upper blocks up to column n
  const int c = i + d;
  return c >= 1 && c <= n && d >= -2 && d <= 2 && d != 0;
}

// One warp per record (row i of line iv): writes the internal record.
template <typename TM, typename TC, bool PER>
__global__ void __launch_bounds__(32 * kPrepWarps) prep_kernel(Args a) {
  __shared__ cd sm[kPrepWarps][kPrepSm];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const long long task = (long long)blockIdx.x * kPrepWarps + warp;
  if (task >= (long long)a.n * a.nsys) return;
  const int iv = (int)(task / a.n), i = (int)(task % a.n) + 1;
  const int n = a.n;
  cd* Dg = sm[warp];       // factored diagonal block of row i
  cd* Li = Dg + 25;        // L_ii^-1
  cd* Ui = Dg + 50;        // U_ii^-1
  cd* Di = Dg + 75;        // D_i^-1
  cd* S = Dg + 100;        // a stored off-diagonal block
  cd* Uc = Dg + 125;       // U_cc of its column
  cd* Tm = Dg + 150;       // S U_cc
  const TM* mat = reinterpret_cast<const TM*>(a.mat);
  TC* chn = reinterpret_cast<TC*>(a.chn);
  const long long rc = rec_of(a, i, iv);
  const TM* rec = mat + 125 * rc;
  const int m = lane % 5, q = lane / 5;
  if (lane < 25) Dg[m + 5 * q] = ld_cd(rec + 2 + 5 * m + 25 * q);
  __syncwarp();
  if (lane < 5) {
    const int j = lane;
    // column j of L_ii^-1: L = I - strict lower part of the stored block
    cd z[5];
#pragma unroll
    for (int mm = 0; mm < 5; ++mm) {
      cd v = cd{mm == j ? 1.0 : 0.0, 0.0};
#pragma unroll
      for (int k = 0; k < 5; ++k)
        if (k < mm && k >= j) v = fmac(v, Dg[mm + 5 * k], z[k]);
      z[mm] = mm < j ? cd{0.0, 0.0} : v;
    }
#pragma unroll
    for (int mm = 0; mm < 5; ++mm) Li[mm + 5 * j] = z[mm];
    // column j of U_ii^-1: U = upper part with the diagonal
#pragma unroll
    for (int mm = 4; mm >= 0; --mm) {
      cd v = cd{mm == j ? 1.0 : 0.0, 0.0};
#pragma unroll
      for (int k = 0; k < 5; ++k)
        if (k > mm) v = fmsc(v, Dg[mm + 5 * k], z[k]);
      z[mm] = mm > j ? cd{0.0, 0.0} : mul(v, rcp(Dg[mm + 5 * mm]));
    }
#pragma unroll
    for (int mm = 0; mm < 5; ++mm) Ui[mm + 5 * j] = z[mm];
  }
  __syncwarp();
  const bool act = lane < 25;  // lanes 25..31 idle in the block products
  if (act) Di[lane] = mm5(Ui, Li, m, q, false);
  __syncwarp();
  TC* out = chn + 125 * rc;
  if (lane < 25) st_t(out + lane, Di[lane]);
  bool written[5] = {true, false, false, false, false};
  for (int d = -4; d <= 4; ++d) {
    if (d == 0) continue;
    const bool has = PER ? has_p(i, n, d) : has_bc(i, n, d);
    if (!has) continue;
    const int pos = PER ? pos_p(d) : pos_bc(i, n, d);
    const int c = i + d;
    if (lane < 25) S[lane] = ld_cd(rec + (slot_bc(i, c) - 1) + 5 * m + 25 * q);
    if (d < 0 && lane < 25)
      Uc[lane] = m <= q ? ld_cd(mat + 125 * rec_of(a, c, iv) + 2 + 5 * m + 25 * q) : cd{0.0, 0.0};
    __syncwarp();
    cd v{0.0, 0.0};
    if (d < 0) {
      if (act) Tm[lane] = mm5(S, Uc, m, q, true);
      __syncwarp();
      if (act) v = mm5(Di, Tm, m, q, false);
      v = cd{-v.x, -v.y};
    } else if (act) {
      v = mm5(Ui, S, m, q, false);
    }
    if (lane < 25) st_t(out + 25 * pos + lane, v);
    written[pos] = true;
    __syncwarp();
  }
  for (int p = 1; p < 5; ++p)
    if (!written[p] && lane < 25) st_t(out + 25 * p + lane, cd{0.0, 0.0});
}

// ------------------------------------------------------------ the sweeps
// s = D^-1 r in place for the records of rows 1..n (periodic lines: rows
// 1..n-2, the border rows keep their right-hand side); bx is the block index
// within the problem.  Five lanes per record (lane m forms s_m), six records
// per warp: a load instruction of the warp reads six 5-entry column runs of
// D instead of 32 scattered records, and each output keeps the order of
// accumulation of a per-record loop.  The record's r is read by all five
// lanes before any of them writes (the __syncwarp between).
constexpr int kScaleRecsPerWarp = 6;
__host__ __device__ constexpr long long scale_blocks(long long recs, int threads = 256) {
  return (recs + (long long)(threads / 32) * kScaleRecsPerWarp - 1) / ((long long)(threads / 32) * kScaleRecsPerWarp);
}
template <typename T>
__device__ __forceinline__ void scale_body(const Args& a, long long bx) {
  const int lane = threadIdx.x % 32, mm = lane % 5;
  const long long t = (bx * blockDim.x + threadIdx.x) / 32 * kScaleRecsPerWarp + lane / 5;
  bool on = lane < 5 * kScaleRecsPerWarp && t < (long long)a.n * a.nsys;
  const T* D = nullptr;
  T* r = nullptr;
  T x[5];
  int i = 0, iv = 0;
  if (on) {
    if (a.row_stride == 1) i = (int)(t % a.n) + 1, iv = (int)(t / a.n);
    else iv = (int)(t % a.nsys), i = (int)(t / a.nsys) + 1;
    on = !a.bord || i <= a.n - 2;  // a periodic line's border rows keep b2
  }
  if (on) {
    const long long rc = rec_of(a, i, iv);
    D = reinterpret_cast<const T*>(a.chn) + 125 * rc;
    r = reinterpret_cast<T*>(a.rhs) + 5 * rc;
#pragma unroll
    for (int k = 0; k < 5; ++k) x[k] = r[k];
  }
  __syncwarp();
  if (on) {
    T acc = zero<T>();
#pragma unroll
    for (int k = 0; k < 5; ++k) acc = fmac(acc, D[mm + 5 * k], x[k]);
    r[mm] = acc;
  }
}
template <typename T>
__global__ void scale_kernel(Args a) { scale_body<T>(a, blockIdx.x); }

// Work tables of the batched launches: entry k of a phase's table runs block
// y of problem x (several problems in one launch, one ADI phase).  The
// batched kernels are persistent: a fixed grid strides over the table, whose
// length *cnt they read from device memory.
template <typename T>
__global__ void scale_batch_kernel(const Args* __restrict__ list, const int2* __restrict__ table,
                                   const int* __restrict__ active, const int* __restrict__ cnt) {
  for (int k = blockIdx.x; k < *cnt; k += gridDim.x) {
    const int2 w = table[k];
    if (active[w.x]) scale_body<T>(list[w.x], w.y);
  }
}

// kAhead: rows staged ahead of the recurrence.  kSplit: warps per line; the
// FP64 recurrences give the real and the imaginary part of a row to two warps
// (on two SM sub-partitions), which halves the dependent FP64 instructions
// each warp issues per row and doubles the sub-partitions a sweep uses.
template <typename T> struct ChainCfg;
template <> struct ChainCfg<cd> { static constexpr int kAhead = 12, kSplit = 2; };
template <> struct ChainCfg<cf> { static constexpr int kAhead = 24, kSplit = 1; };
constexpr int kChainWarps = 2;                 // lines per CTA of the single-problem launches
constexpr int kStage = 55;                     // 50 block entries + 5 right-hand-side entries
constexpr int kXchg = 20;                      // split lines: 2 parities x 2 parts x 5 components (doubles)

template <typename T>
constexpr int chain_threads(int lines_per_cta = kChainWarps) {
  return 32 * ChainCfg<T>::kSplit * lines_per_cta;
}
template <typename T>
constexpr size_t chain_smem_bytes(int lines_per_cta = kChainWarps) {
  return (size_t)lines_per_cta *
         ((ChainCfg<T>::kAhead + 1) * kStage * sizeof(T) + (ChainCfg<T>::kSplit > 1 ? kXchg * sizeof(double) : 0));
}

// sum over q of lane (m,q)'s partial, for m = this lane's q
template <typename T>
__device__ __forceinline__ T gather5(T p, int qq) {
  const unsigned full = 0xffffffffu;
  T s = shfl(full, p, qq);
  s = add(s, shfl(full, p, qq + 5));
  s = add(s, shfl(full, p, qq + 10));
  s = add(s, shfl(full, p, qq + 15));
  s = add(s, shfl(full, p, qq + 20));
  return s;
}

// Stage one row into a ring slot: the 50 block entries at src (its record
// plus the sweep's offset) and the 5 right-hand-side entries at rhs.
template <typename T>
__device__ __forceinline__ void chain_stage(T* slot, const T* src, const T* rhs, int lane) {
  cp_async_el(slot + lane, src + lane);
  const int e = lane + 32;
  if (e < 50) cp_async_el(slot + e, src + e);
  else if (e < 55) cp_async_el(slot + e, rhs + (e - 50));
}

// Forward recurrence yh_i = s_i - sum_c F_ic yh_c over rows 1..top (top = n,
// or n-2 for periodic lines, whose border rows follow in btail_kernel).  The
// staging, ring and output positions advance by pointer increments.
template <typename T, bool PER, int W>
__device__ __forceinline__ void chain_fwd_body(const Args& a, int bx, unsigned char* smem_raw) {
  constexpr int kAhead = ChainCfg<T>::kAhead, kRing = kAhead + 1;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int iv = bx * W + warp;
  if (iv >= a.nsys) return;
  T* const ring = reinterpret_cast<T*>(smem_raw) + warp * kRing * kStage;
  T* const rend = ring + kRing * kStage;
  const int n = a.n, top = PER ? n - 2 : n;
  const int m = lane % 5, qq = min(lane / 5, 4), l = min(lane, 24);
  T* grhs = reinterpret_cast<T*>(a.rhs);
  const T* gchn = reinterpret_cast<const T*>(a.chn);
  const long long rs = a.row_stride, rec1 = a.line_stride * (long long)iv;
  const T* sp = gchn + 125 * rec1 + 25;  // staging cursor: record of the next row to stage
  const T* rp = grhs + 5 * rec1;         // and its right-hand side
  T* ws = ring;                          // slot of the next row to stage
  for (int r = 1; r <= kAhead; ++r) {
    if (r <= top) chain_stage(ws, sp, rp, lane);
    cp_async_commit();
    sp += 125 * rs, rp += 5 * rs, ws += kStage;
  }
  const T* st = ring;                // slot of row i
  T* out = grhs + 5 * rec1 + qq;     // component qq of row i
  T z1 = zero<T>(), z2 = zero<T>(), z3 = zero<T>(), z4 = zero<T>();  // yh of rows i-1..i-4, component qq
  for (int i = 1; i <= top; ++i) {
    __syncwarp();  // every lane is done with the slot about to be refilled
    if (i + kAhead <= top) chain_stage(ws, sp, rp, lane);
    cp_async_commit();
    sp += 125 * rs, rp += 5 * rs, ws += kStage;
    if (ws == rend) ws = ring;
    cp_async_wait<kAhead>();
    __syncwarp();
    T p;
    if (PER || (i >= 3 && i <= n - 2)) {
      p = fmac(mul(st[l], z1), st[25 + l], z2);
    } else if (i == 1) {
      p = zero<T>();
    } else if (i == 2) {
      p = mul(st[l], z1);
    } else {
      const T* g = gchn + 125 * rec_of(a, i, iv);
      p = fmac(mul(st[l], z1), st[25 + l], z2);
      if (i == n - 1) {
        p = fmac(p, g[100 + l], z3);
      } else {
        p = fmac(p, g[75 + l], z3);
        p = fmac(p, g[100 + l], z4);
      }
    }
    const T yv = sub(st[50 + qq], gather5(p, qq));
    z4 = z3; z3 = z2; z2 = z1; z1 = yv;
    if (lane < 25 && m == 0) *out = yv;
    out += 5 * rs;
    st += kStage;
    if (st == rend) st = ring;
  }
  cp_async_wait<0>();
}

// Backward recurrence x_i = c_i - sum_c B_ic x_c from row top down to 1
// (top = n; periodic: n-2, the border rows left out: z = A11^-1 b1).
template <typename T, bool PER, int W>
__device__ __forceinline__ void chain_bwd_body(const Args& a, int bx, unsigned char* smem_raw) {
  constexpr int kAhead = ChainCfg<T>::kAhead, kRing = kAhead + 1;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int iv = bx * W + warp;
  if (iv >= a.nsys) return;
  T* const ring = reinterpret_cast<T*>(smem_raw) + warp * kRing * kStage;
  T* const rend = ring + kRing * kStage;
  const int n = a.n, top = PER ? n - 2 : n;
  const int m = lane % 5, qq = min(lane / 5, 4), l = min(lane, 24);
  T* grhs = reinterpret_cast<T*>(a.rhs);
  const T* gchn = reinterpret_cast<const T*>(a.chn);
  const long long rs = a.row_stride, rect = a.line_stride * (long long)iv + rs * (top - 1);  // record of row top
  const T* sp = gchn + 125 * rect + 75;
  const T* rp = grhs + 5 * rect;
  T* ws = ring;  // ring slot k holds the k-th row processed (row top - k)
  for (int k = 0; k < kAhead; ++k) {
    if (top - k >= 1) chain_stage(ws, sp, rp, lane);
    cp_async_commit();
    sp -= 125 * rs, rp -= 5 * rs, ws += kStage;
  }
  const T* st = ring;
  T* out = grhs + 5 * rect + qq;
  // x of rows i+1..i+4, component qq (periodic lines: z = A11^-1 b1, the
  // border rows left out)
  T x1 = zero<T>(), x2 = zero<T>(), x3 = zero<T>(), x4 = zero<T>();
  for (int k = 0; k < top; ++k) {
    __syncwarp();  // every lane is done with the slot about to be refilled
    const int i = top - k;
    if (top - (k + kAhead) >= 1) chain_stage(ws, sp, rp, lane);
    cp_async_commit();
    sp -= 125 * rs, rp -= 5 * rs, ws += kStage;
    if (ws == rend) ws = ring;
    cp_async_wait<kAhead>();
    __syncwarp();
    T p;
    if (PER || (i >= 3 && i <= n - 2)) {
      p = fmac(mul(st[l], x1), st[25 + l], x2);
    } else if (i == n) {
      p = zero<T>();
    } else if (i == n - 1) {
      p = mul(st[l], x1);
    } else {
      const T* g = gchn + 125 * rec_of(a, i, iv);
      p = fmac(mul(st[l], x1), st[25 + l], x2);
      if (i == 2) {
        p = fmac(p, g[50 + l], x3);
      } else {
        p = fmac(p, g[25 + l], x3);
        p = fmac(p, g[50 + l], x4);
      }
    }
    const T xv = sub(st[50 + qq], gather5(p, qq));
    x4 = x3; x3 = x2; x2 = x1; x1 = xv;
    if (lane < 25 && m == 0) *out = xv;
    out -= 5 * rs;
    st += kStage;
    if (st == rend) st = ring;
  }
  cp_async_wait<0>();
}

// ---------------------------------------------- FP64 recurrences, split lines
// Two warps per line: warp part c = 0 computes the real parts of a row, c = 1
// the imaginary parts.  Lane l = m + 5 q holds component q of the previous
// rows (both parts) and accumulates part c of block entry (m, q) times it;
// the sum over q is a three-level tree that leaves output component m in lane
// m, and a shuffle hands component qq back to lane group qq.  Each row, both
// warps post their part of the new row to a shared exchange slot and meet at
// a named barrier of the pair, which also publishes the rows the two warps
// staged: each warp stages half of every row into the line's ring and waits
// for its own copies one row before the barrier that precedes their use.

__device__ __forceinline__ void pair_sync(int id) { asm volatile("bar.sync %0, 64;\n" ::"r"(id) : "memory"); }

// Stage thread t's part of one row (the 50 block entries at src, the 5
// right-hand-side entries at rhs) into a ring slot shared by the pair.
__device__ __forceinline__ void chain_stage_half(cd* slot, const cd* src, const cd* rhs, int t) {
  if (t < 50) cp_async_el(slot + t, src + t);
  else if (t < 55) cp_async_el(slot + t, rhs + (t - 50));
}

// acc + part C of -(F z): re -(F.x z.x - F.y z.y), im -(F.x z.y + F.y z.x)
template <int C>
__device__ __forceinline__ double part_msub(double acc, cd f, cd z) {
  if constexpr (C == 0) return fma(f.y, z.y, fma(-f.x, z.x, acc));
  else return fma(-f.y, z.x, fma(-f.x, z.y, acc));
}

// sum over q of lane (m, q)'s partial into lane m, then component qq to
// every lane of group qq
__device__ __forceinline__ double tree5(double p, int qq) {
  const unsigned full = 0xffffffffu;
  const double t4 = __shfl_down_sync(full, p, 20);
  const double a = p + __shfl_down_sync(full, p, 10);
  const double b = a + __shfl_down_sync(full, a, 5);
  return __shfl_sync(full, b + t4, qq);
}

template <bool PER, int W, int C>
__device__ __forceinline__ void chain2_fwd_body(const Args& a, int bx, unsigned char* smem_raw) {
  constexpr int kAhead = ChainCfg<cd>::kAhead, kRing = kAhead + 1;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int ln = warp >> 1, t = C * 32 + lane;  // warp & 1 == C
  const int iv = bx * W + ln;
  if (iv >= a.nsys) return;  // both warps of the pair leave together
  const int bar = 1 + ln;
  cd* ring = reinterpret_cast<cd*>(smem_raw) + ln * kRing * kStage;
  double* xch = reinterpret_cast<double*>(reinterpret_cast<cd*>(smem_raw) + W * kRing * kStage) + ln * kXchg;
  const int n = a.n, top = PER ? n - 2 : n;
  const int m = lane % 5, qq = min(lane / 5, 4), l = min(lane, 24);
  double* grhs = reinterpret_cast<double*>(a.rhs);
  const cd* gchn = reinterpret_cast<const cd*>(a.chn);
  cd* const rend = ring + kRing * kStage;
  const long long rs = a.row_stride, rec1 = a.line_stride * (long long)iv;
  const cd* sp = gchn + 125 * rec1 + 25;                       // staging cursor (record, rhs)
  const cd* rp = reinterpret_cast<const cd*>(a.rhs) + 5 * rec1;
  cd* ws = ring;
  for (int r = 1; r <= kAhead; ++r) {
    if (r <= top) chain_stage_half(ws, sp, rp, t);
    cp_async_commit();
    sp += 125 * rs, rp += 5 * rs, ws += kStage;
  }
  cp_async_wait<kAhead - 1>();
  pair_sync(bar);
  const cd* st = ring;                          // slot of row i
  double* out = grhs + 2 * (5 * rec1 + qq) + C;  // part C of component qq of row i
  cd z1{0.0, 0.0}, z2{0.0, 0.0}, z3{0.0, 0.0}, z4{0.0, 0.0};  // yh of rows i-1..i-4, component qq
  for (int i = 1; i <= top; ++i) {
    // refills the slot of row i-1, which both warps finished
    if (i + kAhead <= top) chain_stage_half(ws, sp, rp, t);
    cp_async_commit();
    sp += 125 * rs, rp += 5 * rs, ws += kStage;
    if (ws == rend) ws = ring;
    double p = 0.0;
    if (lane < 5) p = C ? st[50 + lane].y : st[50 + lane].x;
    if (PER || (i >= 3 && i <= n - 2)) {
      p = part_msub<C>(p, st[25 + l], z2);
      p = part_msub<C>(p, st[l], z1);
    } else if (i == 2) {
      p = part_msub<C>(p, st[l], z1);
    } else if (i > 2) {
      const cd* g = gchn + 125 * rec_of(a, i, iv);
      if (i == n - 1) {
        p = part_msub<C>(p, g[100 + l], z3);
      } else {
        p = part_msub<C>(p, g[75 + l], z3);
        p = part_msub<C>(p, g[100 + l], z4);
      }
      p = part_msub<C>(p, st[25 + l], z2);
      p = part_msub<C>(p, st[l], z1);
    }
    const double yc = tree5(p, qq);
    const int par = i & 1;
    if (lane < 25 && m == 0) {
      xch[par * 10 + C * 5 + qq] = yc;
      *out = yc;
    }
    out += 10 * rs;
    st += kStage;
    if (st == rend) st = ring;
    cp_async_wait<kAhead - 1>();  // this thread's half of row i+1
    pair_sync(bar);
    const double yo = xch[par * 10 + (1 - C) * 5 + qq];
    z4 = z3; z3 = z2; z2 = z1;
    z1 = C ? cd{yo, yc} : cd{yc, yo};
  }
  cp_async_wait<0>();
}

template <bool PER, int W, int C>
__device__ __forceinline__ void chain2_bwd_body(const Args& a, int bx, unsigned char* smem_raw) {
  constexpr int kAhead = ChainCfg<cd>::kAhead, kRing = kAhead + 1;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int ln = warp >> 1, t = C * 32 + lane;  // warp & 1 == C
  const int iv = bx * W + ln;
  if (iv >= a.nsys) return;
  const int bar = 1 + ln;
  cd* ring = reinterpret_cast<cd*>(smem_raw) + ln * kRing * kStage;
  double* xch = reinterpret_cast<double*>(reinterpret_cast<cd*>(smem_raw) + W * kRing * kStage) + ln * kXchg;
  const int n = a.n, top = PER ? n - 2 : n;
  const int m = lane % 5, qq = min(lane / 5, 4), l = min(lane, 24);
  double* grhs = reinterpret_cast<double*>(a.rhs);
  const cd* grc = reinterpret_cast<const cd*>(a.rhs);
  const cd* gchn = reinterpret_cast<const cd*>(a.chn);
  cd* const rend = ring + kRing * kStage;
  const long long rs = a.row_stride, rect = a.line_stride * (long long)iv + rs * (top - 1);  // record of row top
  const cd* sp = gchn + 125 * rect + 75;
  const cd* rp = grc + 5 * rect;
  cd* ws = ring;  // ring slot k holds the k-th row processed (row top - k)
  for (int k = 0; k < kAhead; ++k) {
    if (top - k >= 1) chain_stage_half(ws, sp, rp, t);
    cp_async_commit();
    sp -= 125 * rs, rp -= 5 * rs, ws += kStage;
  }
  const cd* st = ring;
  double* out = grhs + 2 * (5 * rect + qq) + C;
  cd x1{0.0, 0.0}, x2{0.0, 0.0}, x3{0.0, 0.0}, x4{0.0, 0.0};  // x of rows i+1..i+4, component qq
  cp_async_wait<kAhead - 1>();
  pair_sync(bar);
  for (int k = 0; k < top; ++k) {
    const int i = top - k;
    if (top - (k + kAhead) >= 1) chain_stage_half(ws, sp, rp, t);
    cp_async_commit();
    sp -= 125 * rs, rp -= 5 * rs, ws += kStage;
    if (ws == rend) ws = ring;
    double p = 0.0;
    if (lane < 5) p = C ? st[50 + lane].y : st[50 + lane].x;
    if (PER || (i >= 3 && i <= n - 2)) {
      p = part_msub<C>(p, st[25 + l], x2);
      p = part_msub<C>(p, st[l], x1);
    } else if (i == n - 1) {
      p = part_msub<C>(p, st[l], x1);
    } else if (i < n - 1) {
      const cd* g = gchn + 125 * rec_of(a, i, iv);
      if (i == 2) {
        p = part_msub<C>(p, g[50 + l], x3);
      } else {
        p = part_msub<C>(p, g[25 + l], x3);
        p = part_msub<C>(p, g[50 + l], x4);
      }
      p = part_msub<C>(p, st[25 + l], x2);
      p = part_msub<C>(p, st[l], x1);
    }
    const double xc = tree5(p, qq);
    const int par = k & 1;
    if (lane < 25 && m == 0) {
      xch[par * 10 + C * 5 + qq] = xc;
      *out = xc;
    }
    out -= 10 * rs;
    st += kStage;
    if (st == rend) st = ring;
    cp_async_wait<kAhead - 1>();
    pair_sync(bar);
    const double xo = xch[par * 10 + (1 - C) * 5 + qq];
    x4 = x3; x3 = x2; x2 = x1;
    x1 = C ? cd{xo, xc} : cd{xc, xo};
  }
  cp_async_wait<0>();
}

template <typename T, bool PER, int W>
__device__ __forceinline__ void chain_fwd_any(const Args& a, int bx, unsigned char* smem_raw) {
  if constexpr (ChainCfg<T>::kSplit > 1) {
    if ((threadIdx.x / 32) & 1) chain2_fwd_body<PER, W, 1>(a, bx, smem_raw);
    else chain2_fwd_body<PER, W, 0>(a, bx, smem_raw);
  } else {
    chain_fwd_body<T, PER, W>(a, bx, smem_raw);
  }
}
template <typename T, bool PER, int W>
__device__ __forceinline__ void chain_bwd_any(const Args& a, int bx, unsigned char* smem_raw) {
  if constexpr (ChainCfg<T>::kSplit > 1) {
    if ((threadIdx.x / 32) & 1) chain2_bwd_body<PER, W, 1>(a, bx, smem_raw);
    else chain2_bwd_body<PER, W, 0>(a, bx, smem_raw);
  } else {
    chain_bwd_body<T, PER, W>(a, bx, smem_raw);
  }
}

// ------------------------------------ FP64 periodic lines, rows in pairs
// The band rows of a periodic line all have the form
//   yh_i = s_i - F1_i yh_{i-1} - F2_i yh_{i-2},  x_i = c_i - B1_i x_{i+1} - B2_i x_{i+2}
// (the blocks of the first rows zero).  Substituting the odd row into the
// even one,
//   yh_{i+1} = s'_{i+1} - G yh_{i-1} - H yh_{i-2},
//   G = F2_{i+1} - F1_{i+1} F1_i,  H = -F1_{i+1} F2_i,  s'_{i+1} = s_{i+1} - F1_{i+1} s_i,
// so both rows of a pair (i, i+1), i odd, are two block products of the
// same two rows of the previous pair, and a step of the recurrence covers
// two rows.  Likewise downwards in pairs (i, i-1) from the top row (odd):
//   x_{i-1} = c'_{i-1} - G' x_{i+1} - H' x_{i+2},
//   G' = B2_{i-1} - B1_{i-1} B1_i,  H' = -B1_{i-1} B2_i,  c'_{i-1} = c_{i-1} - B1_{i-1} c_i.
// The even rows' records hold G, H (blocks 1, 2) and G', H' (blocks 3, 4);
// the pair array holds, per even record, its own F1 and B1, with which
// even_kernel forms s' before the forward and c' before the backward pairs
// (point-parallel, one thread per entry).  Used when the band has an odd
// number of rows (top = n - 2 odd).
//
// Lines with boundary-closure rows (top = n even) pair the same way, upwards
// (1, 2) ... (n-1, n) and downwards (n, n-1) ... (2, 1), so the forward
// second rows are even and the backward ones odd.  Their end rows reach one
// row further: row n-1 has F3 and row n becomes G, H and J = F4 - F1 F3'
// (block 3) on the rows of the previous pair and of the one before; row 2
// has B3 and row 1 becomes G', H' and J' = B4 - B1 B3' (block 1).  Rows 2
// and n-1 keep their blocks (their products meet zero rows only).
constexpr int kPairAhead = 6;         // pairs staged ahead
constexpr int kPStage = 2 * kStage;   // a pair's two staged rows
constexpr int kPXchg = 40;            // 2 parities x 2 rows x 2 parts x 5 components (doubles)
constexpr int kPairLines = 2;         // lines (four warps each) per CTA
constexpr size_t pair_smem_bytes(int lines_per_cta = kPairLines) {
  return (size_t)lines_per_cta * ((kPairAhead + 1) * kPStage * sizeof(cd) + kPXchg * sizeof(double));
}

// One warp per even record e of the band (2 <= e <= n-3): G, H, G', H' into
// the record, its F1 and B1 into the pair array (formed in FP64 from the
// FP64 records, after the border's W, which uses the records row by row).
__global__ void __launch_bounds__(32 * kPrepWarps) pair_prep_kernel(Args a) {
  __shared__ cd sm[kPrepWarps][8 * 25];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int rows = (a.n - 3) / 2;  // even rows 2..n-3
  const long long task = (long long)blockIdx.x * kPrepWarps + warp;
  if (task >= (long long)rows * a.nsys) return;
  const int iv = (int)(task / rows), e = 2 * (int)(task % rows) + 2;
  cd* chn = reinterpret_cast<cd*>(a.chn);
  cd* re = chn + 125 * rec_of(a, e, iv);
  const cd* rlo = chn + 125 * rec_of(a, e - 1, iv);
  const cd* rhi = chn + 125 * rec_of(a, e + 1, iv);
  cd* F1 = sm[warp];
  cd *F2 = F1 + 25, *B1 = F1 + 50, *B2 = F1 + 75, *F1l = F1 + 100, *F2l = F1 + 125, *B1h = F1 + 150,
     *B2h = F1 + 175;
  const int m = lane % 5, q = lane / 5;
  if (lane < 25) {
    F1[lane] = re[25 + lane], F2[lane] = re[50 + lane], B1[lane] = re[75 + lane], B2[lane] = re[100 + lane];
    F1l[lane] = rlo[25 + lane], F2l[lane] = rlo[50 + lane];
    B1h[lane] = rhi[75 + lane], B2h[lane] = rhi[100 + lane];
  }
  __syncwarp();
  if (lane < 25) {
    const cd g = sub(F2[lane], mm5(F1, F1l, m, q, false));
    const cd h = mm5(F1, F2l, m, q, false);
    const cd g2 = sub(B2[lane], mm5(B1, B1h, m, q, false));
    const cd h2 = mm5(B1, B2h, m, q, false);
    re[25 + lane] = g;
    re[50 + lane] = cd{-h.x, -h.y};
    re[75 + lane] = g2;
    re[100 + lane] = cd{-h2.x, -h2.y};
    cd* pr = reinterpret_cast<cd*>(a.pairs) + 50 * rec_of(a, e, iv);
    pr[lane] = F1[lane];
    pr[25 + lane] = B1[lane];
  }
}

// Lines with boundary-closure rows (n even): one warp per record, the even
// rows' forward and the odd rows' backward blocks combined (above), each
// row's own F1 (even) or B1 (odd) into the pair array.  A row writes only
// blocks its neighbours' combinations do not read.
__global__ void __launch_bounds__(32 * kPrepWarps) pair_prep_bc_kernel(Args a) {
  __shared__ cd sm[kPrepWarps][6 * 25];
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int n = a.n;
  const long long task = (long long)blockIdx.x * kPrepWarps + warp;
  if (task >= (long long)n * a.nsys) return;
  const int iv = (int)(task / n), r = (int)(task % n) + 1;
  cd* chn = reinterpret_cast<cd*>(a.chn);
  cd* rr = chn + 125 * rec_of(a, r, iv);
  cd* pr = reinterpret_cast<cd*>(a.pairs) + 50 * rec_of(a, r, iv);
  const int m = lane % 5, q = lane / 5;
  cd* A = sm[warp];  // own first block (F1 or B1)
  cd *X = A + 25, *Y = A + 50, *Z = A + 75, *U = A + 100, *V = A + 125;
  const bool act = lane < 25;
  if (r % 2 == 0) {
    // forward: own F1 at block 1; the odd row below: F1 (25), F2 (50), F3 (100 on row n-1)
    if (act) pr[lane] = rr[25 + lane];
    if (r == 2) return;
    const cd* lo = chn + 125 * rec_of(a, r - 1, iv);
    if (act) {
      A[lane] = rr[25 + lane];
      X[lane] = lo[25 + lane], Y[lane] = lo[50 + lane], Z[lane] = r == n ? lo[100 + lane] : cd{0.0, 0.0};
      U[lane] = rr[50 + lane];                                  // F2
      V[lane] = r == n ? rr[75 + lane] : cd{0.0, 0.0};          // F3 of row n
    }
    const cd F4 = (act && r == n) ? rr[100 + lane] : cd{0.0, 0.0};
    __syncwarp();
    if (act) {
      const cd g = sub(U[lane], mm5(A, X, m, q, false));
      const cd h = sub(V[lane], mm5(A, Y, m, q, false));      // row n: F3 - F1 F2'; else -F1 F2'
      rr[25 + lane] = g;
      rr[50 + lane] = h;
      if (r == n) rr[75 + lane] = sub(F4, mm5(A, Z, m, q, false));  // J
    }
  } else {
    // backward: own B1 at block 3; the even row above: B1 (75), B2 (100), B3 (50 on row 2)
    if (act) pr[25 + lane] = rr[75 + lane];
    if (r == n - 1) return;
    const cd* hi = chn + 125 * rec_of(a, r + 1, iv);
    if (act) {
      A[lane] = rr[75 + lane];
      X[lane] = hi[75 + lane], Y[lane] = hi[100 + lane], Z[lane] = r == 1 ? hi[50 + lane] : cd{0.0, 0.0};
      U[lane] = rr[100 + lane];                                 // B2
      V[lane] = r == 1 ? rr[25 + lane] : cd{0.0, 0.0};          // B3 of row 1
    }
    const cd B4 = (act && r == 1) ? rr[50 + lane] : cd{0.0, 0.0};
    __syncwarp();
    if (act) {
      const cd g = sub(U[lane], mm5(A, X, m, q, false));
      const cd h = sub(V[lane], mm5(A, Y, m, q, false));      // row 1: B3 - B1 B2'; else -B1 B2'
      rr[75 + lane] = g;
      rr[100 + lane] = h;
      if (r == 1) rr[25 + lane] = sub(B4, mm5(A, Z, m, q, false));  // J'
    }
  }
}

// The second rows' right-hand sides before a paired recurrence:
// s'_j = s_j - F1_j s_{j-1} (UP = false) or c'_j = c_j - B1_j c_{j+1}
// (UP = true) on rows j = first, first + 2, ... (rows per line); one thread
// per entry, only those rows written.
template <bool UP>
__global__ void even_kernel(Args a, int first, int rows) {
  const long long t5 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long t = t5 / 5;
  const int mm = (int)(t5 - 5 * t);
  if (t >= (long long)rows * a.nsys) return;
  int k, iv;
  if (a.row_stride == 1) k = (int)(t % rows), iv = (int)(t / rows);
  else iv = (int)(t % a.nsys), k = (int)(t / a.nsys);
  const long long rj = rec_of(a, first + 2 * k, iv);
  cd* grhs = reinterpret_cast<cd*>(a.rhs);
  const cd* B = reinterpret_cast<const cd*>(a.pairs) + 50 * rj + (UP ? 25 : 0);
  const cd* nb = grhs + 5 * (UP ? rj + a.row_stride : rj - a.row_stride);
  cd acc = grhs[5 * rj + mm];
#pragma unroll
  for (int q = 0; q < 5; ++q) acc = fmsc(acc, B[mm + 5 * q], nb[q]);
  grhs[5 * rj + mm] = acc;
}

// Stage one pair (rows r0 and r1 = r0 +- 1; the second only when `two`):
// each row's 50 block entries at its record plus off and its 5
// right-hand-side entries; thread t < 110 of the line's team copies one.
__device__ __forceinline__ void pair_stage(cd* slot, const cd* gchn, const cd* grc, long long rec0,
                                           long long rec1, int off, bool two, int t) {
  if (t >= 110) return;
  const int r = t >= 55, e = r ? t - 55 : t;
  if (r && !two) return;
  const long long rc = r ? rec1 : rec0;
  if (e < 50) cp_async_el(slot + t, gchn + 125 * rc + off + e);
  else cp_async_el(slot + t, grc + 5 * rc + (e - 50));
}

__device__ __forceinline__ void team_sync(int id) { asm volatile("bar.sync %0, 128;\n" ::"r"(id) : "memory"); }

// Both recurrences of a paired line: DOWN = false forward over pairs (2k+1,
// 2k+2), DOWN = true backward over pairs (top-2k, top-2k-1).  Four warps per
// line: warp 2P + C forms part C of row P of each pair (the split layout of
// chain2: lane (m, q), a three-level tree of DADD), and the four post their
// parts to a shared exchange slot and meet at the line's named barrier, which
// also publishes the rows the team staged.
template <int W, int P, int C, bool DOWN, bool BC>
__device__ __forceinline__ void pair_body(const Args& a, int bx, unsigned char* smem_raw) {
  constexpr int kRing = kPairAhead + 1;
  const int warp = threadIdx.x / 32, lane = threadIdx.x % 32;
  const int ln = warp >> 2, t = (warp & 3) * 32 + lane;
  const int iv = bx * W + ln;
  if (iv >= a.nsys) return;  // the four warps of a line leave together
  const int bar = 1 + ln;
  cd* ring = reinterpret_cast<cd*>(smem_raw) + ln * kRing * kPStage;
  double* xch = reinterpret_cast<double*>(reinterpret_cast<cd*>(smem_raw) + W * kRing * kPStage) + ln * kPXchg;
  const int top = BC ? a.n : a.n - 2, npair = (top + 1) / 2;
  const int m = lane % 5, qq = min(lane / 5, 4), l = min(lane, 24);
  double* grhs = reinterpret_cast<double*>(a.rhs);
  const cd* grc = reinterpret_cast<const cd*>(a.rhs);
  const cd* gchn = reinterpret_cast<const cd*>(a.chn);
  cd* const rend = ring + kRing * kPStage;
  // the end pair's third block (BC): forward rows n-1 (F3, block 4) and n
  // (J, block 3); backward rows 2 (B3, block 2) and 1 (J', block 1)
  const cd* g3 = nullptr;
  if (BC) {
    const int r3 = DOWN ? 2 - P : a.n - 1 + P;
    const int b3 = DOWN ? (P ? 25 : 50) : (P ? 75 : 100);
    g3 = gchn + 125 * rec_of(a, r3, iv) + b3;
  }
  const long long rs = a.row_stride, base = a.line_stride * (long long)iv;
  const long long step = DOWN ? -2 * rs : 2 * rs;              // records per pair
  const long long dr = DOWN ? -rs : rs;                       // the pair's second row
  const int off = DOWN ? 75 : 25;                             // the recurrence's two blocks
  long long srec = base + rs * (DOWN ? top - 1 : 0);          // first row of the next pair to stage
  cd* ws = ring;
  for (int k = 0; k < kPairAhead; ++k) {
    if (k < npair) pair_stage(ws, gchn, grc, srec, srec + dr, off, 2 * k + 2 <= top, t);
    cp_async_commit();
    srec += step, ws += kPStage;
  }
  cp_async_wait<kPairAhead - 1>();
  team_sync(bar);
  const cd* st = ring;
  double* out = grhs + 2 * (5 * (base + rs * (DOWN ? top - 1 - P : P)) + qq) + C;
  cd z1{0.0, 0.0}, z2{0.0, 0.0};  // the previous pair's rows: second, first (component qq)
  cd z3{0.0, 0.0};                // the second row of the pair before (BC end rows)
  for (int k = 0; k < npair; ++k) {
    if (k + kPairAhead < npair) pair_stage(ws, gchn, grc, srec, srec + dr, off, 2 * (k + kPairAhead) + 2 <= top, t);
    cp_async_commit();
    srec += step, ws += kPStage;
    if (ws == rend) ws = ring;
    const bool live = P == 0 || 2 * k + 2 <= top;  // the last pair has its first row only
    const cd* rw = st + P * kStage;
    double p = 0.0;
    if (lane < 5) p = C ? rw[50 + lane].y : rw[50 + lane].x;
    if (BC && k == npair - 1) p = part_msub<C>(p, g3[l], z3);
    p = part_msub<C>(p, rw[25 + l], z2);
    p = part_msub<C>(p, rw[l], z1);
    const double yc = tree5(p, qq);
    const int par = k & 1;
    if (live && lane < 25 && m == 0) {
      xch[par * 20 + P * 10 + C * 5 + qq] = yc;
      *out = yc;
    }
    out += DOWN ? -20 * rs : 20 * rs;
    st += kPStage;
    if (st == rend) st = ring;
    cp_async_wait<kPairAhead - 1>();  // this thread's part of the next pair
    team_sync(bar);
    const double* x = xch + par * 20 + qq;
    z3 = z1;
    z2 = cd{x[0], x[5]};    // first row of the pair
    z1 = cd{x[10], x[15]};  // second row
  }
  cp_async_wait<0>();
}

template <int W, bool DOWN, bool BC>
__device__ __forceinline__ void pair_any(const Args& a, int bx, unsigned char* smem_raw) {
  switch ((threadIdx.x / 32) & 3) {
    case 0: pair_body<W, 0, 0, DOWN, BC>(a, bx, smem_raw); break;
    case 1: pair_body<W, 0, 1, DOWN, BC>(a, bx, smem_raw); break;
    case 2: pair_body<W, 1, 0, DOWN, BC>(a, bx, smem_raw); break;
    default: pair_body<W, 1, 1, DOWN, BC>(a, bx, smem_raw); break;
  }
}
// Launch with 128 * W threads and pair_smem_bytes(W) bytes.  BC: lines with
// boundary-closure rows (n even) instead of periodic ones.
template <bool DOWN, bool BC = false, int W = kPairLines>
__global__ void __launch_bounds__(128 * W) pair_chain_kernel(Args a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  pair_any<W, DOWN, BC>(a, blockIdx.x, smem_raw);
}

// Launch with chain_threads<T>(W) threads and chain_smem_bytes<T>(W) bytes.
template <typename T, bool PER, int W = kChainWarps>
__global__ void __launch_bounds__(chain_threads<T>(W)) chain_fwd_kernel(Args a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  chain_fwd_any<T, PER, W>(a, blockIdx.x, smem_raw);
}
template <typename T, bool PER, int W = kChainWarps>
__global__ void __launch_bounds__(chain_threads<T>(W)) chain_bwd_kernel(Args a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  chain_bwd_any<T, PER, W>(a, blockIdx.x, smem_raw);
}
// The recurrences' entries are lines of problems of different lengths, so
// their CTAs take the next entry from a counter (*next, cleared before the
// launch) rather than a fixed stride.  Each line's warps reuse their own
// ring and exchange slots from entry to entry; the first barrier of an entry
// orders them after the last reads of the previous one.
__device__ __forceinline__ int next_entry(int* next, int* slot) {
  if (threadIdx.x == 0) *slot = atomicAdd(next, 1);
  __syncthreads();
  const int k = *slot;
  __syncthreads();  // every thread has read the slot before it is refilled
  return k;
}
template <typename T, bool PER, int W>
__global__ void __launch_bounds__(chain_threads<T>(W)) chain_fwd_batch_kernel(const Args* __restrict__ list,
                                                                             const int2* __restrict__ table,
                                                                             const int* __restrict__ active,
                                                                             const int* __restrict__ cnt,
                                                                             int* next) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int slot;
  const int n = *cnt;
  for (int k = next_entry(next, &slot); k < n; k = next_entry(next, &slot)) {
    const int2 w = table[k];
    if (active[w.x]) chain_fwd_any<T, PER, W>(list[w.x], w.y, smem_raw);
  }
}
template <typename T, bool PER, int W>
__global__ void __launch_bounds__(chain_threads<T>(W)) chain_bwd_batch_kernel(const Args* __restrict__ list,
                                                                             const int2* __restrict__ table,
                                                                             const int* __restrict__ active,
                                                                             const int* __restrict__ cnt,
                                                                             int* next) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ int slot;
  const int n = *cnt;
  for (int k = next_entry(next, &slot); k < n; k = next_entry(next, &slot)) {
    const int2 w = table[k];
    if (active[w.x]) chain_bwd_any<T, PER, W>(list[w.x], w.y, smem_raw);
  }
}

// ----------------------------------------------------- periodic border
// The sixteen border blocks of a periodic line's LHS, before factoring: row,
// reference slot (column i+slot-3, wrapped) and column.  0..5: A12 (rows 1,
// 2, n-3, n-2 at columns n-1, n), 6..11: A21, 12..15: A22.
struct BBlk {
  int row, slot, col;
};
__host__ __device__ inline BBlk bblk(int k, int n) {
  switch (k) {
    case 0: return {1, 1, n - 1};
    case 1: return {1, 2, n};
    case 2: return {2, 1, n};
    case 3: return {n - 3, 5, n - 1};
    case 4: return {n - 2, 4, n - 1};
    case 5: return {n - 2, 5, n};
    case 6: return {n - 1, 1, n - 3};
    case 7: return {n - 1, 2, n - 2};
    case 8: return {n - 1, 5, 1};
    case 9: return {n, 1, n - 2};
    case 10: return {n, 4, 1};
    case 11: return {n, 5, 2};
    case 12: return {n - 1, 3, n - 1};
    case 13: return {n - 1, 4, n};
    case 14: return {n, 2, n - 1};
    default: return {n, 3, n};
  }
}

// Copies the sixteen border blocks of every line from the unfactored LHS
// (reference storage, entry (slot, m, q) at slot-1 + 5 m + 25 q) into the
// raw part of the border data; one thread per entry.
__global__ void bcopy_kernel(Args a) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)a.nsys * 400) return;
  const int iv = (int)(t / 400), k = (int)(t / 25 % 16), e = (int)(t % 25);
  const BBlk b = bblk(k, a.n);
  const cd* mat = reinterpret_cast<const cd*>(a.mat) + 125 * rec_of(a, b.row, iv);
  cd* out = reinterpret_cast<cd*>(a.bord) + (long long)kBordCd * iv + kBordRaw + 25 * k;
  out[e] = mat[(b.slot - 1) + 5 * (e % 5) + 25 * (e / 5)];
}

// The reference's periodic factorisation adds, at pivot row n-5, row n-3's
// update of column n-1 (M X: M its multiplier block at column n-5, X row
// n-5's fill block at column n-1) to column n-2 instead (src/cpenta1p.f and
// src/cpenta2p.f at i = n-5; penta_p_kernel keeps it unless the exact
// factorisation is chosen).  Its factors are then those of the matrix whose
// row n-3 has M X added at column n-2 and taken from column n-1; the band
// records already hold the first, and this kernel makes the border block at
// (n-3, n-1) the second, so that the bordered solve agrees with the
// reference's.  One thread per entry (m, q); mat and per factored.
__global__ void bquirk_kernel(Args a) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)a.nsys * 25) return;
  const int iv = (int)(t / 25), e = (int)(t % 25), m = e % 5, q = e / 5;
  const int n = a.n;
  const cd* M = reinterpret_cast<const cd*>(a.mat) + 125 * rec_of(a, n - 3, iv);   // slot 1: column n-5
  const cd* X = reinterpret_cast<const cd*>(a.per) + 50 * rec_of(a, n - 5, iv);    // per(1): column n-1
  cd d{0.0, 0.0};
#pragma unroll
  for (int nc = 0; nc < 5; ++nc) d = fmac(d, M[5 * m + 25 * nc], X[2 * nc + 10 * q]);
  cd* raw = reinterpret_cast<cd*>(a.bord) + (long long)kBordCd * iv + kBordRaw + 25 * 3;   // (n-3, n-1)
  raw[m + 5 * q] = sub(raw[m + 5 * q], d);
}

// Column j of A12 (the coefficients of component j % 5 of border row
// n-1 + j / 5) as a right-hand side: rows 1, 2, n-3, n-2 of rhs, which the
// caller has cleared; one thread per (line, block, component).
template <typename TC>
__global__ void brhs_kernel(Args a, int j) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)a.nsys * 30) return;
  const int iv = (int)(t / 30), k = (int)(t / 5 % 6), m = (int)(t % 5);
  const BBlk b = bblk(k, a.n);
  if ((b.col == a.n ? 1 : 0) != j / 5) return;
  const cd* blk = reinterpret_cast<const cd*>(a.bord) + (long long)kBordCd * iv + kBordRaw + 25 * k;
  st_t(reinterpret_cast<TC*>(a.rhs) + 5 * rec_of(a, b.row, iv) + m, blk[m + 5 * (j % 5)]);
}

// Column j of W = A11^-1 A12 from the solved rows 1..n-2 of rhs into the
// fill array (entry (m, j) of a record's W at m + 5 j).
template <typename TC>
__global__ void bw_kernel(Args a, int j) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const int rows = a.n - 2;
  if (t >= (long long)a.nsys * rows * 5) return;
  const int m = (int)(t % 5);
  const long long r = t / 5;
  const int iv = (int)(r / rows), i = (int)(r % rows) + 1;
  const long long rc = rec_of(a, i, iv);
  reinterpret_cast<TC*>(a.fillE)[50 * rc + m + 5 * j] = reinterpret_cast<const TC*>(a.rhs)[5 * rc + m];
}

// S = A22 - A21 W, inverted by Gauss-Jordan elimination with partial
// pivoting, into the kept part of the border data with the A21 blocks; one
// thread per line (formed once per factorisation, in FP64).
template <typename TC>
__global__ void bschur_kernel(Args a, int* status) {
  const int iv = blockIdx.x * blockDim.x + threadIdx.x;
  if (iv >= a.nsys) return;
  const int n = a.n;
  cd* bd = reinterpret_cast<cd*>(a.bord) + (long long)kBordCd * iv;
  const cd* raw = bd + kBordRaw;
  const TC* W = reinterpret_cast<const TC*>(a.fillE);
  cd M[10][20];  // [S | I]
  for (int k = 0; k < 10; ++k) {
    const int bk = k / 5, m = k % 5;
    for (int j = 0; j < 10; ++j) {
      const int bj = j / 5, p = j % 5;
      cd s = raw[25 * (12 + 2 * bk + bj) + m + 5 * p];   // A22 block (bk, bj)
      for (int kk = 0; kk < 3; ++kk) {                 // A21 blocks of border row bk
        const int blk = 6 + 3 * bk + kk;
        const cd* A = raw + 25 * blk;
        const TC* w = W + 50 * rec_of(a, bblk(blk, n).col, iv) + 5 * j;
        for (int q = 0; q < 5; ++q) s = fmsc(s, A[m + 5 * q], ld_cd(w + q));
      }
      M[k][j] = s;
      M[k][10 + j] = cd{k == j ? 1.0 : 0.0, 0.0};
    }
  }
  bool ok = true;
  for (int c = 0; c < 10; ++c) {
    int piv = c;
    double best = -1.0;
    for (int r = c; r < 10; ++r) {
      const double v = fabs(M[r][c].x) + fabs(M[r][c].y);
      if (v > best) best = v, piv = r;
    }
    if (!(best > 0.0) || !isfinite(best)) {
      ok = false;
      break;
    }
    if (piv != c)
      for (int j = 0; j < 20; ++j) {
        const cd t = M[c][j];
        M[c][j] = M[piv][j];
        M[piv][j] = t;
      }
    const cd inv = rcp(M[c][c]);
    for (int j = 0; j < 20; ++j) M[c][j] = mul(M[c][j], inv);
    for (int r = 0; r < 10; ++r) {
      if (r == c) continue;
      const cd f = M[r][c];
      for (int j = 0; j < 20; ++j) M[r][j] = fmsc(M[r][j], f, M[c][j]);
    }
  }
  if (!ok) {
    atomicExch(status, 1);
    return;
  }
  for (int k = 0; k < 10; ++k)
    for (int j = 0; j < 10; ++j) bd[kBordSinv + k + 10 * j] = M[k][10 + j];
  for (int e = 0; e < 150; ++e) bd[kBordA21 + e] = raw[25 * 6 + e];
}

// Per step, after the recurrences gave z in rows 1..n-2: x2 = S^-1 (b2 -
// A21 z) into rows n-1, n (which hold b2).  One warp per line, lane
// k = m + 5 b < 10 forms entry k in FP64.
constexpr int kBTailLines = 4;
template <typename T>
__device__ __forceinline__ void btail_body(const Args& a, int iv) {
  const int lane = threadIdx.x % 32;
  if (iv >= a.nsys) return;
  const int n = a.n;
  const cd* bd = reinterpret_cast<const cd*>(a.bord) + (long long)kBordCd * iv;
  T* grhs = reinterpret_cast<T*>(a.rhs);
  const int k = min(lane, 9), b = k / 5, m = k % 5;
  const long long rb = rec_of(a, n - 1 + b, iv);
  cd t = ld_cd(grhs + 5 * rb + m);
  for (int kk = 0; kk < 3; ++kk) {
    const int blk = 6 + 3 * b + kk;
    const cd* A = bd + kBordA21 + 25 * (3 * b + kk);
    const T* z = grhs + 5 * rec_of(a, bblk(blk, n).col, iv);
#pragma unroll
    for (int q = 0; q < 5; ++q) t = fmsc(t, A[m + 5 * q], ld_cd(z + q));
  }
  cd x{0.0, 0.0};
#pragma unroll
  for (int j = 0; j < 10; ++j) {
    const cd tj{__shfl_sync(0xffffffffu, t.x, j), __shfl_sync(0xffffffffu, t.y, j)};
    x = fmac(x, bd[kBordSinv + k + 10 * j], tj);
  }
  if (lane < 10) st_t(grhs + 5 * rb + m, x);
}
template <typename T>
__global__ void __launch_bounds__(32 * kBTailLines) btail_kernel(Args a) {
  btail_body<T>(a, blockIdx.x * kBTailLines + threadIdx.x / 32);
}
template <typename T>
__global__ void __launch_bounds__(32 * kBTailLines) btail_batch_kernel(const Args* __restrict__ list,
                                                                      const int2* __restrict__ table,
                                                                      const int* __restrict__ active,
                                                                      const int* __restrict__ cnt) {
  for (int k = blockIdx.x; k < *cnt; k += gridDim.x) {
    const int2 w = table[k];
    if (active[w.x]) btail_body<T>(list[w.x], w.y * kBTailLines + threadIdx.x / 32);
  }
}

// Periodic lines, last: x_i = z_i - W_i x2 for rows 1..n-2 (and row np,
// which repeats row 1), one thread per entry of x_i (thread 5 t + m forms
// entry m of record t), so a warp's loads cover a few consecutive records'
// W runs; each entry sums the columns of border row n-1, then of row n.
__host__ __device__ constexpr long long fill_blocks(long long recs, int threads = 256) {
  return (5 * recs + threads - 1) / threads;
}
template <typename T>
__device__ __forceinline__ void fill_body(const Args& a, long long bx) {
  const long long t5 = bx * blockDim.x + threadIdx.x;
  const long long t = t5 / 5;
  const int mm = (int)(t5 - 5 * t);
  const int rows = a.n - 2;
  if (t >= (long long)rows * a.nsys) return;
  int i, iv;
  if (a.row_stride == 1) i = (int)(t % rows) + 1, iv = (int)(t / rows);
  else iv = (int)(t % a.nsys), i = (int)(t / a.nsys) + 1;
  T* grhs = reinterpret_cast<T*>(a.rhs);
  const long long rc = rec_of(a, i, iv);
  const T* E = reinterpret_cast<const T*>(a.fillE) + 50 * rc + mm;
  const T* xa = grhs + 5 * rec_of(a, a.n - 1, iv);
  const T* xb = grhs + 5 * rec_of(a, a.n, iv);
  T acc = grhs[5 * rc + mm];
#pragma unroll
  for (int k = 0; k < 5; ++k) acc = fmsc(acc, E[5 * k], xa[k]);
#pragma unroll
  for (int k = 0; k < 5; ++k) acc = fmsc(acc, E[25 + 5 * k], xb[k]);
  grhs[5 * rc + mm] = acc;
  if (i == 1) grhs[5 * rec_of(a, a.n + 1, iv) + mm] = acc;  // row np = row 1
}

template <typename T>
__global__ void fill_kernel(Args a) { fill_body<T>(a, blockIdx.x); }
template <typename T>
__global__ void fill_batch_kernel(const Args* __restrict__ list, const int2* __restrict__ table,
                                  const int* __restrict__ active, const int* __restrict__ cnt) {
  for (int k = blockIdx.x; k < *cnt; k += gridDim.x) {
    const int2 w = table[k];
    if (active[w.x]) fill_body<T>(list[w.x], w.y);
  }
}

}  // namespace chain
}  // namespace lns
