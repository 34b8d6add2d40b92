// Direct FP64 periodic block-pentadiagonal line solver (penta1p / penta2p /
// cpenta1p / cpenta2p semantics).
//
// A periodic line of np = n + 1 rows solves n unknowns (row np repeats row
// 1).  Its block rows reach around the ends, so Gaussian elimination fills
// columns n-1, n of every row and rows n-1, n at every column.  The fill
// follows the reference storage (src/penta2p.f:44-57, src/cpenta1p.f:52-77):
//   per(1|2, row)      columns n-1 | n of rows 1..n-3 (row n-3's column n-1
//                      is its slot 5);
//   per2(n-1|n, col)   rows n-1 | n at the columns left of their band.
// A team of TEAM threads owns a line (one warp, or a CTA of 64..256 threads
// when there are few lines; results do not depend on TEAM).  Band rows
// 1..n-2 stream through a shared-memory
// ring (with their per blocks); rows n-1 and n stay resident for the whole
// elimination, with their fill held in a three-column window.  Each pivot
// row has up to four blocks right of the diagonal (i+1, i+2, n-1, n) and up
// to four rows below it (i+1, i+2, n-1, n); the phases are those of the
// boundary-closure solver (penta_direct.cuh).
#pragma once
#include "penta_direct.cuh"

namespace lns {

constexpr int kPRowSz = 180;  // 5 slots + per(1), per(2) (7 x 25) + 5 rhs
constexpr int kPWarpsPerCta = 2;
constexpr int kPWarpSmem = kRing * kPRowSz + 2 * 130 + 2 * 75 + 16;

struct PeriodicArgs {
  void* mat;
  void* rhs;
  void* per;    // per(2,5,5,np,nsys) layout of mat's rows
  void* per2;   // complex: per2(2,5,5,np,nsys); real: unused (scratch in the reference)
  int n;        // unknowns (np - 1)
  int nrows;    // np
  int nsys;
  long long row_stride, line_stride;
  int code;
  int compat;   // reproduce the reference fill placement at row n-5
  int store_per2;
  int* status;
};

template <typename T, int TEAM = 32>
struct PLine {
  T* ring;     // kRing rows of kPRowSz: [0,125) slots, [125,175) per(1), per(2), [175,180) rhs
  T* res;      // rows n-1, n: 125 slots + 5 rhs each
  T* fw;       // fill windows of rows n-1, n: 3 blocks each, column c at (c-1)%3
  T* scratch;
  const PeriodicArgs* a;
  int iv, lane, n;  // lane: thread index within the team
  __device__ void sync() const {
    if constexpr (TEAM == 32) __syncwarp();
    else __syncthreads();
  }

  __device__ T* ringrow(int r) const { return ring + ((r - 1) % kRing) * kPRowSz; }
  __device__ long long rec(int r) const { return a->row_stride * (r - 1) + a->line_stride * iv; }
  __device__ T* rhs(int r) const {
    return r >= n - 1 ? res + (r - (n - 1)) * 130 + 125 : ringrow(r) + 175;
  }
  __device__ T* slot(int r, int k) const {
    return r >= n - 1 ? res + (r - (n - 1)) * 130 + 25 * (k - 1) : ringrow(r) + 25 * (k - 1);
  }
  // Block of row t at column c (src/penta2p.f storage), or null.
  __device__ T* get(int t, int c) const {
    if (t == n - 1) {
      if (c <= n - 4) return fw + 25 * ((c - 1) % 3);
      return slot(t, c - t + 3);
    }
    if (t == n) {
      if (c <= n - 3) return fw + 75 + 25 * ((c - 1) % 3);
      return slot(t, c - t + 3);
    }
    if ((c == n - 1 || c == n) && t <= n - 3 && !(t == n - 3 && c == n - 1))
      return ringrow(t) + 125 + (c == n ? 25 : 0);
    const int k = c - t + 3;
    return (k >= 1 && k <= 5) ? slot(t, k) : nullptr;
  }

  __device__ void load_band_row(int r, bool factor, bool with_rhs) const {
    const T* gm = reinterpret_cast<const T*>(a->mat) + 125 * rec(r);
    T* s = ringrow(r);
    for (int e = lane; e < 125; e += TEAM) {
      const int k = e % 5, m = (e / 5) % 5, q = e / 25;
      cp_async_el(s + k * 25 + m * 5 + q, gm + e);
    }
    if (!factor) {  // factored per blocks from the earlier factorisation
      const T* gp = reinterpret_cast<const T*>(a->per) + 50 * rec(r);
      for (int e = lane; e < 50; e += TEAM) {
        const int j = e % 2, m = (e / 2) % 5, q = e / 10;
        cp_async_el(s + 125 + 25 * j + m * 5 + q, gp + e);
      }
    }
    if (with_rhs && lane < 5) cp_async_el(s + 175 + lane, reinterpret_cast<const T*>(a->rhs) + 5 * rec(r) + lane);
  }
  // Fill set-up of a freshly landed band row, src/penta2p.f:44-51.
  __device__ void setup_band_row(int r) const {
    T* s = ringrow(r);
    for (int e = lane; e < 50; e += TEAM) {
      const int j = e / 25, mq = e % 25;
      T v = zero<T>();
      if (r == 1) v = s[25 * j + mq];          // per(1) = slot 1, per(2) = slot 2
      if (r == 2 && j == 1) v = s[mq];         // per(2) = slot 1
      s[125 + e] = v;
    }
  }
  __device__ void store_band_row(int r, bool with_mat, bool with_rhs) const {
    T* s = ringrow(r);
    if (with_mat) {
      T* gm = reinterpret_cast<T*>(a->mat) + 125 * rec(r);
      for (int e = lane; e < 125; e += TEAM) {
        const int k = e % 5, m = (e / 5) % 5, q = e / 25;
        gm[e] = s[k * 25 + m * 5 + q];
      }
      T* gp = reinterpret_cast<T*>(a->per) + 50 * rec(r);
      for (int e = lane; e < 50; e += TEAM) {
        const int j = e % 2, m = (e / 2) % 5, q = e / 10;
        gp[e] = s[125 + 25 * j + m * 5 + q];
      }
    }
    if (with_rhs && lane < 5) reinterpret_cast<T*>(a->rhs)[5 * rec(r) + lane] = s[175 + lane];
  }
  __device__ void load_res_rows(bool with_rhs) const {
    for (int rr = 0; rr < 2; ++rr) {
      const T* gm = reinterpret_cast<const T*>(a->mat) + 125 * rec(n - 1 + rr);
      T* s = res + rr * 130;
      for (int e = lane; e < 125; e += TEAM) {
        const int k = e % 5, m = (e / 5) % 5, q = e / 25;
        cp_async_el(s + k * 25 + m * 5 + q, gm + e);
      }
      if (with_rhs && lane < 5)
        cp_async_el(s + 125 + lane, reinterpret_cast<const T*>(a->rhs) + 5 * rec(n - 1 + rr) + lane);
    }
  }
  __device__ void store_res_rows(bool with_mat, bool with_rhs) const {
    for (int rr = 0; rr < 2; ++rr) {
      T* s = res + rr * 130;
      if (with_mat) {
        T* gm = reinterpret_cast<T*>(a->mat) + 125 * rec(n - 1 + rr);
        for (int e = lane; e < 125; e += TEAM) {
          const int k = e % 5, m = (e / 5) % 5, q = e / 25;
          gm[e] = s[k * 25 + m * 5 + q];
        }
      }
      if (with_rhs && lane < 5) reinterpret_cast<T*>(a->rhs)[5 * rec(n - 1 + rr) + lane] = s[125 + lane];
    }
  }
  // per2(n-1|n, m, q, col) <-> fill window block of column col
  __device__ void store_fill(int col) const {
    if (!a->store_per2) return;
    T* gp = reinterpret_cast<T*>(a->per2) + 50 * rec(col);
    for (int e = lane; e < 50; e += TEAM) {
      const int j = e % 2, m = (e / 2) % 5, q = e / 10;
      const int lim = j == 0 ? n - 4 : n - 3;
      if (col <= lim) gp[e] = fw[75 * j + 25 * ((col - 1) % 3) + m * 5 + q];
    }
  }
  __device__ void load_fill(int col) const {
    const T* gp = reinterpret_cast<const T*>(a->per2) + 50 * rec(col);
    for (int e = lane; e < 50; e += TEAM) {
      const int j = e % 2, m = (e / 2) % 5, q = e / 10;
      const int lim = j == 0 ? n - 4 : n - 3;
      if (col <= lim) fw[75 * j + 25 * ((col - 1) % 3) + m * 5 + q] = gp[e];
    }
  }
  // The complex reference clears per and per2 before factoring
  // (src/cpenta1p.f:52-62); clear the parts the elimination never writes.
  __device__ void clear_unused_fill() const {
    for (int r = n - 1; r <= n + 1; ++r) {
      T* gp = reinterpret_cast<T*>(a->per) + 50 * rec(r);
      for (int e = lane; e < 50; e += TEAM) gp[e] = zero<T>();
    }
    if (!a->store_per2) return;
    for (int c = n - 3; c <= n + 1; ++c) {
      T* gp = reinterpret_cast<T*>(a->per2) + 50 * rec(c);
      for (int e = lane; e < 50; e += TEAM) {
        const int lim = (e % 2) == 0 ? n - 4 : n - 3;
        if (c > lim) gp[e] = zero<T>();
      }
    }
  }
  __device__ void zero_fill(int col) const {
    for (int e = lane; e < 50; e += TEAM) fw[75 * (e / 25) + 25 * ((col - 1) % 3) + e % 25] = zero<T>();
  }
};

__device__ __forceinline__ int p_cols(int i, int n, int* c) {
  int cnt = 0;
  const int cand[4] = {i + 1, i + 2, n - 1, n};
  for (int a = 0; a < 4; ++a) {
    const int v = cand[a];
    if (v <= i || v > n) continue;
    bool dup = false;
    for (int b = 0; b < cnt; ++b) dup |= c[b] == v;
    if (!dup) c[cnt++] = v;
  }
  return cnt;  // ascending by construction
}

template <typename T, int TEAM>
__device__ void pivot_p(const PLine<T, TEAM>& L, int i, bool factor, bool with_rhs) {
  const int n = L.n, lane = L.lane;
  T* D = L.get(i, i);
  T* ri = L.rhs(i);
  int rc[4], tg[4];
  const int nr = p_cols(i, n, rc);
  const int nt = p_cols(i, n, tg);  // rows below holding column i: the same set
  T* mults = L.scratch;
  T* facts = L.scratch + 5;

  if (factor) {
    for (int nc = 0; nc < 4; ++nc) {
      const T r = rcp(D[nc * 5 + nc]);
      if (lane == 0) facts[nc] = r;
      const int w = 4 - nc;
      const int ncol = w + 5 * nr + (with_rhs ? 1 : 0);
      for (int idx = lane; idx < w * ncol; idx += TEAM) {
        const int l = nc + 1 + idx / ncol, j = idx % ncol;
        const T mult = negmul(D[l * 5 + nc], r);
        T *X, *Xp;
        if (j < w) {
          X = D + l * 5 + nc + 1 + j;
          Xp = D + nc * 5 + nc + 1 + j;
        } else if (j < w + 5 * nr) {
          const int jj = j - w;
          T* B = L.get(i, rc[jj / 5]);
          X = B + l * 5 + jj % 5;
          Xp = B + nc * 5 + jj % 5;
        } else {
          X = ri + l;
          Xp = ri + nc;
        }
        *X = fmac(*X, mult, *Xp);
        if (j == 0) mults[l] = mult;
      }
      L.sync();
      if (lane < w) D[(nc + 1 + lane) * 5 + nc] = mults[nc + 1 + lane];
      L.sync();
    }
    if (lane == 0) facts[4] = rcp(D[24]);
    L.sync();
    if (lane < 5 * nt) {
      const int t = tg[lane / 5], m = lane % 5;
      T* B = L.get(t, i);
      T acc[5];
#pragma unroll
      for (int q = 0; q < 5; ++q) acc[q] = B[m * 5 + q];
#pragma unroll
      for (int nc = 0; nc < 5; ++nc) {
        const T M = negmul(acc[nc], facts[nc]);
        B[m * 5 + nc] = M;
#pragma unroll
        for (int q = nc + 1; q < 5; ++q) acc[q] = fmac(acc[q], M, D[nc * 5 + q]);
      }
    }
    L.sync();
  } else if (with_rhs) {
    if (lane < 5) {
      T acc = ri[lane];
      for (int nc = 0; nc < 4; ++nc) {
        const T x = shfl(0x1fu, acc, nc);
        if (lane > nc) acc = fmac(acc, D[lane * 5 + nc], x);
      }
      ri[lane] = acc;
    }
    L.sync();
  }

  const int per = (factor ? 25 * nr : 0) + (with_rhs ? 5 : 0);
  for (int idx = lane; idx < nt * per; idx += TEAM) {
    const int t = tg[idx / per], j = idx % per;
    const T* M = L.get(t, i);
    if (factor && j < 25 * nr) {
      const int c = rc[j / 25], m = (j % 25) / 5, q = j % 5;
      int cy = c;
      if (L.a->compat && i == n - 5 && t == n - 3 && c == n - 1) cy = n - 2;  // src/penta2p.f:278,339
      T* Y = L.get(t, cy);
      const T* X = L.get(i, c);
      T acc = Y[m * 5 + q];
#pragma unroll
      for (int nc = 0; nc < 5; ++nc) acc = fmac(acc, M[m * 5 + nc], X[nc * 5 + q]);
      Y[m * 5 + q] = acc;
    } else {
      const int m = factor ? j - 25 * nr : j;
      T* rt = L.rhs(t);
      T acc = rt[m];
#pragma unroll
      for (int nc = 0; nc < 5; ++nc) acc = fmac(acc, M[m * 5 + nc], ri[nc]);
      rt[m] = acc;
    }
  }
  L.sync();
}

// x of rows n-1, n live in the resident rows; x of i+1, i+2 in the ring.
template <typename T, int TEAM>
__device__ void backsub_p(const PLine<T, TEAM>& L, int i) {
  const int n = L.n, lane = L.lane;
  const T* D = L.get(i, i);
  T* ri = L.rhs(i);
  int rc[4];
  const int nr = p_cols(i, n, rc);
  if (lane < 5) {
    const int m = lane;
    const T rd = rcp(D[m * 5 + m]);
    T acc = ri[m];
    for (int q = 0; q < 5; ++q)
      for (int b = 0; b < nr; ++b) acc = fmsc(acc, L.get(i, rc[b])[m * 5 + q], L.rhs(rc[b])[q]);
#pragma unroll
    for (int mm = 4; mm >= 0; --mm) {
      const T xm = shfl(0x1fu, mul(acc, rd), mm);
      if (lane < mm) acc = fmsc(acc, D[lane * 5 + mm], xm);
      if (lane == mm) acc = xm;
    }
    ri[m] = acc;
  }
  L.sync();
}

// TEAM = 32: kPWarpsPerCta lines per CTA, one per warp; TEAM > 32: one line
// per CTA of TEAM threads.
template <typename T, int TEAM = 32>
__global__ void __launch_bounds__(TEAM == 32 ? 32 * kPWarpsPerCta : TEAM) penta_p_kernel(PeriodicArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int iv, lane;
  T* base;
  if constexpr (TEAM == 32) {
    const int warp = threadIdx.x / 32;
    lane = threadIdx.x % 32;
    iv = blockIdx.x * kPWarpsPerCta + warp;
    base = reinterpret_cast<T*>(smem_raw) + warp * kPWarpSmem;
  } else {
    lane = threadIdx.x;
    iv = blockIdx.x;
    base = reinterpret_cast<T*>(smem_raw);
  }
  if (iv >= args.nsys) return;  // whole teams exit; only team barriers are used below
  PLine<T, TEAM> L{base, base + kRing * kPRowSz, base + kRing * kPRowSz + 260, base + kRing * kPRowSz + 410,
                   &args, iv, lane, args.n};
  const int n = args.n;
  const bool factor = args.code != 1, solve = args.code != 0;

  // resident rows n-1, n and the first band rows
  L.load_res_rows(solve);
  for (int r = 1; r <= 3; ++r) L.load_band_row(r, factor, solve);
  cp_async_commit();
  int loaded = 3;
  cp_async_wait<0>();
  L.sync();
  if (factor) {
    // fill set-up, src/penta2p.f:44-57
    for (int r = 1; r <= 3; ++r) L.setup_band_row(r);
    for (int e = lane; e < 150; e += TEAM) L.fw[e] = zero<T>();
    L.sync();
    for (int e = lane; e < 25; e += TEAM) {
      L.fw[e] = L.slot(n - 1, 5)[e];            // row n-1, column 1
      L.fw[75 + e] = L.slot(n, 4)[e];           // row n, column 1
      L.fw[75 + 25 + e] = L.slot(n, 5)[e];      // row n, column 2
    }
  } else {
    L.load_fill(1);
    L.load_fill(2);
  }
  L.sync();

  for (int i = 1; i <= n; ++i) {
    // band rows up to min(i+2, n-2) must be resident; prefetch one more
    const int want = min(i + 3, n - 2);
    const int need = min(i + 2, n - 2);
    while (loaded < want) L.load_band_row(++loaded, factor, solve);
    cp_async_commit();
    if (loaded > need) cp_async_wait<1>(); else cp_async_wait<0>();
    L.sync();
    // row i+2 lands for this pivot: initialise its fill (rows 1..3 above)
    if (factor && i >= 2 && i + 2 <= n - 2) L.setup_band_row(i + 2);
    if (!factor && solve && i + 2 <= n - 3) L.load_fill(i + 2);
    L.sync();
    pivot_p(L, i, factor, solve);
    if (args.status && lane == 0 && factor && !finite_s(L.get(i, i)[24])) atomicExch(args.status, 1);
    if (factor) {
      L.store_fill(i);
      L.sync();
      if (i + 3 <= n - 3) L.zero_fill(i + 3);
    }
    if (i <= n - 2 && (i < n - 6 || !solve)) L.store_band_row(i, factor, solve);
    L.sync();
  }
  if (factor) L.clear_unused_fill();
  if (!solve) {
    L.store_res_rows(true, false);
    return;
  }
  for (int i = n; i >= 1; --i) {
    if (i <= n - 2 && i < n - 6) {
      cp_async_wait<0>();
      L.sync();
    }
    if (i - 1 >= 1 && i - 1 < n - 6) {
      L.load_band_row(i - 1, false, true);
      cp_async_commit();
    }
    backsub_p(L, i);
    if (i <= n - 2 && i >= n - 6) L.store_band_row(i, factor, false);
    if (i <= n - 2) L.store_band_row(i, false, true);
  }
  L.store_res_rows(factor, true);
  // row np repeats row 1 (src/penta2p.f:749-751)
  if (lane < 5) reinterpret_cast<T*>(args.rhs)[5 * L.rec(n + 1) + lane] = L.rhs(1)[lane];
}

}  // namespace lns
