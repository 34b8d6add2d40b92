// Direct FP64 block-pentadiagonal line solver, boundary-closure rows
// (penta1bc / penta2bc / cpenta1bc / cpenta2bc semantics).
//
// A team of TEAM threads owns one line: one warp (TEAM = 32, several lines
// per CTA) when there are lines enough to fill the GPU, else a whole CTA of
// 64..256 threads per line.  The line's block rows stream through a five-row
// ring in shared memory (cp.async prefetch of the row three ahead), so the
// elimination of pivot row i sees rows i..i+2 (i..n near the end of the
// line) resident.  Each pivot row runs
//   A  in-block elimination of the diagonal block, applied to the blocks
//      right of it and (code 2) to the right-hand side;
//   B  multipliers of the rows below, one lane per (target row, block row),
//      stored in place of the eliminated blocks as the complex reference
//      solvers do (src/cpenta1bc.f:82-83);
//   C  the Schur update of the rows below, one lane per output element;
// and the row is written back.  Back substitution re-reads the factored
// rows in reverse.  Every element receives its updates in the reference
// order (pivot row, pivot column ascending); multiplications by a
// reciprocal replace the reference's divisions and all multiply-adds are
// fused, so results agree with the reference to rounding, not bit-for-bit.
#pragma once
#include <cstdint>

#include "scalar.cuh"

namespace lns {

constexpr int kRing = 5;       // resident block rows per line
constexpr int kRowSz = 130;    // 5 slots x 25 + 5 right-hand-side entries
constexpr int kWarpsPerCta = 4;

struct PentaArgs {
  void* mat;
  void* rhs;
  int n;             // unknown rows per line
  int nsys;          // lines
  long long row_stride;   // in row records between consecutive rows of a line
  long long line_stride;  // in row records between consecutive lines
  int code;          // 0 factor, 1 solve with stored factors, 2 both
  int* status;       // set non-zero on a non-finite pivot (may be null)
};

__device__ __forceinline__ int mod5(int x) { return ((x % 5) + 5) % 5; }
// Slot (1..5) of column c in row t of a boundary-closure line; valid for the
// columns the row holds (src/lhsbt1f.f90:43-48,102-107,199-204).
__device__ __forceinline__ int slot_bc(int t, int c) { return mod5(c - t + 2) + 1; }
// Last column held by row i (rows 1 and 2 reach column 5).
__device__ __forceinline__ int lastcol_bc(int i, int n) { return i <= 2 ? 5 : min(i + 2, n); }
// Last row below i holding column i.
__device__ __forceinline__ int maxtarget_bc(int i, int n) { return i >= n - 4 ? n : min(i + 2, n); }

template <typename T>
__device__ __forceinline__ void cp_async_el(T* dst, const T* src) {
  unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if constexpr (sizeof(T) == 16) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src));
  } else {
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(d), "l"(src), "n"(sizeof(T)));
  }
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

template <typename T, int TEAM = 32>
struct LineCtx {
  T* ring;              // kRing * kRowSz
  T* scratch;           // 16 entries: [0,5) multipliers, [5,10) pivot reciprocals
  const PentaArgs* a;
  int iv, lane, n;      // lane: thread index within the team
  __device__ void sync() const {
    if constexpr (TEAM == 32) __syncwarp();
    else __syncthreads();
  }

  __device__ T* row(int r) const { return ring + ((r - 1) % kRing) * kRowSz; }
  __device__ T* blk(int r, int k) const { return row(r) + 25 * (k - 1); }
  __device__ T* rhs(int r) const { return row(r) + 125; }
  __device__ long long rec(int r) const { return a->row_stride * (r - 1) + a->line_stride * iv; }

  // Asynchronous load of row r (matrix record in the reference layout
  // mat(k,m,q), stored in shared memory as [k][m][q]) and its right-hand side.
  __device__ void load_row(int r, bool with_rhs) const {
    const T* gm = reinterpret_cast<const T*>(a->mat) + 125 * rec(r);
    T* s = row(r);
    for (int e = lane; e < 125; e += TEAM) {
      int k = e % 5, m = (e / 5) % 5, q = e / 25;
      cp_async_el(s + k * 25 + m * 5 + q, gm + e);
    }
    if (with_rhs && lane < 5) cp_async_el(s + 125 + lane, reinterpret_cast<const T*>(a->rhs) + 5 * rec(r) + lane);
  }
  __device__ void store_row(int r, bool with_mat, bool with_rhs) const {
    T* s = row(r);
    if (with_mat) {
      T* gm = reinterpret_cast<T*>(a->mat) + 125 * rec(r);
      for (int e = lane; e < 125; e += TEAM) {
        int k = e % 5, m = (e / 5) % 5, q = e / 25;
        gm[e] = s[k * 25 + m * 5 + q];
      }
    }
    if (with_rhs && lane < 5) reinterpret_cast<T*>(a->rhs)[5 * rec(r) + lane] = s[125 + lane];
  }
};

// Factor (and with_rhs: forward-eliminate the right-hand side) pivot row i.
template <typename T, int TEAM>
__device__ void pivot_bc(const LineCtx<T, TEAM>& L, int i, bool factor, bool with_rhs) {
  const int n = L.n, lane = L.lane;
  T* D = L.blk(i, 3);
  T* ri = L.rhs(i);
  const int nr = lastcol_bc(i, n) - i;
  const int nt = maxtarget_bc(i, n) - i;
  T* mults = L.scratch;
  T* facts = L.scratch + 5;

  if (factor) {
    // A: in-block elimination, "first four columns" (src/cpenta1bc.f:52-71)
    for (int nc = 0; nc < 4; ++nc) {
      const T r = rcp(D[nc * 5 + nc]);
      if (lane == 0) facts[nc] = r;
      const int w = 4 - nc;
      const int ncol = w + 5 * nr + (with_rhs ? 1 : 0);
      const int total = w * ncol;
      for (int idx = lane; idx < total; idx += TEAM) {
        const int l = nc + 1 + idx / ncol, j = idx % ncol;
        const T mult = negmul(D[l * 5 + nc], r);
        T *X, *Xp;
        if (j < w) {
          X = D + l * 5 + nc + 1 + j;
          Xp = D + nc * 5 + nc + 1 + j;
        } else if (j < w + 5 * nr) {
          const int jj = j - w, b = jj / 5, q = jj % 5;
          T* B = L.blk(i, slot_bc(i, i + 1 + b));
          X = B + l * 5 + q;
          Xp = B + nc * 5 + q;
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
    // B: multipliers of the rows below (src/cpenta1bc.f:75-83), in place.
    if (lane < 5 * nt) {
      const int t = i + 1 + lane / 5, m = lane % 5;
      T* B = L.blk(t, slot_bc(t, i));
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
    // forward elimination with stored multipliers (src/cpenta1bc.f:505-512)
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

  // C: Schur update of the rows below (src/cpenta1bc.f:84-101)
  const int per = (factor ? 25 * nr : 0) + (with_rhs ? 5 : 0);
  for (int idx = lane; idx < nt * per; idx += TEAM) {
    const int a = idx / per, j = idx % per, t = i + 1 + a;
    const T* M = L.blk(t, slot_bc(t, i));
    if (factor && j < 25 * nr) {
      const int b = j / 25, m = (j % 25) / 5, q = j % 5, c = i + 1 + b;
      T* Y = L.blk(t, slot_bc(t, c));
      const T* X = L.blk(i, slot_bc(i, c));
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

// Back substitution of row i (src/cpenta1bc.f:760-847); x of the rows to
// the right are the already solved right-hand sides in the ring.
template <typename T, int TEAM>
__device__ void backsub_bc(const LineCtx<T, TEAM>& L, int i) {
  const int n = L.n, lane = L.lane;
  const T* D = L.blk(i, 3);
  T* ri = L.rhs(i);
  const int nr = lastcol_bc(i, n) - i;
  if (lane < 5) {
    const int m = lane;
    const T rd = rcp(D[m * 5 + m]);
    T acc = ri[m];
    for (int q = 0; q < 5; ++q)
      for (int b = 0; b < nr; ++b) {
        const int c = i + 1 + b;
        acc = fmsc(acc, L.blk(i, slot_bc(i, c))[m * 5 + q], L.rhs(c)[q]);
      }
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

// TEAM = 32: kWarpsPerCta lines per CTA, one per warp; TEAM > 32: one line
// per CTA of TEAM threads.
template <typename T, int TEAM = 32>
__global__ void __launch_bounds__(TEAM == 32 ? 32 * kWarpsPerCta : TEAM) penta_bc_kernel(PentaArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int iv, lane;
  T* base;
  if constexpr (TEAM == 32) {
    const int warp = threadIdx.x / 32;
    lane = threadIdx.x % 32;
    iv = blockIdx.x * kWarpsPerCta + warp;
    base = reinterpret_cast<T*>(smem_raw) + warp * (kRing * kRowSz + 16);
  } else {
    lane = threadIdx.x;
    iv = blockIdx.x;
    base = reinterpret_cast<T*>(smem_raw);
  }
  if (iv >= args.nsys) return;  // whole teams exit; only team barriers are used below
  LineCtx<T, TEAM> L{base, base + kRing * kRowSz, &args, iv, lane, args.n};
  const int n = args.n;
  const bool factor = args.code != 1, solve = args.code != 0;

  // forward sweep: factor and/or eliminate the right-hand side
  for (int r = 1; r <= 3; ++r) L.load_row(r, solve);
  cp_async_commit();
  int loaded = 3;
  for (int i = 1; i <= n; ++i) {
    if (i >= n - 4) {
      while (loaded < n) L.load_row(++loaded, solve);
      cp_async_commit();
      cp_async_wait<0>();
    } else {
      if (loaded < i + 3) L.load_row(++loaded, solve);
      cp_async_commit();
      cp_async_wait<1>();
    }
    L.sync();
    pivot_bc(L, i, factor, solve);
    if (args.status && lane == 0 && factor && !finite_s(L.blk(i, 3)[24])) atomicExch(args.status, 1);
    // rows n-4..n stay resident for the back substitution
    if (i < n - 4 || !solve) L.store_row(i, factor, solve);
    L.sync();
  }
  if (!solve) return;
  // backward sweep
  for (int i = n; i >= 1; --i) {
    if (i < n - 4) {
      cp_async_wait<0>();
      L.sync();
    }
    if (i - 1 >= 1 && i - 1 < n - 4) {
      L.load_row(i - 1, true);
      cp_async_commit();
    }
    backsub_bc(L, i);
    if (i >= n - 4) L.store_row(i, factor, false);
    L.store_row(i, false, true);
  }
}

}  // namespace lns
