// Solve phase (code 1) of the block-pentadiagonal line solvers: forward
// elimination with the stored multipliers and back substitution, for
// boundary-closure and periodic lines, real or complex, FP64 or FP32.
//
// The solve is a chain of 5-vector operations per row, so a line needs five
// lanes, not a warp: lane (g, m) owns component m of line g, and a warp
// carries kLpw lines in lockstep.  Row records (the 125-entry matrix record,
// the right-hand side, and for periodic lines the per / per2 records) are
// staged into shared memory with cp.async kDepth rows ahead of use.
//
// Forward elimination is written in "pull" form: row i takes the
// contributions of the rows that eliminated its left blocks, in ascending
// column order, then its in-block lower factor.  Every right-hand-side entry
// thereby receives the reference's updates in the reference's order
// (src/cpenta1bc.f:499-748).  Rows n-1, n of a periodic line receive
// contributions from every column; those are pushed as each row finishes.
#pragma once
#include "penta_direct.cuh"

namespace lns {

struct SolveArgs {
  const void* mat;
  void* rhs;
  const void* per;
  const void* per2;
  int n;          // unknowns per line
  int nsys;
  long long row_stride, line_stride;
  int periodic;
};

template <typename T> struct SolveCfg;
template <> struct SolveCfg<double> { static constexpr int kLpw = 6; };
template <> struct SolveCfg<float> { static constexpr int kLpw = 6; };
template <> struct SolveCfg<cd> { static constexpr int kLpw = 3; };
template <> struct SolveCfg<cf> { static constexpr int kLpw = 6; };
constexpr int kDepth = 6;                 // rows staged ahead
constexpr int kSlots = kDepth + 1;        // ring slots per line
constexpr int kRecBc = 130;               // 125 matrix + 5 rhs
constexpr int kRecPer = 230;              // + per (50) + per2 (50)

template <typename T>
constexpr size_t solve_smem_bytes(bool periodic) {
  return (size_t)SolveCfg<T>::kLpw * kSlots * (periodic ? kRecPer : kRecBc) * sizeof(T);
}

template <typename T, bool PER>
struct SolveLine {
  T* stage;      // this line's ring: kSlots records
  const SolveArgs* a;
  int iv, n;
  bool valid;
  static constexpr int kRec = PER ? kRecPer : kRecBc;

  __device__ long long rec(int r) const { return a->row_stride * (r - 1) + a->line_stride * iv; }
  __device__ T* slotrec(int r) const { return stage + ((r - 1) % kSlots) * kRec; }
  // element (k,m,q) of the staged matrix record (reference order k + 5m + 25q)
  __device__ T matel(int r, int k, int m, int q) const { return slotrec(r)[(k - 1) + 5 * m + 25 * q]; }
  __device__ T rhsel(int r, int m) const { return slotrec(r)[125 + m]; }
  // per(j,m,q,r): j = 1 column n-1, j = 2 column n
  __device__ T perel(int r, int j, int m, int q) const { return slotrec(r)[130 + (j - 1) + 2 * m + 10 * q]; }
  // per2(t,m,q,c) staged with record c: t = 0 row n-1, t = 1 row n
  __device__ T per2el(int c, int t, int m, int q) const { return slotrec(c)[180 + t + 2 * m + 10 * q]; }
};

// Stage row r of every line of the warp (all 32 lanes issue copies).
// Lane l copies entries l, l+32, l+64, l+96 of each line's 125-entry
// matrix record (and of the 100-entry per / per2 records of periodic
// lines); lanes 0..4 copy the right-hand side.  Per line only the record
// base is computed, so the copy loop is a handful of instructions per entry.
template <typename T, bool PER>
__device__ __forceinline__ void stage_row(T* base, const SolveArgs& a, int r, int lane) {
  constexpr int kLpw = SolveCfg<T>::kLpw;
  constexpr int kRec = PER ? kRecPer : kRecBc;
  const int slot = (r - 1) % kSlots;
  const T* gmat = reinterpret_cast<const T*>(a.mat);
  const T* grhs = reinterpret_cast<const T*>(a.rhs);
  const long long rowoff = a.row_stride * (r - 1);
#pragma unroll
  for (int g = 0; g < kLpw; ++g) {
    const int iv = min((int)blockIdx.x * kLpw + g, a.nsys - 1);
    const long long rc = rowoff + a.line_stride * iv;
    T* dst = base + (g * kSlots + slot) * kRec;
    const T* src = gmat + 125 * rc;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int e = lane + 32 * k;
      if (e < 125) cp_async_el(dst + e, src + e);
    }
    if (lane < 5) cp_async_el(dst + 125 + lane, grhs + 5 * rc + lane);
    if (PER) {
      const T* sp = reinterpret_cast<const T*>(a.per) + 50 * rc;
      const T* sp2 = reinterpret_cast<const T*>(a.per2) + 50 * rc;
#pragma unroll
      for (int k = 0; k < 2; ++k) {
        const int e = lane + 32 * k;
        if (e < 50) {
          cp_async_el(dst + 130 + e, sp + e);
          cp_async_el(dst + 180 + e, sp2 + e);
        }
      }
    }
  }
}

template <typename T, bool PER>
__global__ void __launch_bounds__(32) penta_solve_kernel(SolveArgs args) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int kLpw = SolveCfg<T>::kLpw;
  constexpr int kRec = SolveLine<T, PER>::kRec;
  const int lane = threadIdx.x;
  const int g = min(lane / 5, kLpw - 1), m = lane % 5;
  const bool active = lane < 5 * kLpw;
  const unsigned mask = 0xffffffffu;
  const int n = args.n;
  T* base = reinterpret_cast<T*>(smem_raw);

  const int my_iv = blockIdx.x * kLpw + g;
  const SolveLine<T, PER> L{base + g * kSlots * kRec, &args, min(my_iv, args.nsys - 1), n, my_iv < args.nsys};
  const bool store = active && L.valid;
  T* grhs = reinterpret_cast<T*>(args.rhs);
  auto src_lane = [&](int comp) { return 5 * g + comp; };

  // ------------------------------------------------------------ forward
  for (int r = 1; r <= min(kDepth, n); ++r) {
    stage_row<T, PER>(base, args, r, lane);
    cp_async_commit();
  }
  T y1 = zero<T>(), y2 = zero<T>(), y3 = zero<T>(), y4 = zero<T>();  // y of rows i-1..i-4, component m
  T rn1 = zero<T>(), rn0 = zero<T>();  // periodic rows n-1, n, pushed contributions
  if (PER) {
    rn1 = grhs[5 * L.rec(n - 1) + m];
    rn0 = grhs[5 * L.rec(n) + m];
  }
  for (int i = 1; i <= n; ++i) {
    // stage row i + kDepth - 1 in the slot freed by row i - 1
    if (i + kDepth - 1 <= n && i > 1) stage_row<T, PER>(base, args, i + kDepth - 1, lane);
    cp_async_commit();
    cp_async_wait<kDepth - 1>();
    __syncwarp();
    T acc = L.rhsel(i, m);
    if (PER && i == n - 1) acc = rn1;
    if (PER && i == n) acc = rn0;
    // pull: blocks of row i left of its diagonal, ascending column
    auto pull = [&](int k, const T& yv) {
#pragma unroll
      for (int nc = 0; nc < 5; ++nc) acc = fmac(acc, L.matel(i, k, m, nc), shfl(mask, yv, src_lane(nc)));
    };
    if (!PER) {
      if (i == n) {
        pull(4, y4); pull(5, y3); pull(1, y2); pull(2, y1);
      } else if (i == n - 1) {
        pull(5, y3); pull(1, y2); pull(2, y1);
      } else if (i >= 3) {
        pull(1, y2); pull(2, y1);
      } else if (i == 2) {
        pull(2, y1);
      }
    } else {
      if (i >= 3) pull(1, y2);
      if (i >= 2) pull(2, y1);
    }
    // in-block lower factor
#pragma unroll
    for (int nc = 0; nc < 4; ++nc) {
      const T xb = shfl(mask, acc, src_lane(nc));
      if (m > nc) acc = fmac(acc, L.matel(i, 3, m, nc), xb);
    }
    if (store) grhs[5 * L.rec(i) + m] = acc;
    if (PER) {  // push into rows n-1, n through their fill at column i
      const bool to1 = i <= n - 4, to0 = i <= n - 3;
#pragma unroll
      for (int nc = 0; nc < 5; ++nc) {
        const T yb = shfl(mask, acc, src_lane(nc));
        if (to1) rn1 = fmac(rn1, L.per2el(i, 0, m, nc), yb);
        if (to0) rn0 = fmac(rn0, L.per2el(i, 1, m, nc), yb);
      }
    }
    y4 = y3; y3 = y2; y2 = y1; y1 = acc;
  }
  cp_async_wait<0>();
  __syncwarp();

  // ----------------------------------------------------------- backward
  // Rows n-kDepth..n are still staged.  After row i is done its slot takes
  // row i-kDepth-1, so a row is staged kDepth iterations before its use.
  // Each lane reads the forward value it wrote itself from global memory.
  T x1 = zero<T>(), x2 = zero<T>(), x3 = zero<T>(), x4 = zero<T>();  // x of rows i+1..i+4
  T xn1 = zero<T>(), xn0 = zero<T>();                                  // periodic x of rows n-1, n
  for (int i = n; i >= 1; --i) {
    if (i < n - kDepth) {
      cp_async_wait<kDepth>();
      __syncwarp();
    }
    T acc = grhs[5 * L.rec(i) + m];
    // right blocks, per column q then ascending block column (src/cpenta1bc.f:760-847)
    if (!PER) {
      if (i == 1) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          acc = fmsc(acc, L.matel(i, 4, m, q), shfl(mask, x1, src_lane(q)));
          acc = fmsc(acc, L.matel(i, 5, m, q), shfl(mask, x2, src_lane(q)));
          acc = fmsc(acc, L.matel(i, 1, m, q), shfl(mask, x3, src_lane(q)));
          acc = fmsc(acc, L.matel(i, 2, m, q), shfl(mask, x4, src_lane(q)));
        }
      } else if (i == 2) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          acc = fmsc(acc, L.matel(i, 4, m, q), shfl(mask, x1, src_lane(q)));
          acc = fmsc(acc, L.matel(i, 5, m, q), shfl(mask, x2, src_lane(q)));
          acc = fmsc(acc, L.matel(i, 1, m, q), shfl(mask, x3, src_lane(q)));
        }
      } else if (i <= n - 2) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          acc = fmsc(acc, L.matel(i, 4, m, q), shfl(mask, x1, src_lane(q)));
          acc = fmsc(acc, L.matel(i, 5, m, q), shfl(mask, x2, src_lane(q)));
        }
      } else if (i == n - 1) {
#pragma unroll
        for (int q = 0; q < 5; ++q) acc = fmsc(acc, L.matel(i, 4, m, q), shfl(mask, x1, src_lane(q)));
      }
    } else {
      if (i <= n - 4) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          acc = fmsc(acc, L.matel(i, 4, m, q), shfl(mask, x1, src_lane(q)));
          acc = fmsc(acc, L.matel(i, 5, m, q), shfl(mask, x2, src_lane(q)));
          acc = fmsc(acc, L.perel(i, 1, m, q), shfl(mask, xn1, src_lane(q)));
          acc = fmsc(acc, L.perel(i, 2, m, q), shfl(mask, xn0, src_lane(q)));
        }
      } else if (i == n - 3) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          acc = fmsc(acc, L.matel(i, 4, m, q), shfl(mask, x1, src_lane(q)));
          acc = fmsc(acc, L.matel(i, 5, m, q), shfl(mask, x2, src_lane(q)));
          acc = fmsc(acc, L.perel(i, 2, m, q), shfl(mask, xn0, src_lane(q)));
        }
      } else if (i == n - 2) {
#pragma unroll
        for (int q = 0; q < 5; ++q) {
          acc = fmsc(acc, L.matel(i, 4, m, q), shfl(mask, x1, src_lane(q)));
          acc = fmsc(acc, L.matel(i, 5, m, q), shfl(mask, x2, src_lane(q)));
        }
      } else if (i == n - 1) {
#pragma unroll
        for (int q = 0; q < 5; ++q) acc = fmsc(acc, L.matel(i, 4, m, q), shfl(mask, x1, src_lane(q)));
      }
    }
    // upper factor of the diagonal block
    const T rd = rcp(L.matel(i, 3, m, m));
#pragma unroll
    for (int mm = 4; mm >= 0; --mm) {
      const T xm = shfl(mask, mul(acc, rd), src_lane(mm));
      if (m < mm) acc = fmsc(acc, L.matel(i, 3, m, mm), xm);
      if (m == mm) acc = xm;
    }
    if (store) grhs[5 * L.rec(i) + m] = acc;
    if (i == n) xn0 = acc;
    if (i == n - 1) xn1 = acc;
    x4 = x3; x3 = x2; x2 = x1; x1 = acc;
    __syncwarp();
    if (i - kDepth - 1 >= 1) stage_row<T, PER>(base, args, i - kDepth - 1, lane);
    cp_async_commit();
  }
  cp_async_wait<0>();
  if (PER && store) grhs[5 * L.rec(n + 1) + m] = x1;  // row np repeats row 1
}

}  // namespace lns
