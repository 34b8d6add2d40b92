// Mixed-precision line solves: FP32 LU factors, FP64 residuals.
//
// The FP64 pipe of the GB300 runs at 1/64 of the FP32 rate, so the factor
// and the triangular solves run in FP32 (the same kernels as the FP64 path,
// instantiated for float), and accuracy is restored by iterative refinement
//   x <- x + LU32^{-1} (b - A x)
// with the residual formed in FP64 from the untouched FP64 matrix.  Each
// refinement multiplies the error by about cond(A) * 2^-24; two steps bring
// a well-conditioned system to FP64 rounding.  With zero refinement steps
// this is the FP32 interior solve of the mixed ADI step.
#pragma once
#include "penta_direct.cuh"

namespace lns {

// FP64 -> FP32 copy of n elements (complex: 2n doubles).
template <typename TH, typename TL>
__global__ void narrow_kernel(const TH* __restrict__ src, TL* __restrict__ dst, long long n) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x)
    dst[k] = to_lo(src[k]);
}

// x (FP64) += d (FP32), or x = d when init.
template <typename TH, typename TL>
__global__ void widen_add_kernel(TH* __restrict__ x, const TL* __restrict__ d, long long n, int init) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += (long long)gridDim.x * blockDim.x) {
    const TH v = to_hi(d[k]);
    x[k] = init ? v : add(x[k], v);
  }
}

struct ResidualArgs {
  const void* mat;   // FP64 matrix, reference layout
  const void* b;     // FP64 right-hand side
  const void* x;     // FP64 iterate
  void* r;           // FP32 residual out
  int n, nrows, nsys;
  long long row_stride, line_stride;
  int periodic;
};

// Column (1-based) of slot k (1..5) of row i.
__device__ __forceinline__ int col_of(int i, int k, int n, int periodic) {
  if (periodic) return ((i + k - 4) % n + n) % n + 1;
  if (i == 1) { const int c[5] = {4, 5, 1, 2, 3}; return c[k - 1]; }
  if (i == 2) { const int c[5] = {5, 1, 2, 3, 4}; return c[k - 1]; }
  if (i == n - 1) { const int o[5] = {-3, -2, -1, 0, -4}; return n + o[k - 1]; }
  if (i == n) { const int o[5] = {-2, -1, 0, -4, -3}; return n + o[k - 1]; }
  return i + k - 3;
}

// r = b - A x for every block row; one thread per (row, block row m).
// Threads are ordered (line, row, m) so that the five threads of a row read
// its 2000-byte matrix record together.
template <typename TH, typename TL>
__global__ void residual_kernel(ResidualArgs a) {
  const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  const long long total = (long long)a.nsys * a.n * 5;
  if (tid >= total) return;
  const int m = (int)(tid % 5);
  const long long rowid = tid / 5;
  const int i = (int)(rowid % a.n) + 1;
  const int iv = (int)(rowid / a.n);
  const long long rec = a.row_stride * (i - 1) + a.line_stride * iv;
  const TH* A = reinterpret_cast<const TH*>(a.mat) + 125 * rec;
  const TH* X = reinterpret_cast<const TH*>(a.x);
  TH acc = reinterpret_cast<const TH*>(a.b)[5 * rec + m];
#pragma unroll
  for (int k = 1; k <= 5; ++k) {
    const int c = col_of(i, k, a.n, a.periodic);
    const TH* xc = X + 5 * (a.row_stride * (c - 1) + a.line_stride * iv);
#pragma unroll
    for (int q = 0; q < 5; ++q) acc = fmsc(acc, A[(k - 1) + 5 * m + 25 * q], xc[q]);
  }
  reinterpret_cast<TL*>(a.r)[5 * rec + m] = to_lo(acc);
}

// Periodic lines: row np of the solution repeats row 1.
template <typename T>
__global__ void copy_periodic_row_kernel(T* x, int np, int nsys, long long row_stride, long long line_stride) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nsys * 5) return;
  const int iv = t / 5, m = t % 5;
  x[5 * (row_stride * (np - 1) + line_stride * iv) + m] = x[5 * (line_stride * iv) + m];
}

}  // namespace lns
