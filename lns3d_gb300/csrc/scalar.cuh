// Scalar arithmetic shared by the line-solver kernels: real double, complex
// double (interleaved re/im, the layout of Fortran complex*16) and their FP32
// counterparts.  Every multiply-add is a fused multiply-add.
#pragma once
#include <cuda_runtime.h>

namespace lns {

struct cd {
  double x, y;
};
struct cf {
  float x, y;
};

template <typename T> struct real_of;
template <> struct real_of<double> { using type = double; };
template <> struct real_of<float> { using type = float; };
template <> struct real_of<cd> { using type = double; };
template <> struct real_of<cf> { using type = float; };

template <typename T> __device__ __forceinline__ T zero();
template <> __device__ __forceinline__ double zero<double>() { return 0.0; }
template <> __device__ __forceinline__ float zero<float>() { return 0.0f; }
template <> __device__ __forceinline__ cd zero<cd>() { return cd{0.0, 0.0}; }
template <> __device__ __forceinline__ cf zero<cf>() { return cf{0.0f, 0.0f}; }

// acc + a*b
__device__ __forceinline__ double fmac(double acc, double a, double b) { return fma(a, b, acc); }
__device__ __forceinline__ float fmac(float acc, float a, float b) { return fmaf(a, b, acc); }
__device__ __forceinline__ cd fmac(cd acc, cd a, cd b) {
  cd r;
  r.x = fma(a.x, b.x, fma(-a.y, b.y, acc.x));
  r.y = fma(a.x, b.y, fma(a.y, b.x, acc.y));
  return r;
}
__device__ __forceinline__ cf fmac(cf acc, cf a, cf b) {
  cf r;
  r.x = fmaf(a.x, b.x, fmaf(-a.y, b.y, acc.x));
  r.y = fmaf(a.x, b.y, fmaf(a.y, b.x, acc.y));
  return r;
}
// acc - a*b
__device__ __forceinline__ double fmsc(double acc, double a, double b) { return fma(-a, b, acc); }
__device__ __forceinline__ float fmsc(float acc, float a, float b) { return fmaf(-a, b, acc); }
__device__ __forceinline__ cd fmsc(cd acc, cd a, cd b) {
  cd r;
  r.x = fma(-a.x, b.x, fma(a.y, b.y, acc.x));
  r.y = fma(-a.x, b.y, fma(-a.y, b.x, acc.y));
  return r;
}
__device__ __forceinline__ cf fmsc(cf acc, cf a, cf b) {
  cf r;
  r.x = fmaf(-a.x, b.x, fmaf(a.y, b.y, acc.x));
  r.y = fmaf(-a.x, b.y, fmaf(-a.y, b.x, acc.y));
  return r;
}
// -(a*b)
__device__ __forceinline__ double negmul(double a, double b) { return -(a * b); }
__device__ __forceinline__ float negmul(float a, float b) { return -(a * b); }
__device__ __forceinline__ cd negmul(cd a, cd b) {
  cd r;
  r.x = fma(a.y, b.y, -(a.x * b.x));
  r.y = fma(-a.x, b.y, -(a.y * b.x));
  return r;
}
__device__ __forceinline__ cf negmul(cf a, cf b) {
  cf r;
  r.x = fmaf(a.y, b.y, -(a.x * b.x));
  r.y = fmaf(-a.x, b.y, -(a.y * b.x));
  return r;
}
__device__ __forceinline__ double mul(double a, double b) { return a * b; }
__device__ __forceinline__ float mul(float a, float b) { return a * b; }
__device__ __forceinline__ cd mul(cd a, cd b) {
  return cd{fma(a.x, b.x, -(a.y * b.y)), fma(a.x, b.y, a.y * b.x)};
}
__device__ __forceinline__ cf mul(cf a, cf b) {
  return cf{fmaf(a.x, b.x, -(a.y * b.y)), fmaf(a.x, b.y, a.y * b.x)};
}
__device__ __forceinline__ double add(double a, double b) { return a + b; }
__device__ __forceinline__ float add(float a, float b) { return a + b; }
__device__ __forceinline__ cd add(cd a, cd b) { return cd{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ cf add(cf a, cf b) { return cf{a.x + b.x, a.y + b.y}; }
__device__ __forceinline__ double sub(double a, double b) { return a - b; }
__device__ __forceinline__ float sub(float a, float b) { return a - b; }
__device__ __forceinline__ cd sub(cd a, cd b) { return cd{a.x - b.x, a.y - b.y}; }
__device__ __forceinline__ cf sub(cf a, cf b) { return cf{a.x - b.x, a.y - b.y}; }

// Reciprocal.  Complex: conj(d) / |d|^2, valid while |d| stays within
// 1e-150 .. 1e150 (the diagonal blocks of the implicit operator are O(1)).
__device__ __forceinline__ double rcp(double d) { return 1.0 / d; }
__device__ __forceinline__ float rcp(float d) { return 1.0f / d; }
__device__ __forceinline__ cd rcp(cd d) {
  double s = 1.0 / fma(d.x, d.x, d.y * d.y);
  return cd{d.x * s, -d.y * s};
}
__device__ __forceinline__ cf rcp(cf d) {
  float s = 1.0f / fmaf(d.x, d.x, d.y * d.y);
  return cf{d.x * s, -d.y * s};
}

// Conversions between precisions.
__device__ __forceinline__ float to_lo(double a) { return (float)a; }
__device__ __forceinline__ cf to_lo(cd a) { return cf{(float)a.x, (float)a.y}; }
__device__ __forceinline__ double to_hi(float a) { return (double)a; }
__device__ __forceinline__ cd to_hi(cf a) { return cd{(double)a.x, (double)a.y}; }
__device__ __forceinline__ double to_hi(double a) { return a; }
__device__ __forceinline__ cd to_hi(cd a) { return a; }

__device__ __forceinline__ bool finite_s(double a) { return isfinite(a); }
__device__ __forceinline__ bool finite_s(float a) { return isfinite(a); }
__device__ __forceinline__ bool finite_s(cd a) { return isfinite(a.x) && isfinite(a.y); }
__device__ __forceinline__ bool finite_s(cf a) { return isfinite(a.x) && isfinite(a.y); }

// Warp shuffles of the scalar types.
__device__ __forceinline__ double shfl(unsigned mask, double v, int src) { return __shfl_sync(mask, v, src); }
__device__ __forceinline__ float shfl(unsigned mask, float v, int src) { return __shfl_sync(mask, v, src); }
__device__ __forceinline__ cd shfl(unsigned mask, cd v, int src) {
  return cd{__shfl_sync(mask, v.x, src), __shfl_sync(mask, v.y, src)};
}
__device__ __forceinline__ cf shfl(unsigned mask, cf v, int src) {
  return cf{__shfl_sync(mask, v.x, src), __shfl_sync(mask, v.y, src)};
}

}  // namespace lns
