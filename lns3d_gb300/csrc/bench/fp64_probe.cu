// Peak-rate probe of the benchmark's FP64 roofline (measurement tooling,
// built into its own library, lib/liblns3d_probe.so, that only bench.py
// loads): a dependent-free DFMA stream (eight independent chains per thread,
// every lane active, 32 warps per SM) timed with CUDA events.  Returns the
// rate in TFLOP/s, or a negative value on failure.
#include <cuda_runtime.h>

namespace {
__global__ void dfma_stream(double* out, int iters, double a, double b) {
  double acc[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) acc[k] = threadIdx.x + k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = fma(acc[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += acc[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" double lns_probe_fp64_tflops(void) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return -1.0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1.0;
  const int threads = 1024, iters = 4096;
  double* out = nullptr;
  if (cudaMalloc(&out, (size_t)sms * threads * sizeof(double)) != cudaSuccess) return -1.0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    cudaEventRecord(e0);
    dfma_stream<<<sms, threads>>>(out, iters, 1.0000001, 1e-9);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0;
    cudaEventElapsedTime(&ms, e0, e1);
    if (rep > 0 && ms < best) best = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  const double flops = 2.0 * sms * threads * (double)iters * 8;
  return flops / (best * 1e-3) / 1e12;
}
