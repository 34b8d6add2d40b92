// C ABI of the line solvers (declared in include/lns3d_gb300.h).
//
// Host-pointer entry points stage the caller's arrays through device
// buffers owned by this library (grown on demand, reused across calls,
// guarded by a mutex), launch on the legacy default stream and copy the
// results back; device-pointer entry points only validate and launch.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/lns3d_gb300.h"
#include "penta_direct.cuh"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
int cuda_fail(cudaError_t e, const char* where) {
  return fail(LNS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Device staging buffers of the host-pointer entry points.
struct Staging {
  std::mutex mu;
  void* buf[4] = {nullptr, nullptr, nullptr, nullptr};
  size_t cap[4] = {0, 0, 0, 0};
  int* status = nullptr;
  int device = -1;
};
Staging g_stage;

int stage_get(int slot, size_t bytes, void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (g_stage.device != dev) {  // buffers belong to the device they were made on
    for (int s = 0; s < 4; ++s) g_stage.buf[s] = nullptr, g_stage.cap[s] = 0;
    g_stage.status = nullptr;
    g_stage.device = dev;
  }
  if (!g_stage.status) {
    e = cudaMalloc(&g_stage.status, sizeof(int));
    if (e != cudaSuccess) return fail(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  if (g_stage.cap[slot] < bytes) {
    if (g_stage.buf[slot]) cudaFree(g_stage.buf[slot]);
    g_stage.buf[slot] = nullptr;
    g_stage.cap[slot] = 0;
    e = cudaMalloc(&g_stage.buf[slot], bytes);
    if (e != cudaSuccess) return fail(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    g_stage.cap[slot] = bytes;
  }
  *out = g_stage.buf[slot];
  return LNS_OK;
}

int check_sizes(int n, int nsys, int nblk, const char* who) {
  if (nblk != 5) return fail(LNS_ERR_ARG, std::string(who) + ": nblk must be 5");
  if (n < 7) return fail(LNS_ERR_ARG, std::string(who) + ": lines need at least 7 rows");
  if (nsys < 0) return fail(LNS_ERR_ARG, std::string(who) + ": nsys < 0");
  return LNS_OK;
}

template <typename T>
int launch_bc(void* mat, void* rhs, int n, int nsys, long long row_stride, long long line_stride, int code,
              cudaStream_t st, int* status) {
  if (nsys == 0) return LNS_OK;
  lns::PentaArgs a{mat, rhs, n, nsys, row_stride, line_stride, code, status};
  const int blocks = (nsys + lns::kWarpsPerCta - 1) / lns::kWarpsPerCta;
  const size_t smem = (size_t)lns::kWarpsPerCta * (lns::kRing * lns::kRowSz + 16) * sizeof(T);
  lns::penta_bc_kernel<T><<<blocks, 32 * lns::kWarpsPerCta, smem, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "penta_bc_kernel launch");
  return LNS_OK;
}

// Host-pointer form: stage, solve, copy back.
template <typename T>
int host_bc(double* mat, double* rhs, int n, int nsys, long long row_stride, long long line_stride, int code,
            bool copy_back_mat) {
  if (nsys == 0) return LNS_OK;
  std::lock_guard<std::mutex> lock(g_stage.mu);
  const size_t mat_bytes = (size_t)125 * n * nsys * sizeof(T);
  const size_t rhs_bytes = (size_t)5 * n * nsys * sizeof(T);
  void *dm = nullptr, *dr = nullptr;
  int rc = stage_get(0, mat_bytes, &dm);
  if (rc) return rc;
  rc = stage_get(1, rhs_bytes, &dr);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(dm, mat, mat_bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "copy mat to device");
  if (code != 0) {
    e = cudaMemcpy(dr, rhs, rhs_bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(e, "copy rhs to device");
  }
  e = cudaMemset(g_stage.status, 0, sizeof(int));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemset");
  rc = launch_bc<T>(dm, dr, n, nsys, row_stride, line_stride, code, 0, g_stage.status);
  if (rc) return rc;
  if (copy_back_mat) {
    e = cudaMemcpy(mat, dm, mat_bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "copy mat to host");
  }
  if (code != 0) {
    e = cudaMemcpy(rhs, dr, rhs_bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "copy rhs to host");
  }
  int status = 0;
  e = cudaMemcpy(&status, g_stage.status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "copy status to host");
  if (status) return fail(LNS_ERR_PIVOT, "zero or non-finite pivot");
  return LNS_OK;
}

}  // namespace

extern "C" {

const char* lns_last_error(void) { return g_err.c_str(); }
const char* lns_version(void) { return "lns3d_gb300 0.1 (sm_103a)"; }

int lns_penta2bc(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs) {
  int rc = check_sizes(n, nsys, nblk, "penta2bc");
  if (rc) return rc;
  return host_bc<double>(mat, rhs, n, nsys, 1, n, 2, false);
}
int lns_penta2bc_dev(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs, void* stream) {
  int rc = check_sizes(n, nsys, nblk, "penta2bc");
  if (rc) return rc;
  return launch_bc<double>(mat, rhs, n, nsys, 1, n, 2, (cudaStream_t)stream, nullptr);
}
int lns_penta1bc(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs) {
  int rc = check_sizes(n, nsys, nblk, "penta1bc");
  if (rc) return rc;
  return host_bc<double>(mat, rhs, n, nsys, nsys, 1, 2, false);
}
int lns_penta1bc_dev(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs, void* stream) {
  int rc = check_sizes(n, nsys, nblk, "penta1bc");
  if (rc) return rc;
  return launch_bc<double>(mat, rhs, n, nsys, nsys, 1, 2, (cudaStream_t)stream, nullptr);
}

int lns_cpenta2bc(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs, int32_t code) {
  int rc = check_sizes(n, nsys, nblk, "cpenta2bc");
  if (rc) return rc;
  if (code < 0 || code > 2) return fail(LNS_ERR_ARG, "cpenta2bc: code must be 0, 1 or 2");
  return host_bc<lns::cd>(mat, rhs, n, nsys, 1, n, code, code != 1);
}
int lns_cpenta2bc_dev(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs, int32_t code,
                      void* stream) {
  int rc = check_sizes(n, nsys, nblk, "cpenta2bc");
  if (rc) return rc;
  if (code < 0 || code > 2) return fail(LNS_ERR_ARG, "cpenta2bc: code must be 0, 1 or 2");
  return launch_bc<lns::cd>(mat, rhs, n, nsys, 1, n, code, (cudaStream_t)stream, nullptr);
}
int lns_cpenta1bc(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs, int32_t code) {
  int rc = check_sizes(n, nsys, nblk, "cpenta1bc");
  if (rc) return rc;
  if (code < 0 || code > 2) return fail(LNS_ERR_ARG, "cpenta1bc: code must be 0, 1 or 2");
  return host_bc<lns::cd>(mat, rhs, n, nsys, nsys, 1, code, code != 1);
}
int lns_cpenta1bc_dev(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs, int32_t code,
                      void* stream) {
  int rc = check_sizes(n, nsys, nblk, "cpenta1bc");
  if (rc) return rc;
  if (code < 0 || code > 2) return fail(LNS_ERR_ARG, "cpenta1bc: code must be 0, 1 or 2");
  return launch_bc<lns::cd>(mat, rhs, n, nsys, nsys, 1, code, (cudaStream_t)stream, nullptr);
}

}  // extern "C"
