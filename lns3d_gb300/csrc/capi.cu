// C ABI of the line solvers (declared in include/lns3d_gb300.h).
//
// Host-pointer entry points stage the caller's arrays through device
// buffers owned by this library (grown on demand, reused across calls,
// guarded by a mutex), launch on the legacy default stream and copy the
// results back; device-pointer entry points only validate and launch.
#include <cuda_runtime.h>

#include <cstdio>
#include <cstring>
#include <algorithm>
#include <atomic>
#include <mutex>
#include <string>
#include <type_traits>

#include "../../include/lns3d_gb300.h"
#include "launch.cuh"

static thread_local std::string g_err;
std::atomic<int> g_periodic_exact{0};

int lns_fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}
int lns_cuda_fail(cudaError_t e, const char* where) {
  return lns_fail(LNS_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

namespace {

using lns::host::launch_bc;
using lns::host::launch_p;
using lns::host::launch_solve;
int fail(int code, const std::string& msg) { return lns_fail(code, msg); }
int cuda_fail(cudaError_t e, const char* where) { return lns_cuda_fail(e, where); }

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

template <typename T>
int host_p(double* mat, double* rhs, double* per, double* per2, int np, int nsys, long long row_stride,
           long long line_stride, int code) {
  if (nsys == 0) return LNS_OK;
  const bool cplx = sizeof(T) == 16;
  std::lock_guard<std::mutex> lock(g_stage.mu);
  const size_t mat_b = (size_t)125 * np * nsys * sizeof(T);
  const size_t rhs_b = (size_t)5 * np * nsys * sizeof(T);
  const size_t per_b = (size_t)50 * np * nsys * sizeof(T);
  void *dm, *dr, *dp, *dp2 = nullptr;
  int rc = stage_get(0, mat_b, &dm);
  if (!rc) rc = stage_get(1, rhs_b, &dr);
  if (!rc) rc = stage_get(2, per_b, &dp);
  if (!rc && cplx) rc = stage_get(3, per_b, &dp2);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(dm, mat, mat_b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && code != 0) e = cudaMemcpy(dr, rhs, rhs_b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && code == 1) e = cudaMemcpy(dp, per, per_b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && code == 1 && cplx) e = cudaMemcpy(dp2, per2, per_b, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "copy to device");
  e = cudaMemset(g_stage.status, 0, sizeof(int));
  if (e != cudaSuccess) return cuda_fail(e, "cudaMemset");
  rc = launch_p<T>(dm, dr, dp, dp2, np, nsys, row_stride, line_stride, code, 0, g_stage.status);
  if (rc) return rc;
  if (cplx && code != 1) {
    e = cudaMemcpy(mat, dm, mat_b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(per, dp, per_b, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(per2, dp2, per_b, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "copy factors to host");
  }
  if (code != 0) {
    e = cudaMemcpy(rhs, dr, rhs_b, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "copy rhs to host");
  }
  int status = 0;
  e = cudaMemcpy(&status, g_stage.status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "copy status to host");
  if (status) return fail(LNS_ERR_PIVOT, "zero or non-finite pivot");
  return LNS_OK;
}

// ---------------------------------------------------------------- mixed
// Workspace of a mixed-precision solve of `rows` x `nsys` block rows:
// FP32 matrix factors, FP32 periodic fill (per, per2), FP32 residual /
// correction, FP64 iterate.
struct MixedLayout {
  size_t w, per, per2, r, x, total;
};
size_t align256(size_t b) { return (b + 255) & ~size_t(255); }
MixedLayout mixed_layout(int rows, int nsys, bool cplx, bool periodic) {
  const size_t el32 = cplx ? 8 : 4, el64 = cplx ? 16 : 8, rs = (size_t)rows * nsys;
  MixedLayout L{};
  size_t off = 0;
  L.w = off; off += align256(125 * rs * el32);
  L.per = off; off += periodic ? align256(50 * rs * el32) : 0;
  L.per2 = off; off += periodic ? align256(50 * rs * el32) : 0;
  L.r = off; off += align256(5 * rs * el32);
  L.x = off; off += align256(5 * rs * el64);
  L.total = off;
  return L;
}

int grid_for(long long n) {
  long long b = (n + 255) / 256;
  return (int)std::min<long long>(std::max<long long>(b, 1), 152 * 32);
}

// code 0: factor (FP32) into work; 1: solve with `refine` FP64 refinement
// steps; 2: both.  mat is read only.
template <typename TH, typename TL>
int mixed_solve(const double* mat, double* rhs, int rows, int nsys, long long row_stride, long long line_stride,
                bool periodic, int code, int refine, void* work, cudaStream_t st) {
  if (nsys == 0) return LNS_OK;
  const bool cplx = std::is_same<TH, lns::cd>::value;
  const MixedLayout Lw = mixed_layout(rows, nsys, cplx, periodic);
  char* wb = reinterpret_cast<char*>(work);
  TL* W = reinterpret_cast<TL*>(wb + Lw.w);
  TL* P = reinterpret_cast<TL*>(wb + Lw.per);
  TL* P2 = reinterpret_cast<TL*>(wb + Lw.per2);
  TL* R = reinterpret_cast<TL*>(wb + Lw.r);
  TH* X = reinterpret_cast<TH*>(wb + Lw.x);
  const long long nmat = 125LL * rows * nsys, nrhs = 5LL * rows * nsys;
  const int n = periodic ? rows - 1 : rows;
  int rc = LNS_OK;
  cudaError_t e;
  if (code != 1) {
    lns::narrow_kernel<TH, TL><<<grid_for(nmat), 256, 0, st>>>(reinterpret_cast<const TH*>(mat), W, nmat);
    rc = periodic ? launch_p<TL>(W, R, P, P2, rows, nsys, row_stride, line_stride, 0, st, nullptr, 1)
                  : launch_bc<TL>(W, R, rows, nsys, row_stride, line_stride, 0, st, nullptr);
    if (rc) return rc;
  }
  if (code != 0) {
    lns::narrow_kernel<TH, TL><<<grid_for(nrhs), 256, 0, st>>>(reinterpret_cast<const TH*>(rhs), R, nrhs);
    for (int it = 0; it <= refine; ++it) {
      if (it > 0) {
        lns::ResidualArgs ra{mat, rhs, X, R, n, rows, nsys, row_stride, line_stride, periodic ? 1 : 0};
        const long long th = 5LL * n * nsys;
        lns::residual_kernel<TH, TL><<<(unsigned)((th + 255) / 256), 256, 0, st>>>(ra);
      }
      rc = periodic ? launch_p<TL>(W, R, P, P2, rows, nsys, row_stride, line_stride, 1, st, nullptr, 1)
                    : launch_bc<TL>(W, R, rows, nsys, row_stride, line_stride, 1, st, nullptr);
      if (rc) return rc;
      lns::widen_add_kernel<TH, TL><<<grid_for(nrhs), 256, 0, st>>>(X, R, nrhs, it == 0 ? 1 : 0);
    }
    e = cudaMemcpyAsync(rhs, X, nrhs * sizeof(TH), cudaMemcpyDeviceToDevice, st);
    if (e != cudaSuccess) return cuda_fail(e, "mixed solve copy-out");
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "mixed solve launch");
  return LNS_OK;
}

// Host-pointer form of the mixed solve (factor + solve), staged like host_bc.
template <typename TH, typename TL>
int host_mixed(const double* mat, double* rhs, int rows, int nsys, long long row_stride, long long line_stride,
               bool periodic, int refine) {
  if (nsys == 0) return LNS_OK;
  std::lock_guard<std::mutex> lock(g_stage.mu);
  const bool cplx = std::is_same<TH, lns::cd>::value;
  const size_t mat_b = (size_t)125 * rows * nsys * sizeof(TH);
  const size_t rhs_b = (size_t)5 * rows * nsys * sizeof(TH);
  const size_t work_b = mixed_layout(rows, nsys, cplx, periodic).total;
  void *dm, *dr, *dw;
  int rc = stage_get(0, mat_b, &dm);
  if (!rc) rc = stage_get(1, rhs_b, &dr);
  if (!rc) rc = stage_get(2, work_b, &dw);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(dm, mat, mat_b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dr, rhs, rhs_b, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(e, "copy to device");
  rc = mixed_solve<TH, TL>(reinterpret_cast<const double*>(dm), reinterpret_cast<double*>(dr), rows, nsys,
                           row_stride, line_stride, periodic, 2, refine, dw, 0);
  if (rc) return rc;
  e = cudaMemcpy(rhs, dr, rhs_b, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "copy rhs to host");
  return LNS_OK;
}

int check_mixed(int code, int refine, const char* who) {
  if (code < 0 || code > 2) return fail(LNS_ERR_ARG, std::string(who) + ": code must be 0, 1 or 2");
  if (refine < 0 || refine > 16) return fail(LNS_ERR_ARG, std::string(who) + ": refine must be 0..16");
  return LNS_OK;
}

int check_p(int np, int nsys, int nblk, const char* who) {
  if (nblk != 5) return fail(LNS_ERR_ARG, std::string(who) + ": nblk must be 5");
  if (np < 8) return fail(LNS_ERR_ARG, std::string(who) + ": periodic lines need np >= 8");
  if (nsys < 0) return fail(LNS_ERR_ARG, std::string(who) + ": nsys < 0");
  return LNS_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// Fixed scratch of lns_cpenta2bc_mixed_static_dev.  A file-scope device
// array, so the entry point never allocates: its address is looked up once
// per device (cudaGetSymbolAddress, with that device current) and cached.
// Nothing in it needs to start at zero: every call writes each scratch
// entry it reads.  All calls on a device share it.
namespace {

constexpr size_t kStaticWorkBytes = size_t(LNS_STATIC_WORKSPACE_BYTES);
static __device__ __align__(256) unsigned char g_static_work[kStaticWorkBytes];

constexpr int kMaxDevices = 64;
std::mutex g_static_mu;
void* g_static_ptr[kMaxDevices] = {};

int static_work(void** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(LNS_ERR_ARG, "static workspace: device ordinal above 63");
  std::lock_guard<std::mutex> lock(g_static_mu);
  if (!g_static_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_work);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(static workspace)");
    g_static_ptr[dev] = p;
  }
  *out = g_static_ptr[dev];
  return LNS_OK;
}

}  // namespace

extern "C" {

size_t lns_mixed_workspace_bytes(int32_t rows, int32_t nsys, int32_t is_complex, int32_t periodic) {
  if (rows <= 0 || nsys < 0) return 0;
  return mixed_layout(rows, nsys, is_complex != 0, periodic != 0).total;
}

int lns_cpenta2bc_mixed_dev(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs, int32_t code,
                            int32_t refine, void* work, void* stream) {
  int rc = check_sizes(n, nsys, nblk, "cpenta2bc_mixed");
  if (!rc) rc = check_mixed(code, refine, "cpenta2bc_mixed");
  if (rc) return rc;
  return mixed_solve<lns::cd, lns::cf>(mat, rhs, n, nsys, 1, n, false, code, refine, work, (cudaStream_t)stream);
}
int lns_cpenta1bc_mixed_dev(int32_t nsys, int32_t n, int32_t nblk, const double* mat, double* rhs, int32_t code,
                            int32_t refine, void* work, void* stream) {
  int rc = check_sizes(n, nsys, nblk, "cpenta1bc_mixed");
  if (!rc) rc = check_mixed(code, refine, "cpenta1bc_mixed");
  if (rc) return rc;
  return mixed_solve<lns::cd, lns::cf>(mat, rhs, n, nsys, nsys, 1, false, code, refine, work, (cudaStream_t)stream);
}
int lns_cpenta2p_mixed_dev(int32_t np, int32_t nsys, int32_t nblk, const double* mat, double* rhs, int32_t code,
                           int32_t refine, void* work, void* stream) {
  int rc = check_p(np, nsys, nblk, "cpenta2p_mixed");
  if (!rc) rc = check_mixed(code, refine, "cpenta2p_mixed");
  if (rc) return rc;
  return mixed_solve<lns::cd, lns::cf>(mat, rhs, np, nsys, 1, np, true, code, refine, work, (cudaStream_t)stream);
}
int lns_cpenta1p_mixed_dev(int32_t nsys, int32_t np, int32_t nblk, const double* mat, double* rhs, int32_t code,
                           int32_t refine, void* work, void* stream) {
  int rc = check_p(np, nsys, nblk, "cpenta1p_mixed");
  if (!rc) rc = check_mixed(code, refine, "cpenta1p_mixed");
  if (rc) return rc;
  return mixed_solve<lns::cd, lns::cf>(mat, rhs, np, nsys, nsys, 1, true, code, refine, work, (cudaStream_t)stream);
}
int lns_cpenta2bc_mixed(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs, int32_t refine) {
  int rc = check_sizes(n, nsys, nblk, "cpenta2bc_mixed");
  if (!rc) rc = check_mixed(2, refine, "cpenta2bc_mixed");
  if (rc) return rc;
  return host_mixed<lns::cd, lns::cf>(mat, rhs, n, nsys, 1, n, false, refine);
}
int lns_penta2bc_mixed_dev(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs, int32_t refine,
                           void* work, void* stream) {
  int rc = check_sizes(n, nsys, nblk, "penta2bc_mixed");
  if (!rc) rc = check_mixed(2, refine, "penta2bc_mixed");
  if (rc) return rc;
  return mixed_solve<double, float>(mat, rhs, n, nsys, 1, n, false, 2, refine, work, (cudaStream_t)stream);
}
int lns_penta1bc_mixed_dev(int32_t nsys, int32_t n, int32_t nblk, const double* mat, double* rhs, int32_t refine,
                           void* work, void* stream) {
  int rc = check_sizes(n, nsys, nblk, "penta1bc_mixed");
  if (!rc) rc = check_mixed(2, refine, "penta1bc_mixed");
  if (rc) return rc;
  return mixed_solve<double, float>(mat, rhs, n, nsys, nsys, 1, false, 2, refine, work, (cudaStream_t)stream);
}

int lns_set_periodic_exact(int32_t on) {
  if (on != 0 && on != 1) return fail(LNS_ERR_ARG, "lns_set_periodic_exact: 0 or 1");
  g_periodic_exact.store(on);
  return LNS_OK;
}

int lns_penta2p(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per, double* per2) {
  int rc = check_p(np, nsys, nblk, "penta2p");
  if (rc) return rc;
  (void)per2;
  return host_p<double>(mat, rhs, per, per2, np, nsys, 1, np, 2);
}
int lns_penta2p_dev(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per,
                    double* per2, void* stream) {
  int rc = check_p(np, nsys, nblk, "penta2p");
  if (rc) return rc;
  return launch_p<double>(mat, rhs, per, per2, np, nsys, 1, np, 2, (cudaStream_t)stream, nullptr);
}
int lns_penta1p(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per, double* per2) {
  int rc = check_p(np, nsys, nblk, "penta1p");
  if (rc) return rc;
  return host_p<double>(mat, rhs, per, per2, np, nsys, nsys, 1, 2);
}
int lns_penta1p_dev(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per,
                    double* per2, void* stream) {
  int rc = check_p(np, nsys, nblk, "penta1p");
  if (rc) return rc;
  return launch_p<double>(mat, rhs, per, per2, np, nsys, nsys, 1, 2, (cudaStream_t)stream, nullptr);
}
int lns_cpenta2p(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per, double* per2,
                 int32_t code) {
  int rc = check_p(np, nsys, nblk, "cpenta2p");
  if (rc) return rc;
  if (code < 0 || code > 2) return fail(LNS_ERR_ARG, "cpenta2p: code must be 0, 1 or 2");
  return host_p<lns::cd>(mat, rhs, per, per2, np, nsys, 1, np, code);
}
int lns_cpenta2p_dev(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per,
                     double* per2, int32_t code, void* stream) {
  int rc = check_p(np, nsys, nblk, "cpenta2p");
  if (rc) return rc;
  if (code < 0 || code > 2) return fail(LNS_ERR_ARG, "cpenta2p: code must be 0, 1 or 2");
  return launch_p<lns::cd>(mat, rhs, per, per2, np, nsys, 1, np, code, (cudaStream_t)stream, nullptr);
}
int lns_cpenta1p(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per, double* per2,
                 int32_t code) {
  int rc = check_p(np, nsys, nblk, "cpenta1p");
  if (rc) return rc;
  if (code < 0 || code > 2) return fail(LNS_ERR_ARG, "cpenta1p: code must be 0, 1 or 2");
  return host_p<lns::cd>(mat, rhs, per, per2, np, nsys, nsys, 1, code);
}
int lns_cpenta1p_dev(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per,
                     double* per2, int32_t code, void* stream) {
  int rc = check_p(np, nsys, nblk, "cpenta1p");
  if (rc) return rc;
  if (code < 0 || code > 2) return fail(LNS_ERR_ARG, "cpenta1p: code must be 0, 1 or 2");
  return launch_p<lns::cd>(mat, rhs, per, per2, np, nsys, nsys, 1, code, (cudaStream_t)stream, nullptr);
}


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

int lns_cpenta2bc_mixed_static_dev(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs,
                                   int32_t refine, void* stream) {
  int rc = check_sizes(n, nsys, nblk, "cpenta2bc_mixed_static");
  if (!rc) rc = check_mixed(2, refine, "cpenta2bc_mixed_static");
  if (rc) return rc;
  const size_t need = mixed_layout(n, nsys, true, false).total;
  if (need > kStaticWorkBytes)
    return fail(LNS_ERR_ARG, "cpenta2bc_mixed_static: n = " + std::to_string(n) + ", nsys = " +
                                 std::to_string(nsys) + " needs " + std::to_string(need) +
                                 " bytes of scratch, more than the fixed " + std::to_string(kStaticWorkBytes) +
                                 "-byte static workspace; use lns_cpenta2bc_mixed_dev with a caller workspace");
  void* w = nullptr;
  rc = static_work(&w);
  if (rc) return rc;
  return mixed_solve<lns::cd, lns::cf>(mat, rhs, n, nsys, 1, n, false, 2, refine, w, (cudaStream_t)stream);
}

}  // extern "C"

// ======================================================================
// Block-tridiagonal solvers of the second-order implicit path (iLHS = 0):
// solve1bc / solve2bc (src/nsolve1bc.f90:2, src/nsolve2bc.f90:2) and
// solve1p / solve2p (src/nsolve1p.f90:2, src/nsolve2p.f90:2)
// ======================================================================
// A block-tridiagonal line, with the blocks that its second-order boundary
// rows add (bc(14,5,5,nsys)), is a block-pentadiagonal line whose other
// blocks are zero, and the reference eliminates it in the pentadiagonal
// solvers' order; each line is copied into pentadiagonal records in a
// workspace and solved (factor and right-hand side in one pass) by the
// pentadiagonal kernels.  Updates by the zero blocks add exact zeros.
namespace {

// Source of the block of row t at column c of a boundary-closure line:
// > 0 the mat slot, < 0 minus the bc index, 0 none (src/nsolve2bc.f90:40-420).
__device__ __forceinline__ int tri_src_bc(int t, int c, int n) {
  const int tab[6][5] = {{2, 3, -1, -2, -3},      // row 1, columns 1..5
                         {1, 2, 3, -4, -5},       // row 2
                         {-7, 1, 2, 3, -6},       // row 3
                         {-8, 1, 2, 3, -9},       // row n-2, columns n-4..n
                         {-10, -11, 1, 2, 3},     // row n-1
                         {-12, -13, -14, 1, 2}};  // row n
  int r = -1, c0 = 1;
  if (t <= 3) r = t - 1;
  else if (t >= n - 2) r = t - (n - 2) + 3, c0 = n - 4;
  if (r >= 0) {
    const int a = c - c0;
    return a >= 0 && a < 5 ? tab[r][a] : 0;
  }
  const int k = c - t + 2;
  return k >= 1 && k <= 3 ? k : 0;
}

// Column held by slot k (1..5) of row t of a pentadiagonal boundary-closure
// line (the inverse of lns::slot_bc).
__device__ __forceinline__ int col_of_slot_bc(int t, int k, int n) {
  const int r1[5] = {4, 5, 1, 2, 3}, r2[5] = {5, 1, 2, 3, 4};
  const int o1[5] = {-3, -2, -1, 0, -4}, o0[5] = {-2, -1, 0, -4, -3};
  if (t == 1) return r1[k - 1];
  if (t == 2) return r2[k - 1];
  if (t == n - 1) return n + o1[k - 1];
  if (t == n) return n + o0[k - 1];
  return t + k - 3;
}

// One thread per entry of the pentadiagonal records of rows 1..rows.
__global__ void tri_to_penta_kernel(const double* __restrict__ tmat, const double* __restrict__ bc,
                                    double* __restrict__ pmat, int rows, int n, int nsys, long long rs,
                                    long long ls, int periodic) {
  const long long task = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (task >= (long long)rows * nsys * 125) return;
  const int e = (int)(task % 25), k = (int)((task / 25) % 5) + 1;
  const long long rr = task / 125;
  const int t = (int)(rr % rows) + 1, iv = (int)(rr / rows);
  const long long rec = rs * (t - 1) + ls * iv;
  const int mq = e;  // m + 5 q
  double v = 0.0;
  if (periodic) {
    if (t <= n && k >= 2 && k <= 4) v = tmat[(k - 2) + 3 * mq + 75 * rec];
  } else {
    const int s = tri_src_bc(t, col_of_slot_bc(t, k, n), n);
    if (s > 0) v = tmat[(s - 1) + 3 * mq + 75 * rec];
    else if (s < 0) v = bc[(-s - 1) + 14 * mq + 350LL * iv];
  }
  pmat[(k - 1) + 5 * mq + 125 * rec] = v;
}

size_t tri_work_bytes(int rows, int nsys, bool periodic) {
  return sizeof(double) * (size_t)rows * nsys * (125 + (periodic ? 50 : 0));
}

int check_tri(int rows, int nsys, int nblk, bool periodic, const char* who) {
  if (nblk != 5) return fail(LNS_ERR_ARG, std::string(who) + ": nblk must be 5");
  if (nsys < 0) return fail(LNS_ERR_ARG, std::string(who) + ": nsys < 0");
  if (rows < (periodic ? 9 : 8))
    return fail(LNS_ERR_ARG, std::string(who) + (periodic ? ": lines need np >= 9 rows" : ": lines need n >= 8 rows") +
                                 " (the reference's boundary rows would overlap)");
  return LNS_OK;
}

// Device form: convert into the workspace, then factor and solve.
int tri_dev(int layout, bool periodic, int rows, int nsys, const double* tmat, double* rhs, const double* bc,
            void* work, cudaStream_t st, int* status) {
  if (nsys == 0) return LNS_OK;
  if (!tmat || !rhs || !work || (!periodic && !bc)) return fail(LNS_ERR_ARG, "tridiagonal solve: null argument");
  const int n = periodic ? rows - 1 : rows;
  const long long rs = layout == 2 ? 1 : nsys, ls = layout == 2 ? rows : 1;
  double* pmat = reinterpret_cast<double*>(work);
  double* per = pmat + (size_t)125 * rows * nsys;
  const long long total = (long long)rows * nsys * 125;
  tri_to_penta_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(tmat, bc, pmat, rows, n, nsys, rs, ls,
                                                                      periodic ? 1 : 0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_fail(e, "tri_to_penta_kernel launch");
  if (periodic) return launch_p<double>(pmat, rhs, per, nullptr, rows, nsys, rs, ls, 2, st, status, 1);
  return launch_bc<double>(pmat, rhs, rows, nsys, rs, ls, 2, st, status);
}

// Host form: stage, solve, copy the solution back (mat and bc are left as
// they were; the reference's copies are scratch on return).
int tri_host(int layout, bool periodic, int rows, int nsys, const double* tmat, double* rhs, const double* bc) {
  if (nsys == 0) return LNS_OK;
  if (!tmat || !rhs || (!periodic && !bc)) return fail(LNS_ERR_ARG, "tridiagonal solve: null argument");
  std::lock_guard<std::mutex> lock(g_stage.mu);
  const size_t mat_b = sizeof(double) * 75 * (size_t)rows * nsys, rhs_b = sizeof(double) * 5 * (size_t)rows * nsys;
  const size_t bc_b = sizeof(double) * 350 * (size_t)nsys;
  void *dm = nullptr, *dr = nullptr, *db = nullptr, *dw = nullptr;
  int rc = stage_get(0, mat_b, &dm);
  if (!rc) rc = stage_get(1, rhs_b, &dr);
  if (!rc && !periodic) rc = stage_get(2, bc_b, &db);
  if (!rc) rc = stage_get(3, tri_work_bytes(rows, nsys, periodic), &dw);
  if (rc) return rc;
  cudaError_t e = cudaMemcpy(dm, tmat, mat_b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dr, rhs, rhs_b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && !periodic) e = cudaMemcpy(db, bc, bc_b, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(g_stage.status, 0, sizeof(int));
  if (e != cudaSuccess) return cuda_fail(e, "stage tridiagonal line");
  rc = tri_dev(layout, periodic, rows, nsys, (const double*)dm, (double*)dr, (const double*)db, dw, 0,
               g_stage.status);
  if (rc) return rc;
  e = cudaMemcpy(rhs, dr, rhs_b, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "copy rhs to host");
  int status = 0;
  e = cudaMemcpy(&status, g_stage.status, sizeof(int), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(e, "copy status to host");
  if (status) return fail(LNS_ERR_PIVOT, "zero or non-finite pivot");
  return LNS_OK;
}

}  // namespace

extern "C" {

size_t lns_tri_workspace_bytes(int32_t rows, int32_t nsys, int32_t periodic) {
  if (rows < 1 || nsys < 0) return 0;
  return tri_work_bytes(rows, nsys, periodic != 0);
}

int lns_solve2bc(int32_t n, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* bc) {
  int rc = check_tri(n, nsys, nblk, false, "solve2bc");
  return rc ? rc : tri_host(2, false, n, nsys, mat, rhs, bc);
}
int lns_solve1bc(int32_t nsys, int32_t n, int32_t nblk, double* mat, double* rhs, double* bc) {
  int rc = check_tri(n, nsys, nblk, false, "solve1bc");
  return rc ? rc : tri_host(1, false, n, nsys, mat, rhs, bc);
}
int lns_solve2p(int32_t np, int32_t nsys, int32_t nblk, double* mat, double* rhs, double* per, double* per2) {
  (void)per, (void)per2;  // the reference's fill scratch; the GPU keeps its fill in the workspace
  int rc = check_tri(np, nsys, nblk, true, "solve2p");
  return rc ? rc : tri_host(2, true, np, nsys, mat, rhs, nullptr);
}
int lns_solve1p(int32_t nsys, int32_t np, int32_t nblk, double* mat, double* rhs, double* per, double* per2) {
  (void)per, (void)per2;
  int rc = check_tri(np, nsys, nblk, true, "solve1p");
  return rc ? rc : tri_host(1, true, np, nsys, mat, rhs, nullptr);
}
int lns_solve2bc_dev(int32_t n, int32_t nsys, int32_t nblk, const double* mat, double* rhs, const double* bc,
                     void* work, void* stream) {
  int rc = check_tri(n, nsys, nblk, false, "solve2bc");
  return rc ? rc : tri_dev(2, false, n, nsys, mat, rhs, bc, work, (cudaStream_t)stream, nullptr);
}
int lns_solve1bc_dev(int32_t nsys, int32_t n, int32_t nblk, const double* mat, double* rhs, const double* bc,
                     void* work, void* stream) {
  int rc = check_tri(n, nsys, nblk, false, "solve1bc");
  return rc ? rc : tri_dev(1, false, n, nsys, mat, rhs, bc, work, (cudaStream_t)stream, nullptr);
}
int lns_solve2p_dev(int32_t np, int32_t nsys, int32_t nblk, const double* mat, double* rhs, void* work,
                    void* stream) {
  int rc = check_tri(np, nsys, nblk, true, "solve2p");
  return rc ? rc : tri_dev(2, true, np, nsys, mat, rhs, nullptr, work, (cudaStream_t)stream, nullptr);
}
int lns_solve1p_dev(int32_t nsys, int32_t np, int32_t nblk, const double* mat, double* rhs, void* work,
                    void* stream) {
  int rc = check_tri(np, nsys, nblk, true, "solve1p");
  return rc ? rc : tri_dev(1, true, np, nsys, mat, rhs, nullptr, work, (cudaStream_t)stream, nullptr);
}

}  // extern "C"
