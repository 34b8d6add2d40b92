// Launch helpers of the line solvers, shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <string>
#include <type_traits>

#include "../../include/lns3d_gb300.h"
#include "mixed.cuh"
#include "penta_direct.cuh"
#include "penta_periodic.cuh"
#include "penta_solve.cuh"

// Error reporting of the C ABI (defined in capi.cu): the message of the last
// failure of the calling thread, returned by lns_last_error().
int lns_fail(int code, const std::string& msg);
int lns_cuda_fail(cudaError_t e, const char* where);
// Process-wide periodic-factorisation mode (lns_set_periodic_exact).
extern std::atomic<int> g_periodic_exact;

namespace lns {
namespace host {

// Solve phase (code 1): lines of kLpw per warp, see penta_solve.cuh.
template <typename T, bool PER>
int launch_solve(const void* mat, void* rhs, const void* per, const void* per2, int n, int nsys,
                 long long row_stride, long long line_stride, cudaStream_t st) {
  if (nsys == 0) return LNS_OK;
  const size_t smem = lns::solve_smem_bytes<T>(PER);
  // Set on every launch: the kernel template is instantiated in more than
  // one translation unit, each registering its own copy, so a once-only
  // flag could leave the copy that a launch resolves to without the limit.
  cudaError_t ea = cudaFuncSetAttribute(lns::penta_solve_kernel<T, PER>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (ea != cudaSuccess) return lns_cuda_fail(ea, "cudaFuncSetAttribute");
  lns::SolveArgs a{mat, rhs, per, per2, n, nsys, row_stride, line_stride, PER ? 1 : 0};
  const int lpw = lns::SolveCfg<T>::kLpw;
  lns::penta_solve_kernel<T, PER><<<(nsys + lpw - 1) / lpw, 32, smem, st>>>(a);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return lns_cuda_fail(e, "penta_solve_kernel launch");
  return LNS_OK;
}

// Threads per line of the factor kernels: a warp when the lines alone fill
// the GPU (several per SM sub-partition), else a CTA per line so that each
// pivot's elimination and Schur update spread over more sub-partitions.
// The periodic pivot touches about four times the elements of a boundary
// one; FP64 lines fill the FP64 pipes sooner than FP32 ones.  Results do
// not depend on the choice.
template <typename T>
inline int bc_team(int nsys) {
  return nsys <= (sizeof(typename lns::real_of<T>::type) == 8 ? 304 : 640) ? 128 : 32;
}
inline int p_team(int nsys) { return nsys <= 160 ? 256 : nsys <= 640 ? 128 : 32; }

template <typename T, int TEAM>
void launch_bc_team(const lns::PentaArgs& a, cudaStream_t st) {
  if constexpr (TEAM == 32) {
    const int blocks = (a.nsys + lns::kWarpsPerCta - 1) / lns::kWarpsPerCta;
    const size_t smem = (size_t)lns::kWarpsPerCta * (lns::kRing * lns::kRowSz + 16) * sizeof(T);
    lns::penta_bc_kernel<T, 32><<<blocks, 32 * lns::kWarpsPerCta, smem, st>>>(a);
  } else {
    const size_t smem = (size_t)(lns::kRing * lns::kRowSz + 16) * sizeof(T);
    lns::penta_bc_kernel<T, TEAM><<<a.nsys, TEAM, smem, st>>>(a);
  }
}

template <typename T, int TEAM>
void launch_p_team(const lns::PeriodicArgs& a, cudaStream_t st) {
  if constexpr (TEAM == 32) {
    const int blocks = (a.nsys + lns::kPWarpsPerCta - 1) / lns::kPWarpsPerCta;
    const size_t smem = (size_t)lns::kPWarpsPerCta * lns::kPWarpSmem * sizeof(T);
    lns::penta_p_kernel<T, 32><<<blocks, 32 * lns::kPWarpsPerCta, smem, st>>>(a);
  } else {
    const size_t smem = (size_t)lns::kPWarpSmem * sizeof(T);
    lns::penta_p_kernel<T, TEAM><<<a.nsys, TEAM, smem, st>>>(a);
  }
}

template <typename T>
void launch_p_any(const lns::PeriodicArgs& a, cudaStream_t st) {
  switch (p_team(a.nsys)) {
    case 256: launch_p_team<T, 256>(a, st); break;
    case 128: launch_p_team<T, 128>(a, st); break;
    default: launch_p_team<T, 32>(a, st); break;
  }
}

// code 0: factor; 1: solve; 2: factor then solve.
template <typename T>
int launch_bc(void* mat, void* rhs, int n, int nsys, long long row_stride, long long line_stride, int code,
              cudaStream_t st, int* status) {
  if (nsys == 0) return LNS_OK;
  // With CTA teams (few lines) the right-hand side is eliminated in the
  // factoring pass (code 2), which measured faster there than a separate
  // solve kernel, with identical results; warp teams factor, then solve.
  const bool cta_team = bc_team<T>(nsys) == 128;
  if (code != 1) {
    lns::PentaArgs a{mat, rhs, n, nsys, row_stride, line_stride, cta_team && code == 2 ? 2 : 0, status};
    if (cta_team) launch_bc_team<T, 128>(a, st);
    else launch_bc_team<T, 32>(a, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lns_cuda_fail(e, "penta_bc_kernel launch");
  }
  if (code == 1 || (code == 2 && !cta_team))
    return launch_solve<T, false>(mat, rhs, nullptr, nullptr, n, nsys, row_stride, line_stride, st);
  return LNS_OK;
}


template <typename T>
int launch_p(void* mat, void* rhs, void* per, void* per2, int np, int nsys, long long row_stride,
             long long line_stride, int code, cudaStream_t st, int* status, int exact = -1) {
  if (nsys == 0) return LNS_OK;
  const bool cplx = std::is_same<T, lns::cd>::value || std::is_same<T, lns::cf>::value;
  const int compat = exact < 0 ? (g_periodic_exact.load() ? 0 : 1) : (exact ? 0 : 1);
  if (!cplx) {
    // Real periodic solves are single pass: the reference's per2 is only a
    // (6,5,5,nsys) scratch window, too small to carry the fill of rows n-1,
    // n to a separate solve phase, so the right-hand side is eliminated
    // during the factorisation.
    lns::PeriodicArgs a{mat, rhs, per, per2, np - 1, np, nsys, row_stride, line_stride, 2, compat, 0, status};
    launch_p_any<T>(a, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lns_cuda_fail(e, "penta_p_kernel launch");
    return LNS_OK;
  }
  if (code != 1) {
    lns::PeriodicArgs a{mat, rhs, per, per2, np - 1, np, nsys, row_stride, line_stride, 0,
                        compat, 1, status};
    launch_p_any<T>(a, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return lns_cuda_fail(e, "penta_p_kernel launch");
  }
  if (code != 0) return launch_solve<T, true>(mat, rhs, per, per2, np - 1, nsys, row_stride, line_stride, st);
  return LNS_OK;
}


}  // namespace host
}  // namespace lns
