// The linearised two-dimensional implicit ADI step (src/impdrv.f90 with
// linear = 1): src/lrhs.f90 for the RHS about the frozen operators of the
// mean flow (genmtrx(vm, 0, vm), src/lns3d.f90:149), rbe/rtb, rhsBC,
// resstat, lhs1f/lhs2f with their boundary rows, the pentadiagonal solves
// (penta2p or penta2bc, penta1p or penta1bc), v += r and itrBC.
//
// With the spanwise wavenumber and the frequency zero these are the
// routines of the single-mode step (src/lrhs3d.f90, src/lhs1f3d.f90, ...)
// applied to real fields: the 3D terms (Dhi, ABhi) vanish and complex
// arithmetic on fields with zero imaginary parts is real arithmetic.  So a
// 2D linear context owns a single-mode context at kz = omega = 0 and a
// complex copy of the state; real fields enter and leave through two
// conversion kernels.  (The reference factors the real LHS again every
// corrector; its factors do not change for a linear run, and the
// single-mode context factors them once.)
#include <cuda_runtime.h>

#include <string>

#include "../../include/lns3d_gb300.h"
#include "adi3d.cuh"

int lns_fail(int code, const std::string& msg);
int lns_cuda_fail(cudaError_t e, const char* where);
int lns_ctx3d_create_planes(const lns_params3d* p, lns_ctx3d** out, bool lin2d_planes);
int lns_ctx3d_set_nbl(lns_ctx3d* c, int nbl);

struct lns_lin2d {
  lns_ctx3d* ctx = nullptr;
  int nx = 0, ny = 0;
  lns::cd* vc = nullptr;      // complex state (5,nx,ny)
  double* vr = nullptr;       // real staging of the host-pointer forms
  double* res = nullptr;      // residual history of the host-pointer forms
  int res_cap = 0;
  size_t bytes = 0;
};

namespace {

__global__ void to_complex_kernel(long long n, const double* __restrict__ v, lns::cd* __restrict__ w) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e < n) w[e] = lns::cd{v[e], 0.0};
}
__global__ void to_real_kernel(long long n, const lns::cd* __restrict__ w, double* __restrict__ v) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e < n) v[e] = w[e].x;
}

int convert(lns_lin2d* c, double* v, bool to_complex, cudaStream_t st) {
  const long long n = 5LL * c->nx * c->ny;
  const unsigned blocks = (unsigned)((n + 255) / 256);
  if (to_complex) to_complex_kernel<<<blocks, 256, 0, st>>>(n, v, c->vc);
  else to_real_kernel<<<blocks, 256, 0, st>>>(n, c->vc, v);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? LNS_OK : lns_cuda_fail(e, "lin2d conversion launch");
}

int dmalloc(lns_lin2d* c, size_t bytes, void** p) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return lns_fail(LNS_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  }
  c->bytes += bytes;
  return LNS_OK;
}

}  // namespace

extern "C" {

int lns_lin2d_create(const lns_params3d* p, lns_lin2d** out) {
  if (!p || !out) return lns_fail(LNS_ERR_ARG, "lin2d_create: null argument");
  *out = nullptr;
  if (p->beta != 0.0 || p->omega != 0.0)
    return lns_fail(LNS_ERR_ARG, "lin2d_create: a 2D linear run has beta = 0 and omega = 0 (Lz = 0 in the deck)");
  if (p->precision != LNS_FP64) return lns_fail(LNS_ERR_ARG, "lin2d_create: precision must be LNS_FP64");
  // a non-periodic xi direction: the zero-disturbance planes (left 0, right 0:
  // v = 0, r = 0 and identity rows in both LHS, src/itrbc.f90:310-316,534-540,
  // src/rhsbc.f90:189-191,238-240, src/lhsbc1f.f90:108-115,183-190,
  // src/lhsbc2f.f90:124-131,164-171) are the single-mode step's; the
  // symmetry plane (left 7) is the single-mode step's left 7 with v = 0 and
  // r = 0 for the second velocity component on the plane, the single-mode
  // context's plane lns::a3::kLinSymLeft; the nonreflecting planes (left 1,
  // right 1) are its planes kLinNrLeft and kLinNrRight.  The linear 2D
  // branches' other planes (left 2-6, right 3) are not built: left 2
  // extrapolates column 1 from columns 2-5 after their wall rows are set, left
  // 3 and right 3 (Giles) and left 4 are time-dependent characteristic
  // inflows, and left 5 keeps the interior LHS row.
  if (p->xper != 1 && !(p->xper == 0 && (p->left == 0 || p->left == 1 || p->left == 7) &&
                        (p->right == 0 || p->right == 1)))
    return lns_fail(LNS_ERR_ARG,
                    "lin2d_create: the linear 2D step needs xper = 1, or xper = 0 with left 0, 1 or 7 and right 0 or 1");
  lns_lin2d* c = new lns_lin2d();
  lns_params3d q3 = *p;
  if (!p->xper && p->left == 7) q3.left = lns::a3::kLinSymLeft;
  if (!p->xper && p->left == 1) q3.left = lns::a3::kLinNrLeft;
  if (!p->xper && p->right == 1) q3.right = lns::a3::kLinNrRight;
  int rc = lns_ctx3d_create_planes(&q3, &c->ctx, true);
  c->nx = p->nx;
  c->ny = p->ny;
  void* q = nullptr;
  const size_t n = 5 * (size_t)p->nx * p->ny;
  if (!rc) rc = dmalloc(c, sizeof(lns::cd) * n, &q), c->vc = (lns::cd*)q;
  if (!rc) rc = dmalloc(c, sizeof(double) * n, &q), c->vr = (double*)q;
  if (rc) {
    lns_lin2d_destroy(c);
    return rc;
  }
  *out = c;
  return LNS_OK;
}

int lns_lin2d_destroy(lns_lin2d* c) {
  if (!c) return LNS_OK;
  if (c->ctx) lns_ctx3d_destroy(c->ctx);
  cudaFree(c->vc);
  cudaFree(c->vr);
  cudaFree(c->res);
  delete c;
  return LNS_OK;
}

size_t lns_lin2d_bytes(const lns_lin2d* c) { return c ? c->bytes + lns_ctx3d_bytes(c->ctx) : 0; }

int lns_lin2d_set_nbl(lns_lin2d* c, int32_t nbl) {
  if (!c) return lns_fail(LNS_ERR_ARG, "lin2d_set_nbl: null context");
  return lns_ctx3d_set_nbl(c->ctx, nbl);
}

int lns_upload_metrics_lin2d(lns_lin2d* c, const double* metrics) {
  if (!c) return lns_fail(LNS_ERR_ARG, "upload_metrics_lin2d: null context");
  return lns_upload_metrics3d(c->ctx, metrics);
}

int lns_upload_mean_lin2d(lns_lin2d* c, const double* vm, double* cfl) {
  if (!c) return lns_fail(LNS_ERR_ARG, "upload_mean_lin2d: null context");
  return lns_upload_mean3d(c->ctx, vm, cfl);
}

int lns_get_dtl_lin2d(lns_lin2d* c, double* dtl) {
  if (!c || !dtl) return lns_fail(LNS_ERR_ARG, "get_dtl_lin2d: null argument");
  return lns_get_field3d(c->ctx, 8, dtl);
}

int lns_itrbc_lin2d_dev(lns_lin2d* c, double* v, void* stream) {
  if (!c || !v) return lns_fail(LNS_ERR_ARG, "itrbc_lin2d: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = convert(c, v, true, st);
  if (!rc) rc = lns_itrbc3d_dev(c->ctx, (double*)c->vc, stream);
  if (!rc) rc = convert(c, v, false, st);
  return rc;
}

int lns_step_lin2d_dev(lns_lin2d* c, double* v, int32_t nsteps, int32_t niter, double* totres_dev, void* stream) {
  if (!c || !v) return lns_fail(LNS_ERR_ARG, "step_lin2d: null argument");
  cudaStream_t st = (cudaStream_t)stream;
  int rc = convert(c, v, true, st);
  if (!rc) rc = lns_step3d_dev(c->ctx, (double*)c->vc, nsteps, niter, totres_dev, stream);
  if (!rc) rc = convert(c, v, false, st);
  return rc;
}

int lns_step_lin2d(lns_lin2d* c, double* v, int32_t nsteps, int32_t niter, double* totres) {
  if (!c || !v) return lns_fail(LNS_ERR_ARG, "step_lin2d: null argument");
  if (nsteps < 0) return lns_fail(LNS_ERR_ARG, "step_lin2d: nsteps must be >= 0");
  const size_t bytes = sizeof(double) * 5 * (size_t)c->nx * c->ny;
  if (nsteps > c->res_cap) {
    cudaFree(c->res);
    c->res = nullptr;
    c->res_cap = 0;
    void* q = nullptr;
    if (int rc = dmalloc(c, sizeof(double) * nsteps, &q)) return rc;
    c->res = (double*)q;
    c->res_cap = nsteps;
  }
  cudaError_t e = cudaMemcpy(c->vr, v, bytes, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return lns_cuda_fail(e, "step_lin2d: copy v in");
  int rc = lns_step_lin2d_dev(c, c->vr, nsteps, niter, c->res, nullptr);
  if (rc) return rc;
  e = cudaMemcpy(v, c->vr, bytes, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && totres && nsteps > 0)
    e = cudaMemcpy(totres, c->res, sizeof(double) * nsteps, cudaMemcpyDeviceToHost);
  return e == cudaSuccess ? LNS_OK : lns_cuda_fail(e, "step_lin2d: copy v out");
}

}  // extern "C"
