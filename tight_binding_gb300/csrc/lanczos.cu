// lanczos.cu — spectral range of a Hermitian sparse matrix on the device.
//
// The reference estimates (E_min, E_max) for GreenFunction(N, HE, ref_HE,
// epsilon) with a Spectra Lanczos eigensolver on the CPU and refuses matrices
// above 5,000 rows (TB/numerical.h:24-46, TB/lattice.h:560-566).  Here: k steps
// of the Hermitian Lanczos three-term recursion on the device (complex128, one
// vector, products by the one-pass step kernel, whose <x|Hx> partial is alpha),
// then the extreme eigenvalues of the k x k tridiagonal matrix by Sturm-sequence
// bisection on the host.  The residual norm beta_{k+1} |s_k| of each extreme
// Ritz pair is returned with it: an eigenvalue of the matrix lies within that
// distance of the Ritz value.
#include <cmath>
#include <vector>

#include "host_model.h"
#include "tbk_internal.h"

namespace tbk {
namespace {

// w -= alpha v + beta vp; per-block partial of |w|^2
__global__ void lanczos_update_kernel(int32_t n, double2* __restrict__ w, const double2* __restrict__ v,
                                      const double2* __restrict__ vp, double alpha, double beta,
                                      double* __restrict__ part) {
  double s = 0.0;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double2 a = w[i];
    const double2 b = v[i], c = vp[i];
    a.x = a.x - alpha * b.x - beta * c.x;
    a.y = a.y - alpha * b.y - beta * c.y;
    w[i] = a;
    s += a.x * a.x + a.y * a.y;
  }
  __shared__ double sh[256];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void lanczos_scale_kernel(int32_t n, double2* __restrict__ w, double s) {
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    w[i].x *= s;
    w[i].y *= s;
  }
}

// number of eigenvalues of the tridiagonal (a, b) below x (Sturm sequence)
int sturm_count(const std::vector<double>& a, const std::vector<double>& b, double x) {
  int c = 0;
  double q = 1.0;
  for (size_t i = 0; i < a.size(); ++i) {
    const double bb = i ? b[i - 1] * b[i - 1] : 0.0;
    q = a[i] - x - (i ? bb / q : 0.0);
    if (q == 0.0) q = 1e-300;
    if (q < 0) ++c;
  }
  return c;
}
// the k-th smallest eigenvalue (0-based) by bisection inside [lo, hi]
double tridiag_eig(const std::vector<double>& a, const std::vector<double>& b, int k, double lo, double hi) {
  for (int it = 0; it < 200 && hi - lo > 1e-15 * std::max(1.0, std::fabs(lo) + std::fabs(hi)); ++it) {
    const double mid = 0.5 * (lo + hi);
    if (sturm_count(a, b, mid) > k) hi = mid;
    else lo = mid;
  }
  return 0.5 * (lo + hi);
}
// last component of the unit eigenvector of the tridiagonal for eigenvalue th
// (forward recurrence of the characteristic polynomials, then normalised)
double last_component(const std::vector<double>& a, const std::vector<double>& b, double th) {
  const size_t k = a.size();
  std::vector<double> x(k);
  x[0] = 1.0;
  if (k > 1) x[1] = (th - a[0]) / b[0];
  for (size_t i = 2; i < k; ++i) {
    x[i] = ((th - a[i - 1]) * x[i - 1] - b[i - 2] * x[i - 2]) / b[i - 1];
    if (std::fabs(x[i]) > 1e150)              // keep the recurrence finite
      for (size_t q = 0; q <= i; ++q) x[q] *= 1e-150;
  }
  double nrm = 0.0, mx = 0.0;
  for (double v : x) mx = std::max(mx, std::fabs(v));
  if (!(mx > 0.0) || !std::isfinite(mx)) return 1.0;
  for (double v : x) nrm += (v / mx) * (v / mx);
  return std::fabs(x[k - 1] / mx) / std::sqrt(nrm);
}

}  // namespace
}  // namespace tbk

using namespace tbk;

extern "C" {

int tbk_spectral_range(tbk_sparse A, int32_t iters, uint64_t seed, double* e_min, double* e_max, double* res_min,
                       double* res_max, void* stream) {
  if (!A || !e_min || !e_max) return fail(TBK_ERR_INVALID, "tbk_spectral_range: null argument");
  if (A->rows != A->cols) return fail(TBK_ERR_INVALID, "tbk_spectral_range: matrix must be square");
  if (iters < 2) return fail(TBK_ERR_INVALID, "tbk_spectral_range: iters must be >= 2");
  cudaStream_t st = as_stream(stream);
  const int32_t n = A->rows;
  int grid = 1, n_tiles = 1;
  TBK_TRY(step_config(A, 1, TBK_PREC_FP64, &grid, &n_tiles, st));
  const int64_t n_pad = (int64_t)A->ell.n_slices * 32;
  DevBuf vb[3], part, upart;
  for (auto& b : vb) {
    TBK_TRY(b.alloc(sizeof(double2) * n_pad));
    TBK_CUDA(cudaMemsetAsync(b.p, 0, b.bytes, st));
  }
  TBK_TRY(part.alloc(sizeof(double) * 2 * grid));
  const int ub = 4 * sm_count();
  TBK_TRY(upart.alloc(sizeof(double) * ub));
  double2* v = vb[0].as<double2>();      // v_j
  double2* vp = vb[1].as<double2>();     // v_{j-1}
  double2* w = vb[2].as<double2>();
  // v_0: the seeded random phases (unit norm)
  TBK_TRY(random_block_any(TBK_PREC_FP64, n, 1, 0, 1, seed, v, st));
  std::vector<double> alpha, beta;       // T = tridiag(beta, alpha, beta)
  std::vector<double> hp(2 * grid), hu(ub);
  double bprev = 0.0;
  const int32_t k_max = std::min<int64_t>(iters, (int64_t)2 * n);
  for (int32_t j = 0; j < k_max; ++j) {
    // w = H v; alpha = <v|H v> from the step's FIRST partial
    TBK_TRY(step_any(A, 1, TBK_PREC_FP64, v, w, nullptr, true, part.as<double>(), grid, n_tiles, st));
    TBK_CUDA(cudaMemcpyAsync(hp.data(), part.p, sizeof(double) * 2 * grid, cudaMemcpyDeviceToHost, st));
    TBK_CUDA(cudaStreamSynchronize(st));
    double a = 0.0;
    for (int g = 0; g < grid; ++g) a += hp[grid + g];
    alpha.push_back(a);
    lanczos_update_kernel<<<ub, 256, 0, st>>>(n, w, v, vp, a, bprev, upart.as<double>());
    TBK_CHECK_LAUNCH();
    TBK_CUDA(cudaMemcpyAsync(hu.data(), upart.p, sizeof(double) * ub, cudaMemcpyDeviceToHost, st));
    TBK_CUDA(cudaStreamSynchronize(st));
    double s = 0.0;
    for (double x : hu) s += x;
    const double b = std::sqrt(s);
    if (j + 1 == k_max || !(b > 1e-13 * std::max(1.0, std::fabs(a)))) {   // invariant subspace or done
      bprev = b;
      break;
    }
    beta.push_back(b);
    lanczos_scale_kernel<<<ub, 256, 0, st>>>(n, w, 1.0 / b);
    TBK_CHECK_LAUNCH();
    double2* t = vp;
    vp = v;
    v = w;
    w = t;
    bprev = b;
  }
  // extreme Ritz values of T_k (Gershgorin interval for the bisection)
  double lo = 1e300, hi = -1e300;
  for (size_t i = 0; i < alpha.size(); ++i) {
    const double r = (i ? std::fabs(beta[i - 1]) : 0.0) + (i < beta.size() ? std::fabs(beta[i]) : 0.0);
    lo = std::min(lo, alpha[i] - r);
    hi = std::max(hi, alpha[i] + r);
  }
  const int k = (int)alpha.size();
  std::vector<double> bb(beta.begin(), beta.begin() + std::max(0, k - 1));
  const double tmin = tridiag_eig(alpha, bb, 0, lo, hi);
  const double tmax = tridiag_eig(alpha, bb, k - 1, lo, hi);
  *e_min = tmin;
  *e_max = tmax;
  if (res_min) *res_min = bprev * last_component(alpha, bb, tmin);
  if (res_max) *res_max = bprev * last_component(alpha, bb, tmax);
  return TBK_OK;
}

}  // extern "C"
