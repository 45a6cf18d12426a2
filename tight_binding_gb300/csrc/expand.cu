// expand.cu — Chebyshev expansions applied to a block of vectors.
//
//   out = sum_{n < n_terms} c_n T_n(H~) |k_r>,   r = 0 .. R-1, c_n complex
//
// The reference walks T_n(H~)|k> with Cheb_first_kind_seq_view
// (TB/numerical.h:346-361) and accumulates c_n T_n(H~)|k> on the host, e.g. the
// single-energy delta projection of conductivity_test_sawtooth
// (TB/snippets.h:173-223, c_n = a_d(n) T_n(e), n = 0 .. N).  Here the three-term
// recursion runs with the one-pass step kernel on site-major work blocks (any
// precision), and every step adds c_n T_n|k> into a complex128 accumulator in
// the same layout; the accumulator is transposed back to Eigen's column-major
// layout once per chunk of vectors.  Coefficient helpers: the delta projection
// above and the time-evolution operator exp(-i H t) (Jacobi-Anger expansion).
#include <algorithm>
#include <cmath>
#include <complex>
#include <vector>

#include "kpm_device.cuh"
#include "tbk_internal.h"

namespace tbk {
namespace {

__device__ __forceinline__ double2 as_c128(float2 v) { return make_double2((double)v.x, (double)v.y); }
__device__ __forceinline__ double2 as_c128(double2 v) { return v; }
__device__ __forceinline__ double2 as_c128(dd2 v) { return make_double2((double)v.x, (double)v.y); }

// acc (+)= c * v over cnt site-major elements
template <typename F>
__global__ void expand_axpy_kernel(int64_t cnt, const typename C2<F>::T* __restrict__ v, double cr, double ci,
                                   double2* __restrict__ acc, int init) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 x = as_c128(v[i]);
    double2 a = init ? make_double2(0.0, 0.0) : acc[i];
    a.x = fma(cr, x.x, fma(-ci, x.y, a.x));
    a.y = fma(cr, x.y, fma(ci, x.x, a.y));
    acc[i] = a;
  }
}

// site-major accumulator (n_pad x Rp) -> columns r0 .. r0+rc-1 of the
// column-major n x R output
__global__ void unload_block_kernel(int32_t n, int32_t R, int32_t r0, int32_t rc, int32_t Rp,
                                    const double2* __restrict__ acc, double2* __restrict__ dst) {
  __shared__ double2 tile[32][33];
  const int32_t i0 = blockIdx.x * 32, c0 = blockIdx.y * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {         // read along vectors of one site
    const int32_t i = i0 + k, c = c0 + threadIdx.x;
    tile[threadIdx.x][k] = (i < n && c < Rp) ? acc[(int64_t)i * Rp + c] : make_double2(0.0, 0.0);
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {         // write along sites of one vector
    const int32_t c = c0 + k, i = i0 + threadIdx.x;
    if (c < rc && i < n && r0 + c < R) dst[(int64_t)(r0 + c) * n + i] = tile[k][threadIdx.x];
  }
}

int chunk_width(int prec, int32_t R) {
  const int cap = prec == TBK_PREC_MIXED ? 32 : 16;
  int w = 1;
  while (w < R && w < cap) w <<= 1;
  return w;
}

template <typename F>
int axpy(int64_t cnt, const void* v, double2 c, double2* acc, bool init, cudaStream_t st) {
  const int g = (int)std::max<int64_t>(1, std::min<int64_t>((cnt + 255) / 256, 8 * sm_count()));
  expand_axpy_kernel<F><<<g, 256, 0, st>>>(cnt, static_cast<const typename C2<F>::T*>(v), c.x, c.y, acc, init ? 1 : 0);
  TBK_CHECK_LAUNCH();
  return TBK_OK;
}

int axpy_any(int prec, int64_t cnt, const void* v, double2 c, double2* acc, bool init, cudaStream_t st) {
  if (prec == TBK_PREC_FP64) return axpy<double>(cnt, v, c, acc, init, st);
  if (prec == TBK_PREC_DD) return axpy<dd>(cnt, v, c, acc, init, st);
  return axpy<float>(cnt, v, c, acc, init, st);
}

}  // namespace
}  // namespace tbk

using namespace tbk;

extern "C" {

int tbk_cheb_expand(tbk_sparse Ht, int32_t n_terms, const double* coef, int32_t R, const double* kets, double* out,
                    int32_t precision, void* stream) {
  if (!Ht || !coef || !kets || !out) return fail(TBK_ERR_INVALID, "tbk_cheb_expand: null argument");
  if (n_terms < 1 || R < 1) return fail(TBK_ERR_INVALID, "tbk_cheb_expand: n_terms and R must be >= 1");
  if (Ht->rows != Ht->cols) return fail(TBK_ERR_INVALID, "tbk_cheb_expand: matrix must be square");
  const int prec = precision;
  if (prec != TBK_PREC_FP64 && prec != TBK_PREC_MIXED && prec != TBK_PREC_DD)
    return fail(TBK_ERR_INVALID, "tbk_cheb_expand: unknown precision %d", prec);
  cudaStream_t st = as_stream(stream);
  const int32_t n = Ht->rows;
  const int Rc = chunk_width(prec, R);
  int grid = 1, n_tiles = 1;
  TBK_TRY(step_config(Ht, Rc, prec, &grid, &n_tiles, st));
  const int64_t n_pad = (int64_t)Ht->ell.n_slices * 32;
  const size_t csz = prec == TBK_PREC_MIXED ? sizeof(float2) : prec == TBK_PREC_DD ? sizeof(dd2) : sizeof(double2);
  const int64_t cnt = n_pad * Rc;
  DevBuf src, dst, va, vb, acc, part;
  TBK_TRY(src.alloc(sizeof(double2) * (size_t)n * R));
  TBK_TRY(dst.alloc(sizeof(double2) * (size_t)n * R));
  TBK_TRY(va.alloc(csz * cnt));
  TBK_TRY(vb.alloc(csz * cnt));
  TBK_TRY(acc.alloc(sizeof(double2) * cnt));
  TBK_TRY(part.alloc(sizeof(double) * 2 * grid));
  TBK_CUDA(cudaMemcpyAsync(src.p, kets, sizeof(double2) * (size_t)n * R, cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemsetAsync(va.p, 0, va.bytes, st));
  TBK_CUDA(cudaMemsetAsync(vb.p, 0, vb.bytes, st));
  auto c_of = [&](int32_t k) { return make_double2(coef[2 * k], coef[2 * k + 1]); };
  for (int32_t r0 = 0; r0 < R; r0 += Rc) {
    void* v_prev = va.p;     // T_{k-1}|k>
    void* v_cur = vb.p;      // T_k|k>
    TBK_TRY(load_block_any(prec, n, R, r0, Rc, src.as<double2>(), v_prev, st));
    TBK_TRY(axpy_any(prec, cnt, v_prev, c_of(0), acc.as<double2>(), true, st));
    if (n_terms > 1) {
      TBK_TRY(step_any(Ht, Rc, prec, v_prev, v_cur, nullptr, true, part.as<double>(), grid, n_tiles, st));
      TBK_TRY(axpy_any(prec, cnt, v_cur, c_of(1), acc.as<double2>(), false, st));
    }
    for (int32_t k = 2; k < n_terms; ++k) {
      // T_k = 2 H~ T_{k-1} - T_{k-2}, written over T_{k-2}
      TBK_TRY(step_any(Ht, Rc, prec, v_cur, v_prev, v_prev, false, part.as<double>(), grid, n_tiles, st));
      std::swap(v_prev, v_cur);
      TBK_TRY(axpy_any(prec, cnt, v_cur, c_of(k), acc.as<double2>(), false, st));
    }
    dim3 g((unsigned)((n + 31) / 32), (unsigned)((Rc + 31) / 32)), b(32, 8);
    unload_block_kernel<<<g, b, 0, st>>>(n, R, r0, std::min(Rc, R - r0), Rc, acc.as<double2>(), dst.as<double2>());
    TBK_CHECK_LAUNCH();
  }
  TBK_CUDA(cudaMemcpyAsync(out, dst.p, sizeof(double2) * (size_t)n * R, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  return TBK_OK;
}

int tbk_cheb_coef_delta(double e, int32_t N, double* coef) {
  if (!coef || N < 0) return fail(TBK_ERR_INVALID, "tbk_cheb_coef_delta: bad argument");
  // Cheb_first_kind_seq_view(e, 1.): T_0 = 1, T_1 = e, T_{k+1} = 2 e T_k - T_{k-1};
  // weight a_d(k) = 1 for k = 0, else 2 (TB/snippets.h:175, 197-202)
  double t0 = 1.0, t1 = e;
  for (int32_t k = 0; k <= N; ++k) {
    coef[2 * k] = (k == 0 ? 1.0 : 2.0) * t0;
    coef[2 * k + 1] = 0.0;
    const double t2 = 2.0 * e * t1 - t0;
    t0 = t1;
    t1 = t2;
  }
  return TBK_OK;
}

int tbk_cheb_coef_evolution(double a, double b, double t, int32_t n_terms, double* coef) {
  if (!coef || n_terms < 1) return fail(TBK_ERR_INVALID, "tbk_cheb_coef_evolution: bad argument");
  // exp(-i H t) with H = a H~ + b:  exp(-i b t) sum_k (2 - delta_k0) (-i)^k J_k(a t) T_k(H~)
  const double z = a * t;
  const std::complex<double> ph = std::exp(std::complex<double>(0.0, -b * t));
  const std::complex<double> mi(0.0, -1.0);
  std::complex<double> p(1.0, 0.0);    // (-i)^k
  for (int32_t k = 0; k < n_terms; ++k) {
    const double j = z >= 0 ? std::cyl_bessel_j((double)k, z) : ((k & 1) ? -1.0 : 1.0) * std::cyl_bessel_j((double)k, -z);
    const std::complex<double> c = ph * p * ((k == 0 ? 1.0 : 2.0) * j);
    coef[2 * k] = c.real();
    coef[2 * k + 1] = c.imag();
    p *= mi;
  }
  return TBK_OK;
}

int tbk_cheb_evolution_terms(double a, double t, double tol, int32_t* n_terms) {
  if (!n_terms || !(tol > 0)) return fail(TBK_ERR_INVALID, "tbk_cheb_evolution_terms: bad argument");
  const double z = std::fabs(a * t);
  // J_k(z) decays faster than (z/2)^k / k! once k > z: first k past z with two
  // consecutive terms below tol
  int32_t k = (int32_t)std::ceil(z) + 1;
  for (; k < (1 << 26); ++k)
    if (std::fabs(std::cyl_bessel_j((double)k, z)) < tol && std::fabs(std::cyl_bessel_j((double)k + 1, z)) < tol) break;
  if (k >= (1 << 26)) return fail(TBK_ERR_INVALID, "tbk_cheb_evolution_terms: |a t| too large");
  *n_terms = k + 1;
  return TBK_OK;
}

}  // extern "C"
