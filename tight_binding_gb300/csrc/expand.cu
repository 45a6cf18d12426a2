// expand.cu — Chebyshev expansions applied to a block of vectors.
//
//   out = sum_{n < n_terms} c_n T_n(H~) |k_r>,   r = 0 .. R-1, c_n complex
//
// The reference walks T_n(H~)|k> with Cheb_first_kind_seq_view
// (TB/numerical.h:346-361) and accumulates c_n T_n(H~)|k> on the host, e.g. the
// single-energy delta projection of conductivity_test_sawtooth
// (TB/snippets.h:173-223, c_n = a_d(n) T_n(e), n = 0 .. N).  Here the sum is
// formed by Clenshaw's recurrence (Clenshaw, Math. Comp. 9, 1955) run
// backwards over the coefficients on site-major work blocks:
//   b_N = 0,  b_{N-1} = c_{N-1} v,  b_k = 2 H~ b_{k+1} - b_{k+2} + c_k v,
//   out = (b_0 - b_2 + c_0 v) / 2,
// each b_k by one pass of the step kernel with the c_k v term fused into it
// (read v, x = b_{k+1}, b_{k+2}; write b_k in place), so no accumulator block
// is read and written per term.  The result is converted to complex128 and
// transposed back to Eigen's column-major layout once per chunk of vectors.
// Coefficient helpers: the delta projection above and the time-evolution
// operator exp(-i H t) (Jacobi-Anger expansion).
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

// out = c v (work precision)
template <typename F>
__global__ void scale_block_kernel(int64_t cnt, const typename C2<F>::T* __restrict__ v, double cr, double ci,
                                   typename C2<F>::T* __restrict__ out) {
  const F r = F(cr), i = F(ci);
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += (int64_t)gridDim.x * blockDim.x) {
    const typename C2<F>::T a = v[q];
    typename C2<F>::T o;
    o.x = r * a.x - i * a.y;
    o.y = r * a.y + i * a.x;
    out[q] = o;
  }
}

// acc = (b0 - b2 + c0 v) / 2 in complex128
template <typename F>
__global__ void clenshaw_final_kernel(int64_t cnt, const typename C2<F>::T* __restrict__ b0,
                                      const typename C2<F>::T* __restrict__ b2, const typename C2<F>::T* __restrict__ v,
                                      double cr, double ci, double2* __restrict__ acc) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < cnt; q += (int64_t)gridDim.x * blockDim.x) {
    const double2 a = as_c128(b0[q]), b = as_c128(b2[q]), x = as_c128(v[q]);
    acc[q] = make_double2(0.5 * (a.x - b.x + (cr * x.x - ci * x.y)), 0.5 * (a.y - b.y + (cr * x.y + ci * x.x)));
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

int grid_for(int64_t cnt) { return (int)std::max<int64_t>(1, std::min<int64_t>((cnt + 255) / 256, 8 * sm_count())); }

int scale_any(int prec, int64_t cnt, const void* v, double2 c, void* out, cudaStream_t st) {
  const int g = grid_for(cnt);
  if (prec == TBK_PREC_FP64)
    scale_block_kernel<double><<<g, 256, 0, st>>>(cnt, static_cast<const double2*>(v), c.x, c.y, static_cast<double2*>(out));
  else if (prec == TBK_PREC_DD)
    scale_block_kernel<dd><<<g, 256, 0, st>>>(cnt, static_cast<const dd2*>(v), c.x, c.y, static_cast<dd2*>(out));
  else
    scale_block_kernel<float><<<g, 256, 0, st>>>(cnt, static_cast<const float2*>(v), c.x, c.y, static_cast<float2*>(out));
  TBK_CHECK_LAUNCH();
  return TBK_OK;
}

int final_any(int prec, int64_t cnt, const void* b0, const void* b2, const void* v, double2 c, double2* acc,
              cudaStream_t st) {
  const int g = grid_for(cnt);
  if (prec == TBK_PREC_FP64)
    clenshaw_final_kernel<double><<<g, 256, 0, st>>>(cnt, static_cast<const double2*>(b0), static_cast<const double2*>(b2),
                                                     static_cast<const double2*>(v), c.x, c.y, acc);
  else if (prec == TBK_PREC_DD)
    clenshaw_final_kernel<dd><<<g, 256, 0, st>>>(cnt, static_cast<const dd2*>(b0), static_cast<const dd2*>(b2),
                                                 static_cast<const dd2*>(v), c.x, c.y, acc);
  else
    clenshaw_final_kernel<float><<<g, 256, 0, st>>>(cnt, static_cast<const float2*>(b0), static_cast<const float2*>(b2),
                                                    static_cast<const float2*>(v), c.x, c.y, acc);
  TBK_CHECK_LAUNCH();
  return TBK_OK;
}

}  // namespace
}  // namespace tbk

using namespace tbk;

// Cheb_first_kind_seq_view (TB/numerical.h:346-361): the two newest blocks of
// each chunk of vectors stay on the device; next() hands out T_i v and
// advances one recursion step.
struct tbk_cheb_view_s {
  tbk_sparse_s* H = nullptr;
  int32_t n = 0, R = 0, Rc = 0, n_chunks = 0, prec = 0, i = 0;
  int grid = 1, n_tiles = 1;
  std::vector<DevBuf> cur, nxt;      // per chunk: T_i v, T_{i+1} v (site-major)
  DevBuf acc, dst, part;
};

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
  DevBuf src, dst, vk, ba, bb, bc, acc, part;
  TBK_TRY(src.alloc(sizeof(double2) * (size_t)n * R));
  TBK_TRY(dst.alloc(sizeof(double2) * (size_t)n * R));
  for (DevBuf* b : {&vk, &ba, &bb, &bc}) TBK_TRY(b->alloc(csz * cnt));
  TBK_TRY(acc.alloc(sizeof(double2) * cnt));
  TBK_TRY(part.alloc(sizeof(double) * 2 * grid));
  TBK_CUDA(cudaMemcpyAsync(src.p, kets, sizeof(double2) * (size_t)n * R, cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemsetAsync(vk.p, 0, vk.bytes, st));
  TBK_CUDA(cudaMemsetAsync(bc.p, 0, bc.bytes, st));                         // padding rows stay zero
  auto c_of = [&](int32_t k) { return make_double2(coef[2 * k], coef[2 * k + 1]); };
  for (int32_t r0 = 0; r0 < R; r0 += Rc) {
    TBK_TRY(load_block_any(prec, n, R, r0, Rc, src.as<double2>(), vk.p, st));
    // Clenshaw: x = b_{k+1}, p = b_{k+2}; b_k is written over p
    void* p = ba.p;
    void* x = bb.p;
    TBK_CUDA(cudaMemsetAsync(p, 0, ba.bytes, st));                         // b_N = 0
    TBK_TRY(scale_any(prec, cnt, vk.p, c_of(n_terms - 1), x, st));          // b_{N-1}
    KStore ks;
    ks.addv = vk.p;
    for (int32_t k = n_terms - 2; k >= 1; --k) {
      ks.addc[0] = coef[2 * k];
      ks.addc[1] = coef[2 * k + 1];
      TBK_TRY(step_ks(Ht, Rc, prec, x, p, p, false, part.as<double>(), grid, n_tiles, st, ks, 3));
      std::swap(x, p);                                                      // x = b_k, p = b_{k+1}
    }
    if (n_terms >= 2) {
      // b_0 out of place (b_2 stays for the final combination)
      ks.addc[0] = coef[0];
      ks.addc[1] = coef[1];
      TBK_TRY(step_ks(Ht, Rc, prec, x, bc.p, p, false, part.as<double>(), grid, n_tiles, st, ks, 3));
      TBK_TRY(final_any(prec, cnt, bc.p, p, vk.p, c_of(0), acc.as<double2>(), st));
    } else {
      // one term: out = c_0 v  (= (b_0 - b_2 + c_0 v)/2 with b_0 = c_0 v, b_2 = 0)
      TBK_TRY(final_any(prec, cnt, x, p, vk.p, c_of(0), acc.as<double2>(), st));
    }
    dim3 g((unsigned)((n + 31) / 32), (unsigned)((Rc + 31) / 32)), b(32, 8);
    unload_block_kernel<<<g, b, 0, st>>>(n, R, r0, std::min(Rc, R - r0), Rc, acc.as<double2>(), dst.as<double2>());
    TBK_CHECK_LAUNCH();
  }
  TBK_CUDA(cudaMemcpyAsync(out, dst.p, sizeof(double2) * (size_t)n * R, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  return TBK_OK;
}

int tbk_cheb_view_create(tbk_cheb_view* out, tbk_sparse Ht, int32_t R, const double* kets, int32_t precision) {
  if (!out || !Ht || !kets || R < 1) return fail(TBK_ERR_INVALID, "tbk_cheb_view_create: bad argument");
  *out = nullptr;
  if (Ht->rows != Ht->cols) return fail(TBK_ERR_INVALID, "tbk_cheb_view_create: matrix must be square");
  if (precision != TBK_PREC_FP64 && precision != TBK_PREC_MIXED && precision != TBK_PREC_DD)
    return fail(TBK_ERR_INVALID, "tbk_cheb_view_create: unknown precision %d", precision);
  cudaStream_t st = nullptr;
  auto* V = new tbk_cheb_view_s();
  V->H = Ht;
  V->n = Ht->rows;
  V->R = R;
  V->prec = precision;
  V->Rc = chunk_width(precision, R);
  V->n_chunks = (R + V->Rc - 1) / V->Rc;
  auto bail = [&](int rc) { delete V; return rc; };
  int rc = step_config(Ht, V->Rc, precision, &V->grid, &V->n_tiles, st);
  if (rc != TBK_OK) return bail(rc);
  const int64_t cnt = (int64_t)Ht->ell.n_slices * 32 * V->Rc;
  const size_t csz = precision == TBK_PREC_MIXED ? sizeof(float2) : precision == TBK_PREC_DD ? sizeof(dd2) : sizeof(double2);
  V->cur.resize(V->n_chunks);
  V->nxt.resize(V->n_chunks);
  DevBuf src;
  if ((rc = src.alloc(sizeof(double2) * (size_t)V->n * R)) != TBK_OK || (rc = V->acc.alloc(sizeof(double2) * cnt)) != TBK_OK ||
      (rc = V->dst.alloc(sizeof(double2) * (size_t)V->n * R)) != TBK_OK ||
      (rc = V->part.alloc(sizeof(double) * 2 * V->grid)) != TBK_OK)
    return bail(rc);
  if (cudaMemcpy(src.p, kets, sizeof(double2) * (size_t)V->n * R, cudaMemcpyHostToDevice) != cudaSuccess)
    return bail(fail(TBK_ERR_CUDA, "tbk_cheb_view_create: upload failed"));
  for (int32_t c = 0; c < V->n_chunks; ++c) {
    if ((rc = V->cur[c].alloc(csz * cnt)) != TBK_OK || (rc = V->nxt[c].alloc(csz * cnt)) != TBK_OK) return bail(rc);
    cudaMemsetAsync(V->cur[c].p, 0, V->cur[c].bytes, st);
    cudaMemsetAsync(V->nxt[c].p, 0, V->nxt[c].bytes, st);
    // v_0 = v, v_1 = x v (the view's constructor)
    if ((rc = load_block_any(precision, V->n, R, c * V->Rc, V->Rc, src.as<double2>(), V->cur[c].p, st)) != TBK_OK ||
        (rc = step_any(Ht, V->Rc, precision, V->cur[c].p, V->nxt[c].p, nullptr, true, V->part.as<double>(), V->grid,
                       V->n_tiles, st)) != TBK_OK)
      return bail(rc);
  }
  if (cudaStreamSynchronize(st) != cudaSuccess) return bail(fail(TBK_ERR_CUDA, "tbk_cheb_view_create: sync failed"));
  *out = V;
  return TBK_OK;
}

int tbk_cheb_view_next(tbk_cheb_view V, int32_t* index, double* block, void* stream) {
  if (!V) return fail(TBK_ERR_INVALID, "tbk_cheb_view_next: null view");
  cudaStream_t st = as_stream(stream);
  const int64_t cnt = (int64_t)V->H->ell.n_slices * 32 * V->Rc;
  for (int32_t c = 0; c < V->n_chunks; ++c) {
    if (block) {
      // T_i v of this chunk -> complex128 -> columns of the host block
      TBK_TRY(final_any(V->prec, cnt, V->cur[c].p, V->cur[c].p, V->cur[c].p, make_double2(2.0, 0.0),
                        V->acc.as<double2>(), st));                    // (a - a + 2 a) / 2 = a, exactly
      dim3 g((unsigned)((V->n + 31) / 32), (unsigned)((V->Rc + 31) / 32)), b(32, 8);
      unload_block_kernel<<<g, b, 0, st>>>(V->n, V->R, c * V->Rc, std::min(V->Rc, V->R - c * V->Rc), V->Rc,
                                           V->acc.as<double2>(), V->dst.as<double2>());
      TBK_CHECK_LAUNCH();
    }
    // T_{i+2} = 2 x T_{i+1} - T_i, written over T_i; then cur <-> nxt
    TBK_TRY(step_any(V->H, V->Rc, V->prec, V->nxt[c].p, V->cur[c].p, V->cur[c].p, false, V->part.as<double>(),
                     V->grid, V->n_tiles, st));
    std::swap(V->cur[c], V->nxt[c]);
  }
  if (block)
    TBK_CUDA(cudaMemcpyAsync(block, V->dst.p, sizeof(double2) * (size_t)V->n * V->R, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  if (index) *index = V->i;
  ++V->i;
  return TBK_OK;
}

void tbk_cheb_view_destroy(tbk_cheb_view V) {
  if (!V) return;
  cudaDeviceSynchronize();
  delete V;
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
