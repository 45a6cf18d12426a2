// kubo.cu — Kubo conductivities from double-Chebyshev moments.
//
//   aL_m = g_m AL T_m(H~) BL |r>,   aR_n = g_n AR T_n(H~) BR |r>
//   mu_mn = sum_{sites, r} conj(aL_m) aR_n                        (a GEMM L^H R)
// Bastin sigma_xy: AL = BL = 1, AR = v_x, BR = v_y        (TB/snippets.h:306-456)
// Greenwood sigma_xx: AL = BL = v_x, AR = BR = 1           (TB/snippets.h:225-304)
// generate_V_moments: as Greenwood with the Dirichlet kernel (TB/snippets.h:491-518)
//
// The stored blocks (Cheb_first_kind_seq_on_bases, TB/numerical.h:333-344) are
// complex64 in HBM in a K-tiled layout: element k of block m lives at
// ((k / 16) * M + m) * 16 + k % 16, so the 16-element K slab of any run of
// consecutive blocks is contiguous (one coalesced 128-byte row per block) for
// the mu GEMM.  They are produced by the fused recursion
// step of kpm.cu running in complex128 on a three-block ring (the outer operator
// AL/AR applied after each step), each stored value rounded to complex64 once.
// Random vectors are processed in chunks so that both sides fit the block
// budget; mu accumulates over chunks in FP64 on the device.  The Gamma
// contractions (FP64) and the Bastin integration follow TB/snippets.h:343-449.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "kpm_device.cuh"
#include "tbk_internal.h"

namespace tbk {

int mu_gemm_tc(const float2* L, const float2* Rb, int32_t M, int64_t K, double* mu_acc,
               cudaStream_t st);   // gemm_tc.cu (tensor cores, split TF32, K-tiled blocks)

namespace {

// ------------------------------------------------------------------ CUDA-core GEMM
// C[m][n] += sum_k conj(L[m][k]) R[n][k] for a K range per CTA (split-K), blocks
// in the K-tiled layout;
// FP32 products, FP32 sums over 32 terms promoted to FP64, FP64 partial tiles.
constexpr int kGT = 32;      // output tile (complex) per CTA side
constexpr int kGK = 32;      // K chunk staged in shared memory

__global__ void __launch_bounds__(256) mu_gemm_cc_kernel(const float2* __restrict__ L, const float2* __restrict__ Rb,
                                                         int32_t M, int64_t K, int64_t ld, int64_t ksplit,
                                                         double2* __restrict__ part) {
  __shared__ float2 Ls[kGT][kGK + 1], Rs[kGT][kGK + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int32_t m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  const int64_t k0 = (int64_t)blockIdx.z * ksplit;
  const int64_t k1 = min(K, k0 + ksplit);
  float ar[2][2] = {{0, 0}, {0, 0}}, ai[2][2] = {{0, 0}, {0, 0}};
  double dr[2][2] = {{0, 0}, {0, 0}}, di[2][2] = {{0, 0}, {0, 0}};
  for (int64_t kb = k0; kb < k1; kb += kGK) {
    for (int q = threadIdx.x; q < kGT * kGK; q += 256) {
      const int row = q / kGK, kk = q % kGK;
      const int64_t k = kb + kk;
      float2 z = make_float2(0.f, 0.f);
      Ls[row][kk] = (m0 + row < M && k < k1) ? L[((k >> 4) * M + (m0 + row)) * 16 + (k & 15)] : z;
      Rs[row][kk] = (n0 + row < M && k < k1) ? Rb[((k >> 4) * M + (n0 + row)) * 16 + (k & 15)] : z;
    }
    __syncthreads();
#pragma unroll 8
    for (int kk = 0; kk < kGK; ++kk) {
      const float2 a0 = Ls[ty * 2][kk], a1 = Ls[ty * 2 + 1][kk];
      const float2 b0 = Rs[tx * 2][kk], b1 = Rs[tx * 2 + 1][kk];
      const float2 a[2] = {a0, a1}, b[2] = {b0, b1};
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          // conj(a) * b
          ar[i][j] += a[i].x * b[j].x + a[i].y * b[j].y;
          ai[i][j] += a[i].x * b[j].y - a[i].y * b[j].x;
        }
    }
    __syncthreads();
    // FP32 sums cover one 32-term chunk only: long FP32 accumulations lose
    // accuracy where the sum is much smaller than its terms (mu_nm at large m, n)
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
      for (int j = 0; j < 2; ++j) { dr[i][j] += ar[i][j]; di[i][j] += ai[i][j]; ar[i][j] = 0; ai[i][j] = 0; }
  }
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      dr[i][j] += ar[i][j];
      di[i][j] += ai[i][j];
      const int32_t m = m0 + ty * 2 + i, n = n0 + tx * 2 + j;
      if (m < M && n < M) part[((int64_t)blockIdx.z * M + m) * M + n] = make_double2(dr[i][j], di[i][j]);
    }
}

__global__ void mu_split_reduce_kernel(const double2* __restrict__ part, int32_t M, int32_t nsplit,
                                       double2* __restrict__ acc) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)M * M) return;
  double r = 0.0, i = 0.0;
  for (int32_t s = 0; s < nsplit; ++s) { const double2 v = part[(int64_t)s * M * M + q]; r += v.x; i += v.y; }
  acc[q].x += r;
  acc[q].y += i;
}

// FP64 reference GEMM on complex128 K-tiled blocks: C[m][n] += sum_k
// conj(L[m][k]) R[n][k] with every product and sum in FP64 (split-K partials,
// reduced in a fixed order by mu_split_reduce_kernel).
constexpr int kGK64 = 16;
__global__ void __launch_bounds__(256) mu_gemm_f64_kernel(const double2* __restrict__ L,
                                                          const double2* __restrict__ Rb, int32_t M, int64_t K,
                                                          int64_t ksplit, double2* __restrict__ part) {
  __shared__ double2 Ls[kGT][kGK64 + 1], Rs[kGT][kGK64 + 1];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int32_t m0 = blockIdx.y * kGT, n0 = blockIdx.x * kGT;
  const int64_t k0 = (int64_t)blockIdx.z * ksplit;
  const int64_t k1 = min(K, k0 + ksplit);
  double dr[2][2] = {{0, 0}, {0, 0}}, di[2][2] = {{0, 0}, {0, 0}};
  for (int64_t kb = k0; kb < k1; kb += kGK64) {
    for (int q = threadIdx.x; q < kGT * kGK64; q += 256) {
      const int row = q / kGK64, kk = q % kGK64;
      const int64_t k = kb + kk;
      const double2 z = make_double2(0.0, 0.0);
      Ls[row][kk] = (m0 + row < M && k < k1) ? L[((k >> 4) * M + (m0 + row)) * 16 + (k & 15)] : z;
      Rs[row][kk] = (n0 + row < M && k < k1) ? Rb[((k >> 4) * M + (n0 + row)) * 16 + (k & 15)] : z;
    }
    __syncthreads();
#pragma unroll 4
    for (int kk = 0; kk < kGK64; ++kk) {
      const double2 a[2] = {Ls[ty * 2][kk], Ls[ty * 2 + 1][kk]};
      const double2 b[2] = {Rs[tx * 2][kk], Rs[tx * 2 + 1][kk]};
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
          dr[i][j] = fma(a[i].x, b[j].x, fma(a[i].y, b[j].y, dr[i][j]));
          di[i][j] = fma(a[i].x, b[j].y, fma(-a[i].y, b[j].x, di[i][j]));
        }
    }
    __syncthreads();
  }
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j) {
      const int32_t m = m0 + ty * 2 + i, n = n0 + tx * 2 + j;
      if (m < M && n < M) part[((int64_t)blockIdx.z * M + m) * M + n] = make_double2(dr[i][j], di[i][j]);
    }
}

// work block -> block m of a complex128 K-tiled store (the FP64 reference form)
__device__ __forceinline__ double2 to_c128(double2 v) { return v; }
__device__ __forceinline__ double2 to_c128(float2 v) { return make_double2(v.x, v.y); }
__device__ __forceinline__ double2 to_c128(dd2 v) {
  return make_double2((double)v.x.hi + (double)v.x.lo, (double)v.y.hi + (double)v.y.lo);
}
template <typename CT>
__global__ void store_block64_kernel(const CT* __restrict__ src, double2* __restrict__ store, int32_t m, int32_t M,
                                     int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    store[((q >> 4) * M + m) * 16 + (q & 15)] = to_c128(src[q]);
}

// work block -> block m of the complex64 K-tiled store (complex128 work blocks
// are rounded once per element); 16 consecutive k form one contiguous 128-byte
// row of the tile
__device__ __forceinline__ float2 to_c64(double2 v) { return make_float2(__double2float_rn(v.x), __double2float_rn(v.y)); }
__device__ __forceinline__ float2 to_c64(float2 v) { return v; }
__device__ __forceinline__ float2 to_c64(dd2 v) { return make_float2(__fadd_rn(v.x.hi, v.x.lo), __fadd_rn(v.y.hi, v.y.lo)); }
template <typename CT>
__global__ void round_block_kernel(const CT* __restrict__ src, float2* __restrict__ store, int32_t m, int32_t M,
                                   int64_t n) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x)
    store[((q >> 4) * M + m) * 16 + (q & 15)] = to_c64(src[q]);
}

// columns [c0, c0 + Rc) of a 2 Rc-wide site-major block <- an Rc-wide block
template <typename CT>
__global__ void pack_cols_kernel(int64_t n_pad, int32_t Rc, int32_t c0, const CT* __restrict__ src,
                                 CT* __restrict__ dst) {
  const int64_t tot = n_pad * Rc;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = q / Rc;
    dst[row * 2 * Rc + c0 + (q - row * Rc)] = src[q];
  }
}
// block m of a K-tiled store (k = row * Rc + column) <- columns [c0, c0 + Rc)
// of a 2 Rc-wide block, rounded to complex64
template <typename CT>
__global__ void round_cols_kernel(int64_t n_pad, int32_t Rc, int32_t c0, const CT* __restrict__ src,
                                  float2* __restrict__ store, int32_t m, int32_t M) {
  const int64_t tot = n_pad * Rc;
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < tot; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t row = q / Rc;
    store[((q >> 4) * M + m) * 16 + (q & 15)] = to_c64(src[row * 2 * Rc + c0 + (q - row * Rc)]);
  }
}

__global__ void mu_kernel_scale_kernel(double2* __restrict__ mu, const double* __restrict__ g, int32_t M) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)M * M) return;
  const double s = g[q / M] * g[q % M];
  mu[q].x *= s;
  mu[q].y *= s;
}

// ------------------------------------------------------------------ Gamma contractions (FP64)
// zeta(e) = sum_mn mu_mn a_m a_n [(e - i n s) e^{i n th} T_m + (e + i m s) e^{-i m th} T_n] / (1-e^2)^2 / vol
//         = sum_m a_m T_m (sum_n mu_mn P_n) + sum_m P'_m (sum_n mu_mn a_n T_n),
//   P_n = a_n (e - i n s) e^{i n th},   P'_m = a_m (e + i m s) e^{-i m th}.
__global__ void bastin_zeta_kernel(const double2* __restrict__ mu, int32_t M, const double* __restrict__ eps,
                                   double vol, double2* __restrict__ zeta) {
  extern __shared__ double2 sm[];
  double2* P = sm;          // P_n
  double2* Q = sm + M;      // a_n T_n (real, stored as complex)
  const double e = eps[blockIdx.x];
  const double s = sqrt(1.0 - e * e), th = acos(e);
  for (int n = threadIdx.x; n < M; n += blockDim.x) {
    double sn, cn;
    sincos(n * th, &sn, &cn);
    const double an = n == 0 ? 1.0 : 2.0;
    // (e - i n s)(cn + i sn)
    P[n] = make_double2(an * (e * cn + n * s * sn), an * (e * sn - n * s * cn));
    Q[n] = make_double2(an * cn, 0.0);
  }
  __syncthreads();
  double zr = 0.0, zi = 0.0;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    double sm_, cm;
    sincos(m * th, &sm_, &cm);
    const double am = m == 0 ? 1.0 : 2.0;
    double r1 = 0.0, i1 = 0.0, r2 = 0.0, i2 = 0.0;
    const double2* row = mu + (int64_t)m * M;
    for (int n = 0; n < M; ++n) {
      const double2 u = row[n];
      r1 += u.x * P[n].x - u.y * P[n].y;
      i1 += u.x * P[n].y + u.y * P[n].x;
      r2 += u.x * Q[n].x;
      i2 += u.y * Q[n].x;
    }
    const double qm = am * cm;                                    // a_m T_m
    const double pr = am * (e * cm + m * s * sm_), pi = am * (-e * sm_ + m * s * cm);   // (e + i m s)(cm - i sm)
    zr += qm * r1 + (pr * r2 - pi * i2);
    zi += qm * i1 + (pr * i2 + pi * r2);
  }
  __shared__ double red[2][32];
  for (int o = 16; o > 0; o >>= 1) { zr += __shfl_xor_sync(0xffffffffu, zr, o); zi += __shfl_xor_sync(0xffffffffu, zi, o); }
  if ((threadIdx.x & 31) == 0) { red[0][threadIdx.x >> 5] = zr; red[1][threadIdx.x >> 5] = zi; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a += red[0][w]; b += red[1][w]; }
    const double den = (1.0 - e * e) * (1.0 - e * e) * vol;
    zeta[blockIdx.x] = make_double2(a / den, b / den);
  }
}

// sigma(e) = -sum_mn Re(mu_mn) a_m a_n T_m(e) T_n(e) / (1 - e^2) / R
__global__ void greenwood_kernel(const double2* __restrict__ mu, int32_t M, const double* __restrict__ eps, double R,
                                 double* __restrict__ sigma) {
  extern __shared__ double2 sm[];
  double* T = reinterpret_cast<double*>(sm);
  const double e = eps[blockIdx.x];
  const double th = acos(e);
  for (int n = threadIdx.x; n < M; n += blockDim.x) T[n] = (n == 0 ? 1.0 : 2.0) * cos(n * th);
  __syncthreads();
  double acc = 0.0;
  for (int m = threadIdx.x; m < M; m += blockDim.x) {
    double r = 0.0;
    const double2* row = mu + (int64_t)m * M;
    for (int n = 0; n < M; ++n) r += row[n].x * T[n];
    acc += T[m] * r;
  }
  __shared__ double red[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) a += red[w];
    sigma[blockIdx.x] = -a / (1.0 - e * e) / R;
  }
}



// timing of the last tbk_kubo_mu call (CUDA events on the caller's stream)
struct KuboTiming { double ms_blocks = 0, ms_gemm = 0, gemm_flops = 0, block_bytes = 0; int chunks = 0; };
KuboTiming g_kubo_timing;        // the last solve's timing (calls may come from several threads)
std::mutex g_kubo_timing_mu;

// TBK_TRACE=1: tbk_kubo_mu prints the host time of its phases to stderr
// (synchronising at each phase boundary, which it otherwise does not)
struct PhaseTrace {
  bool on;
  cudaStream_t st;
  std::chrono::steady_clock::time_point t0;
  std::vector<std::pair<const char*, double>> marks;
  explicit PhaseTrace(cudaStream_t s) : st(s), t0(std::chrono::steady_clock::now()) {
    const char* e = getenv("TBK_TRACE");
    on = e && atoi(e) != 0;
  }
  void mark(const char* name) {
    if (!on) return;
    cudaStreamSynchronize(st);
    marks.emplace_back(name, std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count());
  }
  ~PhaseTrace() {
    if (!on) return;
    double prev = 0.0;
    fprintf(stderr, "tbk_kubo_mu phases (ms):");
    for (auto& m : marks) {
      fprintf(stderr, " %s %.2f", m.first, m.second - prev);
      prev = m.second;
    }
    fprintf(stderr, "\n");
  }
};

// The stored blocks and work blocks of a call made outside a server come
// from a stream-ordered pool that keeps up to kKuboPoolKeep bytes between
// calls: stores of that size are then reused instead of mapped and unmapped
// every call (the 256 x 256, M = 512, R = 16 Bastin case: 8.6 GB, whose
// cudaFree took 5.7 ms of a 36 ms call).
// Larger stores keep plain allocations (a 137 GB store from the pool, then
// trimmed, measured 0.2 s slower than cudaMalloc and cudaFree); each call
// trims the pool back to kKuboPoolKeep before it returns.
constexpr uint64_t kKuboPoolKeep = 16ull << 30;
cudaMemPool_t kubo_pool() {
  static std::mutex mu;
  static cudaMemPool_t pools[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) { cudaGetLastError(); return nullptr; }
  std::lock_guard<std::mutex> lk(mu);
  if (!pools[dev]) {
    cudaMemPoolProps pp = {};
    pp.allocType = cudaMemAllocationTypePinned;
    pp.location.type = cudaMemLocationTypeDevice;
    pp.location.id = dev;
    if (cudaMemPoolCreate(&pools[dev], &pp) != cudaSuccess) {
      cudaGetLastError();
      pools[dev] = nullptr;
      return nullptr;
    }
    uint64_t keep = kKuboPoolKeep;
    cudaMemPoolSetAttribute(pools[dev], cudaMemPoolAttrReleaseThreshold, &keep);
  }
  return pools[dev];
}

int pick_chunk(int R) {
  int c = 1;
  while (c < R && c < 32) c <<= 1;
  return c;
}

}  // namespace
}  // namespace tbk

using namespace tbk;

extern "C" {

int tbk_kubo_mu(tbk_sparse Ht, tbk_sparse AL, tbk_sparse BL, tbk_sparse AR, tbk_sparse BR, int32_t M, int32_t R,
                uint64_t seed, const double* kets, int32_t kernel_kind, double kp0, double kp1, int32_t flags,
                double block_budget_gb, double* mu_out, void* stream) {
  if (!Ht || !mu_out) return fail(TBK_ERR_INVALID, "tbk_kubo_mu: null argument");
  if (M < 1 || R < 1) return fail(TBK_ERR_INVALID, "tbk_kubo_mu: M and R must be >= 1");
  if (Ht->rows != Ht->cols) return fail(TBK_ERR_INVALID, "tbk_kubo_mu: H must be square");
  tbk_sparse ops[4] = {AL, BL, AR, BR};
  for (auto* o : ops)
    if (o && (o->rows != Ht->rows || o->cols != Ht->cols)) return fail(TBK_ERR_INVALID, "tbk_kubo_mu: operator size mismatch");
  cudaStream_t st = as_stream(stream);
  PhaseTrace trace(st);
  // outside a server (which sets its own pool): stores and work blocks that
  // the pool keeps come from kubo_pool (decided below, once their size is known)
  AsyncAllocCtx kctx{};
  const int32_t n = Ht->rows;
  TBK_TRY(ensure_ell(Ht, st));
  for (auto* o : ops) if (o) TBK_TRY(ensure_ell(o, st));
  trace.mark("ell");
  const int64_t n_pad = (int64_t)Ht->ell.n_slices * 32;
  // chunk of random vectors: both stored sides within the budget
  int Rc = pick_chunk(R);
  // default budget: 60% of the free device memory (more vectors per chunk stream
  // the matrix fewer times)
  double budget = block_budget_gb * 1e9;
  if (block_budget_gb <= 0) {
    size_t fr = 0, tot = 0;
    TBK_CUDA(cudaMemGetInfo(&fr, &tot));
    budget = 0.6 * (double)fr;
  }
  const bool f64b = (flags & TBK_MU_FP64_BLOCKS) != 0;   // FP64 reference form: complex128 blocks, FP64 GEMM
  const double sel = f64b ? 16.0 : 8.0;                   // bytes per stored element
  while (Rc > 1 && 2.0 * M * n_pad * Rc * sel > budget) Rc >>= 1;
  if (2.0 * M * n_pad * Rc * sel > budget)
    return fail(TBK_ERR_BUDGET, "stored Chebyshev blocks need %.1f GB > budget %.1f GB", 2.0 * M * n_pad * sel / 1e9,
                budget / 1e9);
  const int64_t blk = n_pad * Rc;                       // complex entries per block
  // stored blocks: complex64.  Recursion and operator applications: complex128
  // work blocks by default (the Chebyshev recursion accumulates rounding error
  // near the band edges, where the Kubo weights 1/(1-e^2)^2 are largest; each
  // stored value is rounded to complex64 exactly once); TBK_MU_MIXED_RECURSION
  // runs them in complex64 with FP32 H~ (HBM-bound instead of FP64-pipe-bound).
  const int prec = (flags & TBK_MU_MIXED_RECURSION) ? TBK_PREC_MIXED
                   : (flags & TBK_MU_DD_RECURSION)  ? TBK_PREC_DD
                                                    : TBK_PREC_FP64;
  const size_t csz = prec == TBK_PREC_MIXED ? sizeof(float2) : sizeof(double2);
  DevBuf Ls, Rs, work, partd, part, macc, gdev, kstage;
  const int64_t blk16 = (blk + 15) / 16 * 16;           // K padded to whole 16-element tiles (zeros)
  if (!tl_async_alloc && 2.0 * sel * blk16 * M + 12.0 * csz * blk <= (double)kKuboPoolKeep) {
    kctx.pool = kubo_pool();
    kctx.stream = st;
  }
  {
    const AsyncAllocCtx* outer = tl_async_alloc;
    if (kctx.pool) tl_async_alloc = &kctx;
    const int a = Ls.alloc((size_t)sel * blk16 * M), b = a == TBK_OK ? Rs.alloc((size_t)sel * blk16 * M) : a;
    tl_async_alloc = outer;
    TBK_TRY(b);
  }
  // both sides as one recursion of width 2 Rc (TBK_MU_BOTH_SIDES) when every
  // output operator can be fused into the step (the gathers move twice the
  // bytes per row; the stored values are the same bits)
  bool both = !f64b && (flags & TBK_MU_BOTH_SIDES) && (flags & TBK_MU_FUSED_OPS) &&
              2 * Rc <= (prec == TBK_PREC_MIXED ? 64 : 32) && (prec != TBK_PREC_MIXED || Rc >= 2);
  for (tbk_sparse_s* o : {AL, AR}) {
    if (!both || !o) continue;
    bool same = false;
    TBK_TRY(same_ell_structure(Ht, o, &same, st));
    both = same;
  }
  {
    const AsyncAllocCtx* outer = tl_async_alloc;
    if (kctx.pool) tl_async_alloc = &kctx;
    const int a = work.alloc(csz * blk * (both ? 12 : 6));
    tl_async_alloc = outer;
    TBK_TRY(a);
  }
  {
    // the stores write every k < n Rc of every block; the entries of padded
    // rows (n <= row < n_pad) and of the K tail up to whole 16-element tiles
    // must read as zero.  In the K-tiled layout, element ((k/16) M + m) 16 +
    // k%16, they all lie in the K tiles from floor(n Rc / 16) on: one
    // contiguous region (the stores overwrite its written part afterwards)
    const int64_t kt0 = (int64_t)n * Rc / 16, kt1 = blk16 / 16;
    const size_t tile = (size_t)sel * 16 * M;           // bytes of one K tile of all M blocks
    if (kt1 > kt0) {
      TBK_CUDA(cudaMemsetAsync(Ls.as<char>() + kt0 * tile, 0, (size_t)(kt1 - kt0) * tile, st));
      TBK_CUDA(cudaMemsetAsync(Rs.as<char>() + kt0 * tile, 0, (size_t)(kt1 - kt0) * tile, st));
    }
  }
  TBK_CUDA(cudaMemsetAsync(work.p, 0, work.bytes, st));
  TBK_TRY(macc.alloc(sizeof(double2) * (size_t)M * M));
  TBK_CUDA(cudaMemsetAsync(macc.p, 0, macc.bytes, st));
  if (kets) {
    TBK_TRY(kstage.alloc(sizeof(double2) * (size_t)n * R));
    TBK_CUDA(cudaMemcpyAsync(kstage.p, kets, sizeof(double2) * (size_t)n * R, cudaMemcpyHostToDevice, st));
  }
  int grid = 1, n_tiles = 1;
  TBK_TRY(step_config(Ht, Rc, prec, &grid, &n_tiles, st));
  int gmax = grid;
  for (auto* o : ops)
    if (o) { int g2, t2; TBK_TRY(step_config(o, Rc, prec, &g2, &t2, st)); gmax = std::max(gmax, g2); }
  int grid2 = 1, tiles2 = 1;
  if (both) {
    TBK_TRY(step_config(Ht, 2 * Rc, prec, &grid2, &tiles2, st));
    gmax = std::max(gmax, grid2);
    if (prec == TBK_PREC_DD)
      for (tbk_sparse_s* o : {AL, AR}) if (o) TBK_TRY(ensure_ell_dd(o, st));
  }
  TBK_TRY(partd.alloc(sizeof(double) * 2 * gmax));
  trace.mark("alloc+classes");
  char* wb = work.as<char>();
  auto wblk = [&](int i) { return static_cast<void*>(wb + (size_t)i * blk * csz); };
  void* v0 = wblk(5);
  // algorithmic DRAM bytes of the block phase: vector blocks read / written,
  // matrix (ELL columns + values + diagonal) per pass, complex64 stores
  double rec_bytes = 0.0;
  const double vecb = (double)blk * csz, stb = (double)blk * 8.0;
  const int vsz = prec == TBK_PREC_MIXED ? 4 : 8;
  // class form (row classes): the row's class byte and diagonal; the table is in shared memory
  auto ell_bytes = [&](tbk_sparse_s* A, bool cols) {
    const double hv = (double)vsz * (A->ell.cplx ? 2 : 1);
    if (cols && A->ell.cls_state == 1) return (double)A->rows * (1.0 + hv);
    return (double)A->ell.n_entries * ((cols ? 4.0 : 0.0) + hv) + (double)A->rows * hv;
  };
  auto apply = [&](tbk_sparse_s* A, const void* x, void* y) -> int {   // y = A x
    rec_bytes += 2 * vecb + ell_bytes(A, true);
    int g, t;
    TBK_TRY(step_config(A, Rc, prec, &g, &t, st));
    return step_any(A, Rc, prec, x, y, nullptr, true, partd.as<double>(), g, t, st, nullptr, 0, 0, true, nullptr,
                    false);
  };
  auto round_to = [&](const void* src, float2* store, int32_t m) -> int {
    rec_bytes += vecb + stb;
    const unsigned g = (unsigned)std::min<int64_t>((blk + 255) / 256, 65535);
    if (prec == TBK_PREC_FP64) round_block_kernel<double2><<<g, 256, 0, st>>>(static_cast<const double2*>(src), store, m, M, blk);
    else if (prec == TBK_PREC_DD) round_block_kernel<dd2><<<g, 256, 0, st>>>(static_cast<const dd2*>(src), store, m, M, blk);
    else round_block_kernel<float2><<<g, 256, 0, st>>>(static_cast<const float2*>(src), store, m, M, blk);
    TBK_CHECK_LAUNCH();
    return TBK_OK;
  };
  // FP64 reference form: block m of the complex128 store from a work block
  auto store64 = [&](const void* src, void* store, int32_t m) -> int {
    rec_bytes += vecb + 2 * stb;
    const unsigned g = (unsigned)std::min<int64_t>((blk + 255) / 256, 65535);
    double2* d = static_cast<double2*>(store);
    if (prec == TBK_PREC_FP64) store_block64_kernel<double2><<<g, 256, 0, st>>>(static_cast<const double2*>(src), d, m, M, blk);
    else if (prec == TBK_PREC_DD) store_block64_kernel<dd2><<<g, 256, 0, st>>>(static_cast<const dd2*>(src), d, m, M, blk);
    else store_block64_kernel<float2><<<g, 256, 0, st>>>(static_cast<const float2*>(src), d, m, M, blk);
    TBK_CHECK_LAUNCH();
    return TBK_OK;
  };
  // block m of `store` = A x, written by the product itself (no work block)
  auto apply_to_store = [&](tbk_sparse_s* A, const void* x, void* scratch, float2* store, int32_t m) -> int {
    rec_bytes += vecb + ell_bytes(A, true) + stb;
    int g, t;
    TBK_TRY(step_config(A, Rc, prec, &g, &t, st));
    return step_any(A, Rc, prec, x, scratch, nullptr, true, partd.as<double>(), g, t, st, store, M, m, false);
  };
  // one side: store[m] = Aout T_m(H~) (Bin v0), m < M; each step writes its
  // complex64 block (Aout absent) or feeds the product that does
  // TBK_MU_FUSED_OPS: with an output operator that shares H~'s ELL structure
  // (a commutator [X, H~] does), step m also forms Aout T_{m-1} from the x it
  // gathers and writes block m-1: one pass over the matrix and the vectors per
  // block instead of two.  The stored values are the same bits either way.
  auto side = [&](tbk_sparse_s* Aout, tbk_sparse_s* Bin, float2* store) -> int {
    void* r[3] = {wblk(0), wblk(1), wblk(2)};
    void* tmpA = wblk(3);
    if (f64b) {                                           // recursion, operator, complex128 store
      if (Bin) TBK_TRY(apply(Bin, v0, r[0]));
      else TBK_CUDA(cudaMemcpyAsync(r[0], v0, csz * blk, cudaMemcpyDeviceToDevice, st));
      for (int32_t m = 0; m < M; ++m) {
        void* y = r[m % 3];
        if (m >= 1) {
          rec_bytes += (m >= 2 ? 3 : 2) * vecb + ell_bytes(Ht, true);
          TBK_TRY(step_any(Ht, Rc, prec, r[(m - 1) % 3], y, m >= 2 ? r[(m - 2) % 3] : nullptr, m == 1,
                           partd.as<double>(), grid, n_tiles, st, nullptr, 0, 0, true, nullptr, false));
        }
        if (Aout) {
          TBK_TRY(apply(Aout, y, tmpA));
          TBK_TRY(store64(tmpA, store, m));
        } else {
          TBK_TRY(store64(y, store, m));
        }
      }
      return TBK_OK;
    }
    bool fuse = false;
    if (Aout && (flags & TBK_MU_FUSED_OPS)) {
      TBK_TRY(same_ell_structure(Ht, Aout, &fuse, st));
      if (fuse && prec == TBK_PREC_DD) TBK_TRY(ensure_ell_dd(Aout, st));
    }
    if (Bin) TBK_TRY(apply(Bin, v0, r[0]));
    else TBK_CUDA(cudaMemcpyAsync(r[0], v0, csz * blk, cudaMemcpyDeviceToDevice, st));
    for (int32_t m = 0; m < M; ++m) {
      void* y = r[m % 3];
      if (m >= 1) {
        const void* x = r[(m - 1) % 3];
        const void* pv = m >= 2 ? r[(m - 2) % 3] : nullptr;
        rec_bytes += (m >= 2 ? 3 : 2) * vecb + ell_bytes(Ht, true) + ((fuse || !Aout) ? stb : 0.0) +
                     (fuse ? ell_bytes(Aout, false) : 0.0);
        if (fuse)
          TBK_TRY(step_any(Ht, Rc, prec, x, y, pv, m == 1, partd.as<double>(), grid, n_tiles, st, store, M, m - 1,
                           true, Aout));
        else
          TBK_TRY(step_any(Ht, Rc, prec, x, y, pv, m == 1, partd.as<double>(), grid, n_tiles, st,
                           Aout ? nullptr : store, M, m, true, nullptr, false));
      }
      if (Aout && !fuse) TBK_TRY(apply_to_store(Aout, y, tmpA, store, m));
      else if (!Aout && m == 0) TBK_TRY(round_to(y, store, 0));
    }
    if (fuse) TBK_TRY(apply_to_store(Aout, r[(M - 1) % 3], tmpA, store, M - 1));
    return TBK_OK;
  };
  // both sides at once: columns [0, Rc) carry the left side (BL v0), [Rc, 2 Rc)
  // the right side (BR v0); step m stores T_m of a side without an output
  // operator as block m and A T_{m-1} of a side with one as block m-1
  auto both_sides = [&]() -> int {
    const size_t b2 = csz * blk * 2;
    char* base = wb + csz * blk * 6;                     // three 2 Rc-wide blocks after the six Rc-wide ones
    void* r[3] = {base, base + b2, base + 2 * b2};
    void* half[2] = {wblk(0), wblk(1)};
    tbk_sparse_s* Bin[2] = {BL, BR};
    tbk_sparse_s* Aout[2] = {AL, AR};
    float2* stores[2] = {Ls.as<float2>(), Rs.as<float2>()};
    const unsigned gp = (unsigned)std::min<int64_t>((blk + 255) / 256, 65535);
    for (int h = 0; h < 2; ++h) {
      if (Bin[h]) TBK_TRY(apply(Bin[h], v0, half[h]));
      else TBK_CUDA(cudaMemcpyAsync(half[h], v0, csz * blk, cudaMemcpyDeviceToDevice, st));
      if (prec == TBK_PREC_FP64)
        pack_cols_kernel<double2><<<gp, 256, 0, st>>>(n_pad, Rc, h * Rc, static_cast<const double2*>(half[h]),
                                                      static_cast<double2*>(r[0]));
      else if (prec == TBK_PREC_DD)
        pack_cols_kernel<dd2><<<gp, 256, 0, st>>>(n_pad, Rc, h * Rc, static_cast<const dd2*>(half[h]),
                                                  static_cast<dd2*>(r[0]));
      else
        pack_cols_kernel<float2><<<gp, 256, 0, st>>>(n_pad, Rc, h * Rc, static_cast<const float2*>(half[h]),
                                                     static_cast<float2*>(r[0]));
      TBK_CHECK_LAUNCH();
      if (!Aout[h]) {
        if (prec == TBK_PREC_FP64)
          round_cols_kernel<double2><<<gp, 256, 0, st>>>(n_pad, Rc, h * Rc, static_cast<const double2*>(r[0]),
                                                         stores[h], 0, M);
        else if (prec == TBK_PREC_DD)
          round_cols_kernel<dd2><<<gp, 256, 0, st>>>(n_pad, Rc, h * Rc, static_cast<const dd2*>(r[0]), stores[h], 0, M);
        else
          round_cols_kernel<float2><<<gp, 256, 0, st>>>(n_pad, Rc, h * Rc, static_cast<const float2*>(r[0]),
                                                        stores[h], 0, M);
        TBK_CHECK_LAUNCH();
      }
    }
    KStore ks;
    ks.halves = 2;
    ks.kM = M;
    for (int h = 0; h < 2; ++h) {
      ks.store[h] = stores[h];
      ks.usev[h] = Aout[h] ? 1 : 0;
      ks.vval[h] = Aout[h] ? ell_vals(Aout[h]->ell, prec) : nullptr;
      ks.vdiag[h] = Aout[h] ? ell_diag(Aout[h]->ell, prec) : nullptr;
    }
    rec_bytes += 2 * (vecb + 2 * vecb);                  // start halves packed into the wide block
    for (int h = 0; h < 2; ++h) rec_bytes += Aout[h] ? 0.0 : 2 * vecb + stb;
    for (int32_t m = 1; m < M; ++m) {
      rec_bytes += 2 * (m >= 2 ? 3 : 2) * vecb + ell_bytes(Ht, true) + 2 * stb;
      for (int h = 0; h < 2; ++h) rec_bytes += Aout[h] ? ell_bytes(Aout[h], false) : 0.0;
      for (int h = 0; h < 2; ++h) ks.km[h] = Aout[h] ? m - 1 : m;
      TBK_TRY(step_ks(Ht, 2 * Rc, prec, r[(m - 1) % 3], r[m % 3], m >= 2 ? r[(m - 2) % 3] : nullptr, m == 1,
                      partd.as<double>(), grid2, tiles2, st, ks));
    }
    if (AL || AR) {                                      // A T_{M-1} -> block M-1 (the new vector is not kept)
      for (int h = 0; h < 2; ++h) ks.km[h] = Aout[h] ? M - 1 : -1;
      TBK_TRY(step_ks(Ht, 2 * Rc, prec, r[(M - 1) % 3], r[M % 3], M >= 2 ? r[(M - 2) % 3] : nullptr, M == 1,
                      partd.as<double>(), grid2, tiles2, st, ks));
    }
    return TBK_OK;
  };
  const bool use_tc = !f64b && (flags & TBK_MU_TENSOR) != 0;
  // split-K: at least 16,384 K values per CTA, at most 64 partial M x M blocks
  const int64_t ksplit = std::max<int64_t>(16384, (blk + 63) / 64);
  const int32_t nsplit = (int32_t)((blk + ksplit - 1) / ksplit);
  if (!use_tc) TBK_TRY(part.alloc(sizeof(double2) * (size_t)nsplit * M * M));
  cudaEvent_t ev[3];
  for (auto& e : ev) TBK_CUDA(cudaEventCreate(&e));
  KuboTiming tm;
  for (int32_t r0 = 0; r0 < R; r0 += Rc) {
    TBK_CUDA(cudaEventRecord(ev[0], st));
    if (kets) TBK_TRY(load_block_any(prec, n, R, r0, Rc, kstage.as<double2>(), v0, st));
    else TBK_TRY(random_block_any(prec, n, R, r0, Rc, seed, v0, st));
    if (both) {
      TBK_TRY(both_sides());
    } else {
      TBK_TRY(side(AL, BL, Ls.as<float2>()));
      TBK_TRY(side(AR, BR, Rs.as<float2>()));
    }
    TBK_CUDA(cudaEventRecord(ev[1], st));
    trace.mark("blocks");
    if (f64b) {
      dim3 g((M + kGT - 1) / kGT, (M + kGT - 1) / kGT, nsplit);
      mu_gemm_f64_kernel<<<g, 256, 0, st>>>(Ls.as<double2>(), Rs.as<double2>(), M, blk, ksplit, part.as<double2>());
      TBK_CHECK_LAUNCH();
      mu_split_reduce_kernel<<<(unsigned)(((int64_t)M * M + 255) / 256), 256, 0, st>>>(part.as<double2>(), M, nsplit,
                                                                                       macc.as<double2>());
      TBK_CHECK_LAUNCH();
    } else if (use_tc) {
      TBK_TRY(mu_gemm_tc(Ls.as<float2>(), Rs.as<float2>(), M, blk, macc.as<double>(), st));
    } else {
      dim3 g((M + kGT - 1) / kGT, (M + kGT - 1) / kGT, nsplit);
      mu_gemm_cc_kernel<<<g, 256, 0, st>>>(Ls.as<float2>(), Rs.as<float2>(), M, blk, blk, ksplit, part.as<double2>());
      TBK_CHECK_LAUNCH();
      mu_split_reduce_kernel<<<(unsigned)(((int64_t)M * M + 255) / 256), 256, 0, st>>>(part.as<double2>(), M, nsplit,
                                                                                       macc.as<double2>());
      TBK_CHECK_LAUNCH();
    }
    TBK_CUDA(cudaEventRecord(ev[2], st));
    TBK_CUDA(cudaEventSynchronize(ev[2]));
    trace.mark("gemm");
    float a = 0.f, b = 0.f;
    TBK_CUDA(cudaEventElapsedTime(&a, ev[0], ev[1]));
    TBK_CUDA(cudaEventElapsedTime(&b, ev[1], ev[2]));
    tm.ms_blocks += a;
    tm.ms_gemm += b;
    tm.gemm_flops += 8.0 * M * (double)M * (double)blk * (use_tc ? 3.0 : 1.0);   // real flops of the products issued
    tm.block_bytes += rec_bytes;
    rec_bytes = 0.0;
    tm.chunks += 1;
  }
  for (auto& e : ev) cudaEventDestroy(e);
  {
    std::lock_guard<std::mutex> lk(g_kubo_timing_mu);
    g_kubo_timing = tm;
  }
  // kernel factors g_m g_n (FP64)
  std::vector<double> g(M);
  TBK_TRY(tbk_kernel_seq(kernel_kind, M, kp0, kp1, g.data()));
  TBK_TRY(gdev.alloc(sizeof(double) * M));
  TBK_CUDA(cudaMemcpyAsync(gdev.p, g.data(), sizeof(double) * M, cudaMemcpyHostToDevice, st));
  mu_kernel_scale_kernel<<<(unsigned)(((int64_t)M * M + 255) / 256), 256, 0, st>>>(macc.as<double2>(), gdev.as<double>(), M);
  TBK_CHECK_LAUNCH();
  TBK_CUDA(cudaMemcpyAsync(mu_out, macc.p, sizeof(double2) * (size_t)M * M, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  trace.mark("scale+readback");
  Ls.release();
  Rs.release();
  work.release();
  if (kctx.pool) {
    TBK_CUDA(cudaStreamSynchronize(st));
    TBK_CUDA(cudaMemPoolTrimTo(kctx.pool, kKuboPoolKeep));   // keep at most kKuboPoolKeep bytes
  }
  trace.mark("free");
  return TBK_OK;
}

int tbk_mu_from_blocks(int32_t M, int64_t K, const double* L, const double* Rb, int32_t flags, double* mu_out,
                       void* stream) {
  if (M < 1 || K < 1 || !L || !Rb || !mu_out) return fail(TBK_ERR_INVALID, "tbk_mu_from_blocks: bad argument");
  cudaStream_t st = as_stream(stream);
  const int64_t K16 = (K + 15) / 16 * 16;
  DevBuf stage, Ld, Rd, acc, part;
  TBK_TRY(stage.alloc(sizeof(double2) * K));
  TBK_TRY(Ld.alloc(sizeof(float2) * M * K16));
  TBK_TRY(Rd.alloc(sizeof(float2) * M * K16));
  TBK_TRY(acc.alloc(sizeof(double2) * (size_t)M * M));
  TBK_CUDA(cudaMemsetAsync(Ld.p, 0, Ld.bytes, st));
  TBK_CUDA(cudaMemsetAsync(Rd.p, 0, Rd.bytes, st));
  TBK_CUDA(cudaMemsetAsync(acc.p, 0, acc.bytes, st));
  for (int side = 0; side < 2; ++side) {
    float2* dst = side ? Rd.as<float2>() : Ld.as<float2>();
    const double* src = side ? Rb : L;
    for (int32_t m = 0; m < M; ++m) {
      TBK_CUDA(cudaMemcpyAsync(stage.p, src + 2 * (int64_t)m * K, sizeof(double2) * K, cudaMemcpyHostToDevice, st));
      round_block_kernel<double2><<<(unsigned)std::min<int64_t>((K + 255) / 256, 4096), 256, 0, st>>>(stage.as<double2>(), dst, m,
                                                                                          M, K);
      TBK_CHECK_LAUNCH();
    }
  }
  cudaEvent_t ev[2];
  for (auto& e : ev) TBK_CUDA(cudaEventCreate(&e));
  TBK_CUDA(cudaEventRecord(ev[0], st));
  if (flags & TBK_MU_TENSOR) {
    TBK_TRY(mu_gemm_tc(Ld.as<float2>(), Rd.as<float2>(), M, K, acc.as<double>(), st));
  } else {
    const int64_t ksplit = 16384;
    const int32_t nsplit = (int32_t)((K + ksplit - 1) / ksplit);
    TBK_TRY(part.alloc(sizeof(double2) * (size_t)nsplit * M * M));
    dim3 g((M + kGT - 1) / kGT, (M + kGT - 1) / kGT, nsplit);
    mu_gemm_cc_kernel<<<g, 256, 0, st>>>(Ld.as<float2>(), Rd.as<float2>(), M, K, 0, ksplit, part.as<double2>());
    TBK_CHECK_LAUNCH();
    mu_split_reduce_kernel<<<(unsigned)(((int64_t)M * M + 255) / 256), 256, 0, st>>>(part.as<double2>(), M, nsplit,
                                                                                     acc.as<double2>());
    TBK_CHECK_LAUNCH();
  }
  TBK_CUDA(cudaEventRecord(ev[1], st));
  TBK_CUDA(cudaMemcpyAsync(mu_out, acc.p, sizeof(double2) * (size_t)M * M, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, ev[0], ev[1]);
  for (auto& e : ev) cudaEventDestroy(e);
  KuboTiming tm;
  tm.ms_gemm = ms;
  tm.gemm_flops = 8.0 * M * (double)M * (double)K * ((flags & TBK_MU_TENSOR) ? 3.0 : 1.0);
  tm.block_bytes = 2.0 * M * (double)K * 8.0;
  tm.chunks = 1;
  {
    std::lock_guard<std::mutex> lk(g_kubo_timing_mu);
    g_kubo_timing = tm;
  }
  return TBK_OK;
}

int tbk_kubo_release(void) {
  cudaMemPool_t pl = kubo_pool();
  if (!pl) return TBK_OK;
  TBK_CUDA(cudaDeviceSynchronize());
  TBK_CUDA(cudaMemPoolTrimTo(pl, 0));
  return TBK_OK;
}

int tbk_kubo_last_timing(double* ms_blocks, double* ms_gemm, double* gemm_flops, double* block_bytes, int32_t* chunks) {
  KuboTiming t;
  {
    std::lock_guard<std::mutex> lk(g_kubo_timing_mu);
    t = g_kubo_timing;
  }
  if (ms_blocks) *ms_blocks = t.ms_blocks;
  if (ms_gemm) *ms_gemm = t.ms_gemm;
  if (gemm_flops) *gemm_flops = t.gemm_flops;
  if (block_bytes) *block_bytes = t.block_bytes;
  if (chunks) *chunks = t.chunks;
  return TBK_OK;
}

int tbk_kubo_bastin_zeta(int32_t M, const double* mu, int32_t n_eps, const double* eps, double vol, double* zeta_out,
                         void* stream) {
  if (M < 1 || !mu || n_eps < 0 || (n_eps && (!eps || !zeta_out))) return fail(TBK_ERR_INVALID, "tbk_kubo_bastin_zeta: bad argument");
  if (n_eps == 0) return TBK_OK;
  cudaStream_t st = as_stream(stream);
  DevBuf dm, de, dz;
  TBK_TRY(dm.alloc(sizeof(double2) * (size_t)M * M));
  TBK_TRY(de.alloc(sizeof(double) * n_eps));
  TBK_TRY(dz.alloc(sizeof(double2) * n_eps));
  TBK_CUDA(cudaMemcpyAsync(dm.p, mu, sizeof(double2) * (size_t)M * M, cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemcpyAsync(de.p, eps, sizeof(double) * n_eps, cudaMemcpyHostToDevice, st));
  const size_t smem = sizeof(double2) * 2 * M;
  if (smem > 48 * 1024) TBK_CUDA(cudaFuncSetAttribute(bastin_zeta_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  bastin_zeta_kernel<<<n_eps, 256, smem, st>>>(dm.as<double2>(), M, de.as<double>(), vol, dz.as<double2>());
  TBK_CHECK_LAUNCH();
  TBK_CUDA(cudaMemcpyAsync(zeta_out, dz.p, sizeof(double2) * n_eps, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  return TBK_OK;
}

int tbk_kubo_greenwood_sigma(int32_t M, const double* mu, int32_t n_eps, const double* eps, double R,
                             double* sigma_out, void* stream) {
  if (M < 1 || !mu || n_eps < 0 || (n_eps && (!eps || !sigma_out)) || !(R > 0))
    return fail(TBK_ERR_INVALID, "tbk_kubo_greenwood_sigma: bad argument");
  if (n_eps == 0) return TBK_OK;
  cudaStream_t st = as_stream(stream);
  DevBuf dm, de, ds;
  TBK_TRY(dm.alloc(sizeof(double2) * (size_t)M * M));
  TBK_TRY(de.alloc(sizeof(double) * n_eps));
  TBK_TRY(ds.alloc(sizeof(double) * n_eps));
  TBK_CUDA(cudaMemcpyAsync(dm.p, mu, sizeof(double2) * (size_t)M * M, cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemcpyAsync(de.p, eps, sizeof(double) * n_eps, cudaMemcpyHostToDevice, st));
  greenwood_kernel<<<n_eps, 256, sizeof(double2) * M, st>>>(dm.as<double2>(), M, de.as<double>(), R, ds.as<double>());
  TBK_CHECK_LAUNCH();
  TBK_CUDA(cudaMemcpyAsync(sigma_out, ds.p, sizeof(double) * n_eps, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  return TBK_OK;
}

// Bastin: drop N/24 nodes at each end, ascending order, cumulative trapezoid from
// E = 0 outward with the half-cell weights of TB/snippets.h:421-449 (host, O(N)).
int tbk_kubo_bastin_integrate(int32_t N, const double* eps, const double* zeta, double* E_out, double* re_out,
                              double* im_out, int32_t* n_out) {
  if (N < 4 || !eps || !zeta || !E_out || !re_out || !im_out || !n_out)
    return fail(TBK_ERR_INVALID, "tbk_kubo_bastin_integrate: bad argument");
  const int32_t cut = N / 24;
  const int32_t n = N - 2 * cut;
  std::vector<double> E(n), zr(n), zi(n);
  for (int32_t k = 0; k < n; ++k) {     // drop(cut) | take(N - 2 cut) | reverse
    const int32_t src = cut + (n - 1 - k);
    E[k] = eps[src];
    zr[k] = zeta[2 * src];
    zi[k] = zeta[2 * src + 1];
  }
  const int32_t e0 = (int32_t)(std::upper_bound(E.begin(), E.end(), 0.0) - E.begin());
  if (e0 < 1 || e0 >= n) return fail(TBK_ERR_INVALID, "bastin integration: E = 0 not inside the node range");
  std::vector<double> ri(n, 0.0), ii(n, 0.0);
  ri[e0] = (zr[e0] * 3 / 4 + zr[e0 - 1] / 4) * (E[e0] - E[e0 - 1]) / 2;
  ri[e0 - 1] = -(zr[e0] / 4 + zr[e0 - 1] * 3 / 4) * (E[e0] - E[e0 - 1]) / 2;
  for (int32_t i = e0 + 1; i < n; ++i) {
    ri[i] = ri[i - 1] + (zr[i] + zr[i - 1]) / 2 * (E[i] - E[i - 1]);
    ii[i] = ii[i - 1] + (zi[i] + zi[i - 1]) / 2 * (E[i] - E[i - 1]);
  }
  for (int32_t i = e0 - 2; i >= 0; --i) {
    ri[i] = ri[i + 1] - (zr[i] + zr[i + 1]) / 2 * (E[i + 1] - E[i]);
    ii[i] = ii[i + 1] - (zi[i] + zi[i + 1]) / 2 * (E[i + 1] - E[i]);
  }
  for (int32_t k = 0; k < n; ++k) { E_out[k] = E[k]; re_out[k] = ri[k]; im_out[k] = ii[k]; }
  *n_out = n;
  return TBK_OK;
}

}  // extern "C"
