// noalloc.cu — Chebyshev moments without any device allocation.
//
// Who needs this: callers that are not allowed to allocate GPU memory while
// they run — code executing inside a fixed, pre-reserved HBM budget (a serving
// process whose admission controller has already handed out every byte),
// plug-in hosts that give an extension device buffers but forbid it from
// calling the allocator, and latency-critical loops where cudaMalloc/cudaFree
// would synchronise the device.  They pass device pointers for the matrix, the
// kets and the output; the two work blocks of the recursion and the per-CTA
// partial sums live in one file-scope __device__ array below instead of memory
// the library would allocate.
//
// Limits and sharing: the array holds two work blocks of at most
// kNoAllocMaxEntries complex128 values each (N * R <= 1,048,576) plus the
// partial sums, 32.06 MiB in total.  The CUDA runtime loads a library's device
// code lazily (the default since CUDA 12.2), so the array is not reserved when
// the library is loaded: the first call on each device loads this file's module
// and reserves the 32.06 MiB then, and can fail for lack of memory if the
// device is already full.  Make that first call during set-up, before the
// memory budget is handed out and before capturing any stream; after it the
// array stays reserved on that device until the process exits and later calls
// allocate nothing.  All calls share the array: two calls whose work overlaps
// on the GPU (different streams, or different host threads) race on the same
// scratch and give wrong results; serialise them.  Each call looks up the
// array's device address on the current device (cudaGetSymbolAddress, a
// lookup once the module is loaded), so a context that was reset and created
// again is never handed a stale address.
#include <cuda_runtime.h>

#include "tbk_internal.h"

namespace tbk {
namespace {

constexpr int64_t kNoAllocMaxEntries = int64_t(1) << 20;   // complex128 entries per work block
constexpr int kNoAllocGrid = 512;                          // CTAs of the step kernel
constexpr int kNoAllocThreads = 256;
constexpr size_t kNoAllocBytes = 2 * size_t(kNoAllocMaxEntries) * sizeof(double2) + 2 * kNoAllocGrid * sizeof(double);

// The scratch: [block A][block B][partials: 2 x kNoAllocGrid doubles].
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocBytes];

// Device address of the scratch on the current device.
int noalloc_scratch(void** out) {
  void* p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return fail(TBK_ERR_CUDA, "cudaGetSymbolAddress(no-alloc scratch): %s", cudaGetErrorString(e));
  *out = p;
  return TBK_OK;
}

// Column-major copy of the kets into work block A (the caller's kets stay intact).
__global__ void noalloc_copy_kernel(int64_t total, const double2* __restrict__ src, double2* __restrict__ dst) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
    dst[g] = src[g];
}

// One recursion step on CSR rows, vectors column-major (index i + r*N):
//   first: y = H x                    else: y = 2 H x - y
//   part[b] = sum Re <bras|y>;  first also part[grid + b] = sum Re <bras|x>.
// Threads walk rows grid-stride (consecutive threads, consecutive rows of one
// vector: coalesced); each thread runs the row for every vector in turn.
__global__ void __launch_bounds__(kNoAllocThreads) noalloc_step_kernel(
    int32_t n, int32_t R, const int32_t* __restrict__ row_ptr, const int32_t* __restrict__ col_idx,
    const double* __restrict__ vals, int cplx, const double2* __restrict__ x, double2* __restrict__ y,
    const double2* __restrict__ bras, int first, double* __restrict__ part) {
  double m0 = 0.0, m1 = 0.0;
  for (int32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const int32_t p0 = row_ptr[i], p1 = row_ptr[i + 1];
    for (int32_t r = 0; r < R; ++r) {
      const int64_t base = (int64_t)r * n;
      const int64_t g = base + i;
      double ar = 0.0, ai = 0.0;
      for (int32_t p = p0; p < p1; ++p) {
        const double2 xv = x[base + col_idx[p]];
        if (cplx) {
          const double hr = vals[2 * p], hi = vals[2 * p + 1];
          ar += hr * xv.x - hi * xv.y;
          ai += hr * xv.y + hi * xv.x;
        } else {
          ar += vals[p] * xv.x;
          ai += vals[p] * xv.y;
        }
      }
      double2 out;
      if (first) { out.x = ar; out.y = ai; }
      else { const double2 pv = y[g]; out.x = 2.0 * ar - pv.x; out.y = 2.0 * ai - pv.y; }
      y[g] = out;
      const double2 b = bras[g];
      m0 += b.x * out.x + b.y * out.y;
      if (first) { const double2 xs = x[g]; m1 += b.x * xs.x + b.y * xs.y; }
    }
  }
  __shared__ double sh[2][kNoAllocThreads / 32];
  for (int o = 16; o > 0; o >>= 1) {
    m0 += __shfl_xor_sync(0xffffffffu, m0, o);
    m1 += __shfl_xor_sync(0xffffffffu, m1, o);
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { sh[0][warp] = m0; sh[1][warp] = m1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, c = 0.0;
    for (int q = 0; q < kNoAllocThreads / 32; ++q) { a += sh[0][q]; c += sh[1][q]; }
    part[blockIdx.x] = a;
    part[gridDim.x + blockIdx.x] = c;
  }
}

// Sums the step's partials in a fixed order: mu[k] = slot 0; the first step also
// writes mu[0] = slot 1.
__global__ void noalloc_reduce_kernel(const double* __restrict__ part, int nblk, int k, int first,
                                      double* __restrict__ mu) {
  __shared__ double sh[2][256];
  double a = 0.0, c = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) { a += part[b]; c += part[nblk + b]; }
  sh[0][threadIdx.x] = a;
  sh[1][threadIdx.x] = c;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) { sh[0][threadIdx.x] += sh[0][threadIdx.x + o]; sh[1][threadIdx.x] += sh[1][threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    mu[k] = sh[0][0];
    if (first) mu[0] = sh[1][0];
  }
}

}  // namespace
}  // namespace tbk

using namespace tbk;

extern "C" int tbk_cheb_moments_noalloc(int32_t n_rows, const int32_t* row_ptr, const int32_t* col_idx,
                                        const double* values, int32_t is_complex, int32_t n_mom,
                                        const double* bras, const double* kets, int32_t R, double* mu_out,
                                        void* stream) {
  if (n_mom < 2) return fail(TBK_ERR_INVALID, "n must be greater than or equal to 2");
  if (n_rows < 1 || R < 1) return fail(TBK_ERR_INVALID, "tbk_cheb_moments_noalloc: empty input");
  if ((int64_t)n_rows * R > kNoAllocMaxEntries)
    return fail(TBK_ERR_INVALID,
                "tbk_cheb_moments_noalloc: N*R = %lld exceeds the fixed scratch (at most %lld complex entries per "
                "work block); use tbk_cheb_braket_* or tbk_kpm_* instead",
                (long long)n_rows * R, (long long)kNoAllocMaxEntries);
  if (!row_ptr || !col_idx || !values || !bras || !kets || !mu_out)
    return fail(TBK_ERR_INVALID, "tbk_cheb_moments_noalloc: null argument");
  void* scratch = nullptr;
  TBK_TRY(noalloc_scratch(&scratch));
  cudaStream_t st = as_stream(stream);
  double2* A = static_cast<double2*>(scratch);
  double2* B = A + kNoAllocMaxEntries;
  double* part = reinterpret_cast<double*>(B + kNoAllocMaxEntries);
  const int64_t total = (int64_t)n_rows * R;
  const double2* k2 = reinterpret_cast<const double2*>(kets);
  const double2* b2 = reinterpret_cast<const double2*>(bras);
  noalloc_copy_kernel<<<kNoAllocGrid, kNoAllocThreads, 0, st>>>(total, k2, A);
  TBK_CHECK_LAUNCH();
  double2* x = A;   // v_{k-1}
  double2* y = B;   // v_{k-2} on entry, v_k on exit
  for (int32_t k = 1; k < n_mom; ++k) {
    const int first = k == 1 ? 1 : 0;
    noalloc_step_kernel<<<kNoAllocGrid, kNoAllocThreads, 0, st>>>(n_rows, R, row_ptr, col_idx, values,
                                                                  is_complex ? 1 : 0, x, y, b2, first, part);
    TBK_CHECK_LAUNCH();
    noalloc_reduce_kernel<<<1, 256, 0, st>>>(part, kNoAllocGrid, k, first, mu_out);
    TBK_CHECK_LAUNCH();
    double2* t = x;
    x = y;
    y = t;
  }
  return TBK_OK;
}
