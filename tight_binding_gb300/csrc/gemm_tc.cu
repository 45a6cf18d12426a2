// gemm_tc.cu — the Kubo moment matrix mu_mn on the 5th-generation tensor cores.
//
// mu_mn = sum_k conj(L_m[k]) R_n[k] over stored complex64 Chebyshev blocks, as a
// real GEMM over interleaved (re, im) pairs:
//   Re mu = A . B^T,  Im mu = A . B'^T,  A = L, B = R, B' = per pair (im, -re),
// computed in split precision (3 x TF32): x = hi + lo with hi, lo TF32, and
//   A.B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi           (FP32 accumulation).
//
// One CTA: a 128 (m) x 32 (n, complex) output tile over a K range (split-K).
// The MMA is tcgen05.mma.cta_group::1.kind::tf32 M=128 N=64 K=8 with
// D = [Re | Im] (128 x 64 FP32) in tensor memory.  Roles:
//   warps 0-7  epilogue: every 256 K-elements read the accumulator with
//              tcgen05.ld and add it into FP64 registers (long FP32 sums lose
//              the accuracy the Kubo weights need), double-buffered in TMEM;
//   warps 8-11 converters: load FP32 rows from HBM, split into TF32 hi/lo and
//              write the UMMA K-major no-swizzle layout (8 x 16 B core matrices)
//              into a 4-stage shared-memory ring;
//   warp 12    TMEM allocation and, lane 0, MMA issue + tcgen05.commit.
// Every mbarrier wait is bounded; on timeout the CTA records an error, waits
// (bounded) for its MMAs in flight and frees its tensor memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "tbk_internal.h"

namespace tbk {
namespace {

constexpr int kTM = 128;            // MMA M (output rows m per CTA)
constexpr int kTNc = 32;            // complex output columns n per CTA
constexpr int kTN = 2 * kTNc;       // MMA N (Re | Im)
constexpr int kKS = 32;             // floats per pipeline slab (4 MMA k-steps of 8)
constexpr int kKC = 256;            // floats per FP32 accumulation chunk
constexpr int kStages = 4;
constexpr int kEpiWarps = 8, kCvtWarps = 4;
constexpr int kThreads = 32 * (kEpiWarps + kCvtWarps + 1);
constexpr int kMmaWarp = kEpiWarps + kCvtWarps;
constexpr uint32_t kTmemCols = 2 * kTN;   // two accumulator buffers
constexpr uint32_t kWait = 1u << 24;

// stage layout: A_hi, A_lo (128 rows), B_hi, B_lo (64 rows: 32 B + 32 B')
constexpr int kAPlane = kTM * kKS * 4;    // 16 KB
constexpr int kBPlane = kTN * kKS * 4;    // 8 KB
constexpr int kStageBytes = 2 * kAPlane + 2 * kBPlane;
constexpr int kSmemBytes = kStages * kStageBytes;
constexpr uint32_t kLBO_A = (kTM / 8) * 128;   // bytes between core matrices along K (A)
constexpr uint32_t kLBO_B = (kTN / 8) * 128;   // (B)
constexpr uint32_t kSBO = 128;                 // bytes between 8-row groups along M/N

enum : int { kErrFull = 1, kErrEmpty = 2, kErrAcc = 4, kErrAccEmpty = 8, kErrDrain = 16 };

__device__ __forceinline__ uint32_t s_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bar_init(uint64_t* b, uint32_t c) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_u32(b)), "r"(c) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(s_u32(b)) : "memory");
}
__device__ __forceinline__ bool bar_wait(uint64_t* b, uint32_t parity) {
  for (uint32_t it = 0; it < kWait; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(s_u32(b)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(s_u32(b))
               : "memory");
}
// Shared-memory matrix descriptor: K-major, no swizzle, version 1.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((kSBO >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}
// Instruction descriptor, kind::tf32: D F32, A/B TF32, both K-major, N, M.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
      "l"(a), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ uint32_t to_tf32(float x) {
  uint32_t r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Byte offset of (row, k) inside one operand plane (K-major, no swizzle).
__device__ __forceinline__ uint32_t plane_off(int row, int k, uint32_t lbo) {
  return (uint32_t)((k >> 2) * lbo + (row >> 3) * kSBO + (row & 7) * 16 + (k & 3) * 4);
}

// L, Rb: M blocks in the K-tiled layout (element k of block m at
// ((k/16)*M + m)*16 + k%16, K padded with zeros to whole 16-element tiles); a
// 32-float slab of 128 consecutive blocks is one contiguous 16 KB run.  The CTA
// covers rows m0.., n0.. and floats [kf0, kf1).  Writes FP64 partial tiles.
__global__ void __launch_bounds__(kThreads, 1) mu_tc_kernel(const float2* __restrict__ L, const float2* __restrict__ Rb,
                                                            int32_t M, int64_t K, int64_t kf_split,
                                                            double* __restrict__ part_re, double* __restrict__ part_im,
                                                            int* __restrict__ err) {
  extern __shared__ __align__(1024) unsigned char smem[];
  __shared__ uint64_t full_bar[kStages], empty_bar[kStages], acc_full[2], acc_empty[2], drain_bar;
  __shared__ uint32_t tmem_base_s;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m_tiles = (M + kTM - 1) / kTM;
  const int32_t m0 = (int32_t)(blockIdx.x % m_tiles) * kTM;
  const int32_t n0 = (int32_t)(blockIdx.x / m_tiles) * kTNc;
  const int64_t KF = 2 * K;                                   // floats
  const int64_t kf0 = (int64_t)blockIdx.y * kf_split;
  const int64_t kf1 = min(KF, kf0 + kf_split);
  const int32_t n_slabs = kf1 > kf0 ? (int32_t)((kf1 - kf0 + kKS - 1) / kKS) : 0;
  const int32_t slabs_per_chunk = kKC / kKS;
  const int32_t n_chunks = (n_slabs + slabs_per_chunk - 1) / slabs_per_chunk;

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) { bar_init(&full_bar[s], kCvtWarps); bar_init(&empty_bar[s], 1); }
    for (int b = 0; b < 2; ++b) { bar_init(&acc_full[b], 1); bar_init(&acc_empty[b], kEpiWarps); }
    bar_init(&drain_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaWarp) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(s_u32(&tmem_base_s)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;

  if (warp >= kEpiWarps && warp < kMmaWarp) {
    // ------------------------------------------------------------ converters
    const int t = threadIdx.x - 32 * kEpiWarps;     // 0..127
    for (int32_t s = 0; s < n_slabs; ++s) {
      const int st = s % kStages;
      const uint32_t ph = (uint32_t)(s / kStages) & 1u;
      if (!bar_wait(&empty_bar[st], ph ^ 1u)) { atomicOr(err, kErrEmpty); break; }
      unsigned char* sb = smem + (size_t)st * kStageBytes;
      const int64_t kf = kf0 + (int64_t)s * kKS;
      // A row t: the 32 floats of K-tile kf/32 of block m0 + t (consecutive threads
      // read consecutive 128-byte rows: one coalesced 16 KB run per slab)
      const int64_t tile = kf >> 5;
      {
        const int32_t m = m0 + t;
        const float4* src = reinterpret_cast<const float4*>(L + (tile * M + m) * 16);
#pragma unroll
        for (int q = 0; q < kKS / 4; ++q) {
          const float4 v = (m < M) ? __ldcs(src + q) : make_float4(0.f, 0.f, 0.f, 0.f);
          const float x[4] = {v.x, v.y, v.z, v.w};
          uint32_t hi[4], lo[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) { hi[e] = to_tf32(x[e]); lo[e] = to_tf32(x[e] - __uint_as_float(hi[e])); }
          const uint32_t o = plane_off(t, 4 * q, kLBO_A);
          *reinterpret_cast<uint4*>(sb + o) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
          *reinterpret_cast<uint4*>(sb + kAPlane + o) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
        }
      }
      // B rows: t < 32 -> row t (R_n) and row 32 + t (pairs (im, -re))
      if (t < kTNc) {
        const int32_t n = n0 + t;
        const float4* src = reinterpret_cast<const float4*>(Rb + (tile * M + n) * 16);
#pragma unroll
        for (int q = 0; q < kKS / 4; ++q) {
          const float4 v = (n < M) ? __ldcs(src + q) : make_float4(0.f, 0.f, 0.f, 0.f);
          const float x[4] = {v.x, v.y, v.z, v.w};
          const float xp[4] = {v.y, -v.x, v.w, -v.z};      // (re, im) -> (im, -re)
          uint32_t hi[4], lo[4], hp[4], lp[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            hi[e] = to_tf32(x[e]); lo[e] = to_tf32(x[e] - __uint_as_float(hi[e]));
            hp[e] = to_tf32(xp[e]); lp[e] = to_tf32(xp[e] - __uint_as_float(hp[e]));
          }
          const uint32_t o = plane_off(t, 4 * q, kLBO_B), op = plane_off(kTNc + t, 4 * q, kLBO_B);
          unsigned char* bh = sb + 2 * kAPlane;
          unsigned char* bl = bh + kBPlane;
          *reinterpret_cast<uint4*>(bh + o) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
          *reinterpret_cast<uint4*>(bl + o) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
          *reinterpret_cast<uint4*>(bh + op) = make_uint4(hp[0], hp[1], hp[2], hp[3]);
          *reinterpret_cast<uint4*>(bl + op) = make_uint4(lp[0], lp[1], lp[2], lp[3]);
        }
      }
      // make the generic-proxy writes visible to the tensor cores, then signal
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      __syncwarp();
      if (lane == 0) bar_arrive(&full_bar[st]);
    }
  } else if (warp == kMmaWarp) {
    // ------------------------------------------------------------ MMA issue
    if (lane == 0) {
      bool ok = true;
      int32_t s = 0;
      for (int32_t c = 0; c < n_chunks && ok; ++c) {
        const int b = c & 1;
        const uint32_t acc = tmem + (uint32_t)(b * kTN);
        if (c >= 2) {
          if (!bar_wait(&acc_empty[b], (uint32_t)((c - 2) >> 1) & 1u)) { atomicOr(err, kErrAccEmpty); ok = false; break; }
          tc_fence_after();
        }
        const int32_t s_end = min(n_slabs, (c + 1) * slabs_per_chunk);
        bool first = true;
        for (; s < s_end; ++s) {
          const int st = s % kStages;
          if (!bar_wait(&full_bar[st], (uint32_t)(s / kStages) & 1u)) { atomicOr(err, kErrFull); ok = false; break; }
          tc_fence_after();
          const uint32_t sb = s_u32(smem + (size_t)st * kStageBytes);
#pragma unroll
          for (int j = 0; j < kKS / 8; ++j) {
            const uint32_t ka = (uint32_t)j * 2u * kLBO_A, kb = (uint32_t)j * 2u * kLBO_B;
            const uint64_t ah = smem_desc(sb + ka, kLBO_A), al = smem_desc(sb + kAPlane + ka, kLBO_A);
            const uint64_t bh = smem_desc(sb + 2 * kAPlane + kb, kLBO_B);
            const uint64_t bl = smem_desc(sb + 2 * kAPlane + kBPlane + kb, kLBO_B);
            mma_tf32(acc, ah, bh, first ? 0u : 1u);
            mma_tf32(acc, ah, bl, 1u);
            mma_tf32(acc, al, bh, 1u);
            first = false;
          }
          tc_commit(&empty_bar[st]);       // frees the stage when these MMAs finish
        }
        if (ok) tc_commit(&acc_full[b]);   // accumulator chunk ready for the epilogue
      }
      // all MMAs this thread issued have completed before tensor memory is freed
      tc_commit(&drain_bar);
      if (!bar_wait(&drain_bar, 0)) atomicOr(err, kErrDrain);
    }
    __syncwarp();
  } else {
    // ------------------------------------------------------------ epilogue
    const int grp = warp & 3;           // TMEM lanes 32*grp .. 32*grp+31
    const int half = warp >> 2;         // 0: Re columns, 1: Im columns
    double acc64[kTNc];
#pragma unroll
    for (int j = 0; j < kTNc; ++j) acc64[j] = 0.0;
    for (int32_t c = 0; c < n_chunks; ++c) {
      const int b = c & 1;
      if (!bar_wait(&acc_full[b], (uint32_t)(c >> 1) & 1u)) { atomicOr(err, kErrAcc); break; }
      tc_fence_after();
      const uint32_t taddr = tmem + ((uint32_t)(32 * grp) << 16) + (uint32_t)(b * kTN + half * kTNc);
      float v[32];
      tmem_ld32(taddr, v);
#pragma unroll
      for (int j = 0; j < 32; ++j) acc64[j] += (double)v[j];
      tc_fence_before();
      __syncwarp();
      if (lane == 0) bar_arrive(&acc_empty[b]);
    }
    const int32_t m = m0 + 32 * grp + lane;
    if (m < M) {
      double* dst = (half ? part_im : part_re) + ((int64_t)blockIdx.y * M + m) * M;
#pragma unroll
      for (int j = 0; j < kTNc; ++j)
        if (n0 + j < M) dst[n0 + j] = acc64[j];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

__global__ void mu_tc_reduce_kernel(const double* __restrict__ pr, const double* __restrict__ pi, int32_t M,
                                    int32_t nsplit, double2* __restrict__ acc) {
  const int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= (int64_t)M * M) return;
  double r = 0.0, i = 0.0;
  for (int32_t s = 0; s < nsplit; ++s) { r += pr[(int64_t)s * M * M + q]; i += pi[(int64_t)s * M * M + q]; }
  acc[q].x += r;
  acc[q].y += i;
}

}  // namespace

int mu_gemm_tc(const float2* L, const float2* Rb, int32_t M, int64_t K, double* mu_acc, cudaStream_t st) {
  if (M < 1 || K < 1) return fail(TBK_ERR_INVALID, "mu_gemm_tc: empty problem");
  if (((uintptr_t)L | (uintptr_t)Rb) & 15) return fail(TBK_ERR_INVALID, "mu_gemm_tc: blocks must be 16-byte aligned");
  static bool configured = false;
  if (!configured) {
    TBK_CUDA(cudaFuncSetAttribute(mu_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
    configured = true;
  }
  const int m_tiles = (M + kTM - 1) / kTM, n_tiles = (M + kTNc - 1) / kTNc;
  const int tiles = m_tiles * n_tiles;
  // split K so that about two waves of CTAs cover the GPU; whole chunks per split
  const int64_t KF = 2 * K;
  int nsplit = std::max(1, (2 * sm_count() + tiles - 1) / tiles);
  int64_t kf_split = (KF + nsplit - 1) / nsplit;
  kf_split = ((kf_split + kKC - 1) / kKC) * kKC;
  nsplit = (int)((KF + kf_split - 1) / kf_split);
  DevBuf pr, pi, errb;
  TBK_TRY(pr.alloc(sizeof(double) * (size_t)nsplit * M * M));
  TBK_TRY(pi.alloc(sizeof(double) * (size_t)nsplit * M * M));
  TBK_TRY(errb.alloc(sizeof(int)));
  TBK_CUDA(cudaMemsetAsync(errb.p, 0, sizeof(int), st));
  dim3 grid(tiles, nsplit);
  mu_tc_kernel<<<grid, kThreads, kSmemBytes, st>>>(L, Rb, M, K, kf_split, pr.as<double>(), pi.as<double>(),
                                                   errb.as<int>());
  TBK_CHECK_LAUNCH();
  mu_tc_reduce_kernel<<<(unsigned)(((int64_t)M * M + 255) / 256), 256, 0, st>>>(pr.as<double>(), pi.as<double>(), M,
                                                                               nsplit, reinterpret_cast<double2*>(mu_acc));
  TBK_CHECK_LAUNCH();
  int herr = 0;
  TBK_CUDA(cudaMemcpyAsync(&herr, errb.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  if (herr) return fail(TBK_ERR_TIMEOUT, "tensor-core mu_nm kernel gave up waiting (code %d)", herr);
  return TBK_OK;
}

}  // namespace tbk
