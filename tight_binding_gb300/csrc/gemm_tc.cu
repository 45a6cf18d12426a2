// gemm_tc.cu — the Kubo moment matrix mu_mn on the 5th-generation tensor cores.
//
// mu_mn = sum_k conj(L_m[k]) R_n[k] over stored complex64 Chebyshev blocks, as a
// real GEMM over interleaved (re, im) pairs:
//   Re mu = A . B^T,  Im mu = A . B'^T,  A = L, B = R, B' = per pair (im, -re),
// computed in split precision (3 x TF32): x = hi + lo with hi = rna_tf32(x) and
// lo = rna_tf32(x - hi) (|lo| <= 2^-11 |x|, and the omitted lo.lo term has no
// sign bias), and
//   A.B ~ A_hi B_hi + A_hi B_lo + A_lo B_hi           (FP32 accumulation).
//
// One CTA: a 128 (m) x 64 (n, complex) output tile over a K range (split-K).
// The MMA is tcgen05.mma.cta_group::1.kind::tf32 M=128 N=128 K=8 with
// D = [Re | Im] (128 x 128 FP32) in tensor memory.  The stored blocks are
// K-tiled (16 complex = 32 floats of K per block row, 128 B), so one K tile of
// 128 consecutive blocks is a 128-row x 128-B box: TMA loads it with the
// 128-byte swizzle straight into the UMMA K-major SWIZZLE_128B layout.  Two
// CTAs of a cluster share an m tile (adjacent n tiles): each loads half of the
// A box and multicasts it to both, and a stage is reused only when both CTAs'
// MMAs have released it (their commits arrive on both CTAs' barriers).  A
// (hi and lo) then lives in tensor memory, B (hi, lo, and B' of each) in
// shared memory, so the MMAs read only B through the shared-memory port.
// Roles:
//   warp 21    TMA producer: one thread issues the A and B boxes of each stage;
//   warps 16-19 converters: each thread takes one A row (its TMEM lane), splits
//              it into hi / lo and stores both with tcgen05.st; B is split in
//              place per 16-byte chunk with B' hi, B lo, B' lo beside it
//              (elementwise, so the swizzle is irrelevant);
//   warp 20    TMEM allocation and, lane 0, MMA issue + tcgen05.commit;
//   warps 0-15 epilogue (32 columns each): every 256 K-floats read the
//              accumulator with tcgen05.ld and add it into float-float (hi, lo)
//              pairs by TwoSum (long FP32 sums lose the accuracy the Kubo
//              weights need; FP64 adds would saturate GB300's FP64 pipe),
//              double-buffered in TMEM; FP64 once at the end.
// Every mbarrier wait is bounded; on timeout the CTA records an error, waits
// (bounded) for its copies and MMAs in flight and frees its tensor memory.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <mutex>
#include <vector>

#include "tbk_internal.h"

namespace tbk {
namespace {

constexpr int kTM = 128;            // MMA M (output rows m per CTA)
constexpr int kTNc = 64;            // complex output columns n per CTA
constexpr int kTN = 2 * kTNc;       // MMA N (Re | Im)
constexpr int kKS = 32;             // floats per stage: one K tile (4 MMA k-steps of 8)
constexpr int kKC = 256;            // floats per FP32 accumulation chunk
constexpr int kStages = 4;
constexpr int kEpiWarps = 16, kCvtWarps = 4;
constexpr int kMmaWarp = kEpiWarps + kCvtWarps;
constexpr int kTmaWarp = kMmaWarp + 1;
constexpr int kThreads = 32 * (kTmaWarp + 1);
// tensor memory columns: two accumulators, then per stage A hi (32) | A lo (32)
constexpr uint32_t kAccCols = 2 * kTN;
constexpr uint32_t kACols = 2 * kKS;
constexpr uint32_t kTmemCols = 512;
static_assert(kAccCols + kStages * kACols <= kTmemCols, "tensor memory budget");
constexpr uint32_t kWait = 1u << 24;

// stage layout (every region 1024-byte aligned, so that derived planes carry
// the raw planes' swizzle): A raw | B raw/hi | B' hi | B lo | B' lo.
// B hi and B' hi form one 128-row operand, B lo and B' lo another.
constexpr int kAPlane = kTM * kKS * 4;    // 16 KB
constexpr int kBPlane = kTNc * kKS * 4;   // 8 KB (64 rows)
constexpr int kOffAraw = 0;
constexpr int kOffBhi = kOffAraw + kAPlane;
constexpr int kOffBphi = kOffBhi + kBPlane;
constexpr int kOffBlo = kOffBphi + kBPlane;
constexpr int kOffBplo = kOffBlo + kBPlane;
constexpr int kStageBytes = kOffBplo + kBPlane;   // 48 KB
constexpr int kSmemBytes = kStages * kStageBytes + 1024;   // + alignment slack
constexpr uint32_t kTxBytes = kAPlane + kBPlane;           // raw bytes per stage
constexpr uint32_t kSBO = 1024;                 // 8 rows x 128 B swizzle atom

enum : int { kErrFull = 1, kErrEmpty = 2, kErrAcc = 4, kErrAccEmpty = 8, kErrDrain = 16, kErrRaw = 32 };

__device__ __forceinline__ uint32_t s_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void bar_init(uint64_t* b, uint32_t c) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(s_u32(b)), "r"(c) : "memory");
}
__device__ __forceinline__ void bar_arrive(uint64_t* b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(s_u32(b)) : "memory");
}
__device__ __forceinline__ void bar_arrive_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(s_u32(b)), "r"(bytes) : "memory");
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
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int32_t x, int32_t y, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          s_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(s_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_2d_mc(void* dst, const CUtensorMap* map, int32_t x, int32_t y, uint64_t* bar,
                                               uint16_t mask) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(s_u32(dst)),
      "l"(map), "r"(x), "r"(y), "r"(s_u32(bar)), "h"(mask)
      : "memory");
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void tc_commit_mc(uint64_t* b, uint16_t mask) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(
          s_u32(b)),
      "h"(mask)
      : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_commit(uint64_t* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(s_u32(b))
               : "memory");
}
// Shared-memory matrix descriptor: K-major, 128-byte swizzle, version 1; the
// leading offset is unused for swizzled K-major operands, the stride offset is
// one 8-row swizzle atom.
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t saddr) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)((kSBO >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  d |= (uint64_t)2 << 61;
  return d;
}
// Instruction descriptor, kind::tf32: D F32, A/B TF32, both K-major, N, M.
constexpr uint32_t kIdesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(kTN >> 3) << 17) |
                            ((uint32_t)(kTM >> 4) << 24);
// D (tmem) += A (tmem: lane = row, column = k) . B (shared-memory descriptor)
__device__ __forceinline__ void mma_tf32_ts(uint32_t d_tmem, uint32_t a_tmem, uint64_t b, uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::tf32 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
      "r"(a_tmem), "l"(b), "r"(kIdesc), "r"(accumulate)
      : "memory");
}
// 16 consecutive columns of this warp's 32 tensor-memory lanes from registers
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t* r) {
  asm volatile(
      "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
          taddr),
      "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]), "r"(r[9]),
      "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
      : "memory");
}
// TF32 value of x, rounded to nearest with ties away from zero (the rounding
// of cvt.rna.tf32.f32), on the integer pipe: TF32 keeps 10 of FP32's 23
// mantissa bits, so adding half a unit of the 13 dropped bits (0x1000) to the
// sign-magnitude pattern and clearing them rounds the magnitude half-up
// (a carry into the exponent is the correct rounding to the next binade).
// Finite inputs only (the stored blocks are finite).
__device__ __forceinline__ float to_tf32_rna(float x) {
  return __uint_as_float((__float_as_uint(x) + 0x1000u) & 0xFFFFE000u);
}
// (hi, lo) += v with TwoSum (Knuth): hi + lo carries the sum to ~2^-48.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float v) {
  const float s = hi + v;
  const float bp = s - hi;
  const float e = (hi - (s - bp)) + (v - bp);
  hi = s;
  lo += e;
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
// L, Rb: M blocks in the K-tiled layout (element k of block m at
// ((k/16)*M + m)*16 + k%16, K padded with zeros to whole 16-element tiles),
// seen by the tensor maps as rows of 32 floats: row (k/16)*M + m.  The CTA
// covers rows m0.., n0.. and floats [kf0, kf1) (kf0 a multiple of kKC).
// Writes FP64 partial tiles.
__global__ void __launch_bounds__(kThreads, 1) mu_tc_kernel(const __grid_constant__ CUtensorMap map_l,
                                                            const __grid_constant__ CUtensorMap map_r, int32_t M,
                                                            int64_t K, int64_t kf_split,
                                                            double* __restrict__ part_re, double* __restrict__ part_im,
                                                            int* __restrict__ err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~(uintptr_t)1023);
  __shared__ uint64_t raw_bar[kStages], full_bar[kStages], empty_bar[kStages], acc_full[2], acc_empty[2], drain_bar;
  __shared__ uint32_t tmem_base_s;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // blockIdx.x = m_tile * n_tiles_p + n_tile (n_tiles_p even): cluster pairs
  // share the m tile
  const int n_tiles_p = ((M + kTNc - 1) / kTNc + 1) & ~1;
  const int32_t m0 = (int32_t)(blockIdx.x / n_tiles_p) * kTM;
  const int32_t n0 = (int32_t)(blockIdx.x % n_tiles_p) * kTNc;
  const uint32_t crank = cluster_rank();
  const int64_t KF = 2 * K;                                   // floats
  const int64_t kf0 = (int64_t)blockIdx.y * kf_split;
  const int64_t kf1 = min(KF, kf0 + kf_split);
  const int32_t n_slabs = kf1 > kf0 ? (int32_t)((kf1 - kf0 + kKS - 1) / kKS) : 0;
  const int32_t slabs_per_chunk = kKC / kKS;
  const int32_t n_chunks = (n_slabs + slabs_per_chunk - 1) / slabs_per_chunk;
  const int32_t tile0 = (int32_t)(kf0 / kKS);

  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) { bar_init(&raw_bar[s], 1); bar_init(&full_bar[s], kCvtWarps); bar_init(&empty_bar[s], 2); }
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
  cluster_sync();        // the peer's barriers exist before any multicast reaches them
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;

  if (warp == kTmaWarp) {
    // ------------------------------------------------------------ TMA producer
    if (lane == 0) {
      asm volatile("prefetch.tensormap [%0];" ::"l"(&map_l) : "memory");
      asm volatile("prefetch.tensormap [%0];" ::"l"(&map_r) : "memory");
      int32_t issued = 0;
      for (int32_t s = 0; s < n_slabs; ++s) {
        const int st = s % kStages;
        const uint32_t ph = (uint32_t)(s / kStages) & 1u;
        if (!bar_wait(&empty_bar[st], ph ^ 1u)) { atomicOr(err, kErrEmpty); break; }
        unsigned char* sb = smem + (size_t)st * kStageBytes;
        const int32_t row = (tile0 + s) * M;
        bar_arrive_tx(&raw_bar[st], kTxBytes);
        // this CTA's half of the A box, to both CTAs of the pair
        tma_load_2d_mc(sb + kOffAraw + crank * (kAPlane / 2), &map_l, 0, row + m0 + (int32_t)crank * (kTM / 2),
                       &raw_bar[st], (uint16_t)0x3);
        tma_load_2d(sb + kOffBhi, &map_r, 0, row + n0, &raw_bar[st]);
        issued = s + 1;
      }
      // copies in flight complete before the CTA may leave (bounded)
      for (int32_t s = max(0, issued - kStages); s < issued; ++s)
        if (!bar_wait(&raw_bar[s % kStages], (uint32_t)(s / kStages) & 1u)) { atomicOr(err, kErrRaw); break; }
    }
    __syncwarp();
  } else if (warp >= kEpiWarps && warp < kMmaWarp) {
    // ------------------------------------------------------------ converters
    const int t = threadIdx.x - 32 * kEpiWarps;     // 0..127
    for (int32_t s = 0; s < n_slabs; ++s) {
      const int st = s % kStages;
      const uint32_t ph = (uint32_t)(s / kStages) & 1u;
      if (!bar_wait(&raw_bar[st], ph)) { atomicOr(err, kErrFull); break; }
      unsigned char* sb = smem + (size_t)st * kStageBytes;
      // A row r (this warp's TMEM lane quarter): its 8 swizzled 16-byte chunks
      // (chunk c of row r sits at chunk c ^ (r & 7) of the 128-byte row)
      const int r = 32 * (warp & 3) + lane;
      const unsigned char* arow = sb + kOffAraw + r * 128;
      const uint32_t acol = tmem + ((uint32_t)(32 * (warp & 3)) << 16) + kAccCols + (uint32_t)st * kACols;
#pragma unroll
      for (int half = 0; half < 2; ++half) {     // 16 floats at a time (registers)
        uint32_t hi[16], lo[16];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const int c = 4 * half + u;
          const float4 v = *reinterpret_cast<const float4*>(arow + ((c ^ (r & 7)) << 4));
          const float x[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            const float h = to_tf32_rna(x[e]);
            hi[4 * u + e] = __float_as_uint(h);
            lo[4 * u + e] = __float_as_uint(to_tf32_rna(x[e] - h));
          }
        }
        tmem_st16(acol + 16u * half, hi);
        tmem_st16(acol + kKS + 16u * half, lo);
      }
      // B: 512 chunks, 4 per thread; B' = per (re, im) pair (im, -re)
      constexpr int kQB = kBPlane / 16 / 128;
      float4* bhp = reinterpret_cast<float4*>(sb + kOffBhi);
      float4 vb[kQB];
#pragma unroll
      for (int q = 0; q < kQB; ++q) vb[q] = bhp[q * 128 + t];
#pragma unroll
      for (int q = 0; q < kQB; ++q) {
        const int c = q * 128 + t;
        const float4 v = vb[q];
        const float4 h = make_float4(to_tf32_rna(v.x), to_tf32_rna(v.y), to_tf32_rna(v.z), to_tf32_rna(v.w));
        const float4 l = make_float4(to_tf32_rna(v.x - h.x), to_tf32_rna(v.y - h.y), to_tf32_rna(v.z - h.z),
                                     to_tf32_rna(v.w - h.w));
        bhp[c] = h;
        reinterpret_cast<float4*>(sb + kOffBphi)[c] = make_float4(h.y, -h.x, h.w, -h.z);
        reinterpret_cast<float4*>(sb + kOffBlo)[c] = l;
        reinterpret_cast<float4*>(sb + kOffBplo)[c] = make_float4(l.y, -l.x, l.w, -l.z);
      }
      asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
      tc_fence_before();
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
          const uint32_t a_hi = tmem + kAccCols + (uint32_t)st * kACols, a_lo = a_hi + kKS;
#pragma unroll
          for (int j = 0; j < kKS / 8; ++j) {
            const uint32_t kb = (uint32_t)j * 32u;     // 8 tf32 = 32 B along the 128-B swizzled row
            const uint64_t bh = smem_desc_sw128(sb + kOffBhi + kb), bl = smem_desc_sw128(sb + kOffBlo + kb);
            mma_tf32_ts(acc, a_hi + 8u * j, bh, first ? 0u : 1u);
            mma_tf32_ts(acc, a_hi + 8u * j, bl, 1u);
            mma_tf32_ts(acc, a_lo + 8u * j, bh, 1u);
            first = false;
          }
          tc_commit_mc(&empty_bar[st], (uint16_t)0x3);   // frees the stage (in both CTAs) when these MMAs finish
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
    const int colq = warp >> 2;         // columns 32*colq ..: 0, 1 Re; 2, 3 Im
    float acc_hi[32], acc_lo[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) { acc_hi[j] = 0.f; acc_lo[j] = 0.f; }
    for (int32_t c = 0; c < n_chunks; ++c) {
      const int b = c & 1;
      if (!bar_wait(&acc_full[b], (uint32_t)(c >> 1) & 1u)) { atomicOr(err, kErrAcc); break; }
      tc_fence_after();
      const uint32_t taddr = tmem + ((uint32_t)(32 * grp) << 16) + (uint32_t)(b * kTN + colq * 32);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float v[16];
        tmem_ld16(taddr + 16u * h, v);
#pragma unroll
        for (int j = 0; j < 16; ++j) two_sum_acc(acc_hi[16 * h + j], acc_lo[16 * h + j], v[j]);
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) bar_arrive(&acc_empty[b]);
    }
    const int32_t m = m0 + 32 * grp + lane;
    const int32_t nb = n0 + 32 * (colq & 1);
    if (m < M) {
      double* dst = (colq >= 2 ? part_im : part_re) + ((int64_t)blockIdx.y * M + m) * M;
#pragma unroll
      for (int j = 0; j < 32; ++j)
        if (nb + j < M) dst[nb + j] = (double)acc_hi[j] + (double)acc_lo[j];
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == kMmaWarp) {
    tc_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
  cluster_sync();        // no multicast or remote arrive targets a CTA that has left
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

using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  });
  return fn;
}

// Tensor map over a K-tiled block store: rows of 32 floats (128 B), `rows`
// rows, boxes of 32 floats x box_rows rows, 128-byte swizzle, zero fill past
// the end.
int block_map(CUtensorMap* map, const float2* base, int64_t rows, uint32_t box_rows) {
  EncodeTiledFn enc = encode_tiled();
  if (!enc) return fail(TBK_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[2] = {32, (cuuint64_t)rows};
  const cuuint64_t strides[1] = {128};
  const cuuint32_t box[2] = {32, box_rows};
  const cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float2*>(base), dims, strides, box, estr,
                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                   CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(TBK_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
  return TBK_OK;
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
  const int64_t tiles16 = (K + 15) / 16;                 // K tiles of the store (zero padded)
  if (tiles16 * (int64_t)M > INT32_MAX) return fail(TBK_ERR_UNSUPPORTED, "mu_gemm_tc: store too large for TMA rows");
  CUtensorMap map_l, map_r;
  TBK_TRY(block_map(&map_l, L, tiles16 * M, kTM / 2));
  TBK_TRY(block_map(&map_r, Rb, tiles16 * M, kTNc));
  const int m_tiles = (M + kTM - 1) / kTM, n_tiles = ((M + kTNc - 1) / kTNc + 1) & ~1;   // pairs
  const int tiles = m_tiles * n_tiles;
  // split K (whole accumulation chunks per split) so that the CTAs fill whole
  // waves of one CTA per SM: the fewest splits whose last wave is >= 95% full
  const int64_t KF = 2 * K;
  const int sms = sm_count();
  const int64_t chunks = (KF + kKC - 1) / kKC;
  int nsplit = 1;
  double best = 0.0;
  for (int ns = 1; ns <= 256 && ns <= chunks; ++ns) {
    const int64_t units = (int64_t)tiles * ns;
    const int64_t waves = (units + sms - 1) / sms;
    const double eff = (double)units / (double)(waves * sms);
    if (eff > best + 1e-9) { best = eff; nsplit = ns; }
    if (eff >= 0.95 && units >= sms) { nsplit = ns; break; }
  }
  int64_t kf_split = (chunks + nsplit - 1) / nsplit * kKC;
  nsplit = (int)((KF + kf_split - 1) / kf_split);
  DevBuf pr, pi, errb;
  TBK_TRY(pr.alloc(sizeof(double) * (size_t)nsplit * M * M));
  TBK_TRY(pi.alloc(sizeof(double) * (size_t)nsplit * M * M));
  TBK_TRY(errb.alloc(sizeof(int)));
  TBK_CUDA(cudaMemsetAsync(errb.p, 0, sizeof(int), st));
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(tiles, nsplit);
  cfg.blockDim = dim3(kThreads);
  cfg.dynamicSmemBytes = kSmemBytes;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = 2;
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  TBK_CUDA(cudaLaunchKernelEx(&cfg, mu_tc_kernel, map_l, map_r, M, K, kf_split, pr.as<double>(), pi.as<double>(),
                              errb.as<int>()));
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
