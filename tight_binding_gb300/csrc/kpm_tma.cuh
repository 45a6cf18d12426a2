// kpm_tma.cuh — TMA-staged, warp-specialised Chebyshev recursion step (sm_103a).
//
// One CTA = 1 producer warp + NCW consumer warps, persistent over row tiles of
// TR rows (TR a multiple of the 32-row ELL slice).  The producer's elected lane
// streams every contiguous operand of a tile into a STAGES-deep shared-memory
// ring with 1-D bulk TMA copies (cp.async.bulk ... mbarrier::complete_tx):
//     v_n rows of the tile, v_{n-1} rows, ELL column/value chunk, diagonal,
//     (bras rows in braket mode).
// Consumer warps wait on the stage's "full" mbarrier, read those operands from
// shared memory, issue only the neighbour gathers v_n[col] (global, mostly L2
// hits), write v_{n+1} with coalesced 128-bit stores and fold the moment dot
// products into the pass; then they arrive on the stage's "empty" mbarrier.
//
// Every wait is bounded: after `wait_limit` polls (kWaitLimit unless the host
// lowered it to exercise this path) a ring wait records an error code in a
// global flag and the warp leaves its loop.  Before it leaves, the producer
// always waits for the copies it still has in flight (bounded by kWaitLimit,
// whatever wait_limit is: the copies are real reads that complete), so no bulk
// copy outlives its CTA even when the consumers stopped early.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tbk {

constexpr uint32_t kWaitLimit = 1u << 24;
enum : int { kErrFullWait = 1, kErrEmptyWait = 2, kErrDrain = 4 };

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait; returns false (and the caller records an error) after `limit`
// polls without completion (limit 0: no poll at all).
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t limit = kWaitLimit) {
  for (uint32_t it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}
// 1-D bulk copy global -> shared, completion counted on `bar` (bytes % 16 == 0,
// both addresses 16-byte aligned).
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
// Same with an L2 cache policy (e.g. evict-first for data read exactly once).
__device__ __forceinline__ void bulk_g2s_hint(void* dst, const void* src, uint32_t bytes, uint64_t* bar,
                                              uint64_t policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], %4;" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar)), "l"(policy)
      : "memory");
}
__device__ __forceinline__ uint64_t policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}

// Shared-memory layout of one stage (byte offsets, all 128-byte aligned).
struct TmaLayout {
  int32_t TR;            // rows per tile
  int32_t wmax;          // max ELL width over all slices
  int32_t vec_bytes;     // TR * R * sizeof(complex)
  int32_t col_bytes;     // TR * wmax * 4
  int32_t val_bytes;     // TR * wmax * sizeof(H value)
  int32_t diag_bytes;    // TR * sizeof(H value)
  int32_t off_x, off_prev, off_bras, off_col, off_val, off_diag, stage_bytes;
};

__host__ __device__ inline int32_t align128(int32_t x) { return (x + 127) & ~127; }

inline TmaLayout make_tma_layout(int TR, int wmax, int R, int csize, int hsize, bool braket) {
  TmaLayout L;
  L.TR = TR;
  L.wmax = wmax;
  L.vec_bytes = TR * R * csize;
  L.col_bytes = TR * wmax * 4;
  L.val_bytes = TR * wmax * hsize;
  L.diag_bytes = TR * hsize;
  int32_t o = 0;
  L.off_x = o; o += align128(L.vec_bytes);
  L.off_prev = o; o += align128(L.vec_bytes);
  L.off_bras = o; o += braket ? align128(L.vec_bytes) : 0;
  L.off_col = o; o += align128(L.col_bytes);
  L.off_val = o; o += align128(L.val_bytes);
  L.off_diag = o; o += align128(L.diag_bytes);
  L.stage_bytes = o;
  return L;
}

constexpr int kTmaConsumerWarps = 8;
constexpr int kTmaThreads = 32 * (kTmaConsumerWarps + 1);

template <typename F, int R, bool CPLX_H, bool BRAKET, int STAGES>
__global__ void __launch_bounds__(kTmaThreads) kpm_tma_step_kernel(
    int32_t n, int32_t n_slices, int32_t n_tiles, TmaLayout L, const int32_t* __restrict__ soff, const int32_t* __restrict__ ecol,
    const F* __restrict__ eval, const F* __restrict__ diag, const typename C2<F>::T* __restrict__ x,
    typename C2<F>::T* y, const typename C2<F>::T* __restrict__ bras, double* __restrict__ part, int store,
    int reverse, int gather, int first, int* __restrict__ err, uint32_t wait_limit) {
  using CT = typename C2<F>::T;
  constexpr int VPL = (R >= VecW<F>::max_vpl) ? VecW<F>::max_vpl : 1;
  constexpr int LPR = R / VPL;          // lanes per row
  constexpr int RPW = 32 / LPR;         // rows per warp pass
  constexpr int HS = CPLX_H ? 2 : 1;    // H value size in F units
  static_assert(LPR >= 1 && LPR <= 32 && (32 % LPR) == 0, "R out of range");

  extern __shared__ __align__(128) unsigned char smem[];
  __shared__ uint64_t full_bar[STAGES], empty_bar[STAGES];
  __shared__ double red[2][kTmaConsumerWarps];

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(&full_bar[s], 1);
      mbar_init(&empty_bar[s], kTmaConsumerWarps);
    }
    mbar_fence_init();
  }
  __syncthreads();

  const int32_t my_tiles = (blockIdx.x < (uint32_t)n_tiles) ? (n_tiles - 1 - (int32_t)blockIdx.x) / (int32_t)gridDim.x + 1 : 0;
  auto tile_of = [&](int32_t k) -> int32_t {
    int32_t t = (int32_t)blockIdx.x + k * (int32_t)gridDim.x;
    return reverse ? (n_tiles - 1 - t) : t;
  };
  const int32_t slices_per_tile = L.TR >> 5;

  if (warp == kTmaConsumerWarps) {
    // ------------------------------------------------------------ producer
    if (lane == 0) {
      int32_t issued = 0;
      bool ok = true;
      const uint64_t once = policy_evict_first();   // v_{n-1}, bras and the ELL are read once
      for (int32_t k = 0; k < my_tiles; ++k) {
        const int st = k % STAGES;
        const uint32_t ph = (uint32_t)(k / STAGES) & 1u;
        if (!mbar_wait_bounded(&empty_bar[st], ph ^ 1u, wait_limit)) { atomicOr(err, kErrEmptyWait); ok = false; break; }
        const int32_t tile = tile_of(k);
        const int32_t r0 = tile * L.TR;
        const int32_t s0 = tile * slices_per_tile;
        // the last tile may hold fewer slices; vectors are padded to whole slices
        const int32_t ns = min(slices_per_tile, n_slices - s0);
        const uint32_t vbytes = (uint32_t)ns * 32u * (uint32_t)(R * sizeof(CT));
        const uint32_t dbytes = (uint32_t)ns * 32u * (uint32_t)(sizeof(F) * HS);
        const int32_t e0 = __ldg(soff + s0), e1 = __ldg(soff + s0 + ns);
        const uint32_t ell_n = (uint32_t)(e1 - e0);
        uint32_t bytes = vbytes + dbytes;
        if (!first) bytes += vbytes;
        if (BRAKET) bytes += vbytes;
        if (gather && ell_n) bytes += ell_n * 4u + ell_n * (uint32_t)(sizeof(F) * HS);
        unsigned char* sb = smem + (size_t)st * L.stage_bytes;
        mbar_arrive_expect_tx(&full_bar[st], bytes);
        bulk_g2s(sb + L.off_x, x + (size_t)r0 * R, vbytes, &full_bar[st]);
        if (!first) bulk_g2s_hint(sb + L.off_prev, y + (size_t)r0 * R, vbytes, &full_bar[st], once);
        if (BRAKET) bulk_g2s_hint(sb + L.off_bras, bras + (size_t)r0 * R, vbytes, &full_bar[st], once);
        if (gather && ell_n) {
          bulk_g2s_hint(sb + L.off_col, ecol + e0, ell_n * 4u, &full_bar[st], once);
          bulk_g2s_hint(sb + L.off_val, eval + (size_t)e0 * HS, ell_n * (uint32_t)(sizeof(F) * HS), &full_bar[st], once);
        }
        bulk_g2s(sb + L.off_diag, diag + (size_t)r0 * HS, dbytes, &full_bar[st]);
        ++issued;
      }
      // wait for the copies still in flight before leaving (bounded): the
      // consumers may have stopped early, and the CTA must not retire while a
      // bulk copy still writes its shared memory
      (void)ok;
      for (int32_t k = issued - STAGES < 0 ? 0 : issued - STAGES; k < issued; ++k)
        if (!mbar_wait_bounded(&full_bar[k % STAGES], (uint32_t)(k / STAGES) & 1u)) atomicOr(err, kErrDrain);
    }
    // producer warp contributes nothing to the moments
    return;
  }

  // -------------------------------------------------------------- consumers
  const int sub = lane % LPR;
  F m0 = 0, m1 = 0;
  constexpr int ROWS_PER_PASS = RPW * kTmaConsumerWarps;
  for (int32_t k = 0; k < my_tiles; ++k) {
    const int st = k % STAGES;
    const uint32_t ph = (uint32_t)(k / STAGES) & 1u;
    if (!mbar_wait_bounded(&full_bar[st], ph, wait_limit)) { atomicOr(err, kErrFullWait); break; }
    const unsigned char* sb = smem + (size_t)st * L.stage_bytes;
    const CT* sx = reinterpret_cast<const CT*>(sb + L.off_x);
    const CT* sp = reinterpret_cast<const CT*>(sb + L.off_prev);
    const CT* sbr = reinterpret_cast<const CT*>(sb + L.off_bras);
    const int32_t* scol = reinterpret_cast<const int32_t*>(sb + L.off_col);
    const F* sval = reinterpret_cast<const F*>(sb + L.off_val);
    const F* sdiag = reinterpret_cast<const F*>(sb + L.off_diag);
    const int32_t tile = tile_of(k);
    const int32_t r0 = tile * L.TR;
    const int32_t s0 = tile * slices_per_tile;
    const int32_t e0 = __ldg(soff + s0);
    const uint32_t tile_rows = (uint32_t)min(L.TR, n_slices * 32 - r0);   // rows staged in shared memory
    // neighbour row c: from the staged tile when it lies inside it, else from global (L2)
    auto nbr = [&](int32_t c) -> LaneV<F, VPL> {
      const uint32_t lc = (uint32_t)(c - r0);
      if (lc < tile_rows) return ld_smem<F, VPL>(sx + ((size_t)lc * LPR + sub) * VPL);
      return ld_ro<F, VPL>(x + ((int64_t)c * LPR + sub) * VPL);
    };
    for (int32_t lr = warp * RPW + lane / LPR; lr < L.TR; lr += ROWS_PER_PASS) {
      // rows past n (slice padding) are skipped; n <= padded rows of this tile
      const int32_t r = r0 + lr;
      if (r >= n) continue;
      const int32_t lme = lr * LPR + sub;
      const LaneV<F, VPL> xs = ld_smem<F, VPL>(sx + (size_t)lme * VPL);
      LaneV<F, VPL> prev;
#pragma unroll
      for (int q = 0; q < VPL; ++q) { prev.re[q] = 0; prev.im[q] = 0; }
      if (!first) prev = ld_smem<F, VPL>(sp + (size_t)lme * VPL);
      LaneV<F, VPL> acc;
#pragma unroll
      for (int q = 0; q < VPL; ++q) { acc.re[q] = 0; acc.im[q] = 0; }
      if (gather) {
        HVal<F, CPLX_H>::load_smem(sdiag, lr).template fma<VPL>(xs, acc);
        const int32_t s = lr >> 5, l = lr & 31;
        const int32_t off = __ldg(soff + s0 + s) - e0;
        const int32_t w = (__ldg(soff + s0 + s + 1) - __ldg(soff + s0 + s)) >> 5;
        // all of a row's gathers in flight together: predicated groups of 4
        for (int kk = 0; kk < w; kk += 4) {
          int32_t c[4];
          HVal<F, CPLX_H> h[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const bool v = kk + u < w;
            c[u] = v ? scol[off + (kk + u) * 32 + l] : r;          // padding: own row (staged)
            h[u] = HVal<F, CPLX_H>::load_smem(sval, v ? off + (kk + u) * 32 + l : off + l);
            if (!v) h[u] = HVal<F, CPLX_H>::zero();
          }
          LaneV<F, VPL> xv[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) xv[u] = nbr(c[u]);
#pragma unroll
          for (int u = 0; u < 4; ++u) h[u].template fma<VPL>(xv[u], acc);
        }
      }
      finish_acc<F, VPL>(acc);
      LaneV<F, VPL> out;
#pragma unroll
      for (int q = 0; q < VPL; ++q) {
        const F two = first ? F(1) : F(2);
        out.re[q] = two * acc.re[q] - prev.re[q];
        out.im[q] = two * acc.im[q] - prev.im[q];
      }
      if constexpr (BRAKET) {
        const LaneV<F, VPL> b = ld_smem<F, VPL>(sbr + (size_t)lme * VPL);
#pragma unroll
        for (int q = 0; q < VPL; ++q) {
          m0 += b.re[q] * out.re[q] + b.im[q] * out.im[q];
          if (first) m1 += b.re[q] * xs.re[q] + b.im[q] * xs.im[q];
        }
      } else {
        // first step: <v_0|v_1> (prev is zero there); later: <v_s|v_{s-1}>
#pragma unroll
        for (int q = 0; q < VPL; ++q) {
          m0 += xs.re[q] * xs.re[q] + xs.im[q] * xs.im[q];
          m1 += first ? (xs.re[q] * out.re[q] + xs.im[q] * out.im[q])
                      : (xs.re[q] * prev.re[q] + xs.im[q] * prev.im[q]);
        }
      }
      if (store) st_v<F, VPL>(y + ((int64_t)r * LPR + sub) * VPL, out);
    }
    __syncwarp();
    if (lane == 0) mbar_arrive(&empty_bar[st]);
  }
  double d0 = (double)m0, d1 = (double)m1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    d0 += __shfl_xor_sync(0xffffffffu, d0, o);
    d1 += __shfl_xor_sync(0xffffffffu, d1, o);
  }
  if (lane == 0) { red[0][warp] = d0; red[1][warp] = d1; }
  // named barrier over the consumer warps only (the producer warp has left)
  asm volatile("bar.sync 1, %0;" ::"r"(kTmaConsumerWarps * 32) : "memory");
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int q = 0; q < kTmaConsumerWarps; ++q) { a += red[0][q]; b += red[1][q]; }
    part[blockIdx.x] = a;
    part[gridDim.x + blockIdx.x] = b;
  }
}

}  // namespace tbk
