// kpm_fused.cuh — two doubling recursion steps per pass over memory.
//
// A pass reads v_s (block A) and v_{s-1} (block B) once and leaves v_{s+2} in
// A and v_{s+1} in B.  Phase 1 of tile t computes v_{s+1}[t] = 2 H v_s - v_{s-1}
// (in place in B) exactly as the one-pass step kernel.  Phase 2 of tile j,
// `lag` tiles behind, computes v_{s+2}[j] = 2 H v_{s+1} - v_s (in place in A)
// from rows that phase 1 wrote moments ago and that are still in L2.  DRAM
// traffic per two steps: 4 vector blocks + the matrix once, against 6 blocks +
// the matrix twice for two one-pass steps.
//
// Work unit: a task of `tpt` consecutive base tiles (one synchronisation per
// task).  Ordering.  Task t's phase 1 runs on CTA t % G in its iteration t / G; a CTA
// that finishes it counts one in wave_cnt[t / G] (release).  Phase 2 of tile j
// may run once every tile that j reads from B, and every tile that reads A[j]
// in phase 1, has finished phase 1: all such tiles are <= dep[j], so it waits
// (acquire, bounded) until the waves up to dep[j] / G are complete.  Tiles whose
// dependencies reach far ahead (periodic bonds that wrap around the vector) are
// deferred to the end of the pass, after every wave.  The grid is launched
// cooperatively, so every CTA is resident and the waits always end; a wait that
// exceeds its bound records an error instead (the host reports TBK_ERR_TIMEOUT).
// Loads of B in phase 1 bypass L1, so phase 2 may cache v_{s+1} in L1.
#pragma once

namespace tbk {

constexpr uint32_t kFuseWait = 1u << 22;

// dep[t] = max(t, tiles that tile t reads, tiles that read tile t); dep preset to t
__global__ void tile_dep_kernel(int32_t n, int32_t rpt, const int32_t* __restrict__ soff,
                                const int32_t* __restrict__ ecol, int32_t* __restrict__ dep) {
  const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int32_t t = r / rpt, s = r >> 5, l = r & 31;
  const int32_t off = soff[s], w = (soff[s + 1] - off) >> 5;
  int32_t m = t;
  for (int32_t k = 0; k < w; ++k) {
    const int32_t u = ecol[off + l + 32 * k] / rpt;
    m = max(m, u);
    if (u != t) atomicMax(&dep[u], t);
  }
  atomicMax(&dep[t], m);
}
__global__ void iota_kernel(int32_t n, int32_t* __restrict__ v) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = i;
}

__device__ __forceinline__ uint32_t ld_acquire_u32(const unsigned int* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// L2-only load (no L1 allocation) and L1-allocating coherent load
template <int VPL>
__device__ __forceinline__ LaneV<float, VPL> ld_cg(const float2* p) {
  LaneV<float, VPL> o;
  if constexpr (VPL == 2) {
    const float4 q = __ldcg(reinterpret_cast<const float4*>(p));
    o.re[0] = q.x; o.im[0] = q.y; o.re[1] = q.z; o.im[1] = q.w;
  } else {
    const float2 q = __ldcg(p);
    o.re[0] = q.x; o.im[0] = q.y;
  }
  return o;
}
template <int VPL>
__device__ __forceinline__ LaneV<float, VPL> ld_ca(const float2* p) {
  LaneV<float, VPL> o;
  if constexpr (VPL == 2) {
    const float4 q = __ldca(reinterpret_cast<const float4*>(p));
    o.re[0] = q.x; o.im[0] = q.y; o.re[1] = q.z; o.im[1] = q.w;
  } else {
    const float2 q = __ldca(p);
    o.re[0] = q.x; o.im[0] = q.y;
  }
  return o;
}

// One row-slice of one recursion step: out = 2 H x - prev (first: H x), the
// doubling partial sums, optional store.
//   phase 1 (P2 false): x = v_s (read-only in effect: every read of a row of A
//     precedes its overwrite), prev = v_{s-1} read with ld.cg, so that no L1
//     ever holds a line of B during the pass;
//   phase 2 (P2 true): x = v_{s+1} and its neighbours, written by other CTAs in
//     this launch before the acquire, read with L1-allocating coherent loads
//     (no L1 can hold an older copy of those lines).
template <int R, bool CPLX_H, bool P2>
__device__ __forceinline__ void fused_rows(int32_t tile, int32_t n, const int32_t* __restrict__ soff,
                                           const int32_t* __restrict__ ecol, const float* __restrict__ eval,
                                           const float* __restrict__ diag, const float2* x, const float2* pv,
                                           float2* y, bool first, bool gather, float& m0, float& m1) {
  constexpr int VPL = (R >= 2) ? 2 : 1;
  constexpr int LPR = R / VPL;
  constexpr int RPW = 32 / LPR;
  constexpr int RPT = RPW * kStepWarps;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, sub = lane % LPR;
  const int32_t r = tile * RPT + warp * RPW + lane / LPR;
  if (r >= n) return;
  const int64_t me = (int64_t)r * LPR + sub;
  const LaneV<float, VPL> xs = P2 ? ld_ca<VPL>(x + me * VPL) : ld_ro<float, VPL>(x + me * VPL);
  LaneV<float, VPL> prev;
  if (!first) {
    prev = P2 ? ld_stream<float, VPL>(pv + me * VPL) : ld_cg<VPL>(pv + me * VPL);
  } else {
#pragma unroll
    for (int q = 0; q < VPL; ++q) { prev.re[q] = 0.f; prev.im[q] = 0.f; }
  }
  LaneV<float, VPL> acc;
#pragma unroll
  for (int q = 0; q < VPL; ++q) { acc.re[q] = 0.f; acc.im[q] = 0.f; }
  if (gather) {
    HVal<float, CPLX_H>::load(diag, r).template fma<VPL>(xs, acc);
    const int32_t s = r >> 5, l = r & 31;
    const int32_t off = soff[s];
    const int32_t w = (soff[s + 1] - off) >> 5;
    const int32_t* cp = ecol + off + l;
    for (int k = 0; k < w; k += 4) {
      int32_t c[4];
      HVal<float, CPLX_H> h[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const bool v = k + u < w;
        c[u] = v ? __ldg(cp + (k + u) * 32) : r;
        h[u] = v ? HVal<float, CPLX_H>::load(eval, off + l + (int64_t)(k + u) * 32) : HVal<float, CPLX_H>::zero();
      }
      LaneV<float, VPL> xv[4];
#pragma unroll
      for (int u = 0; u < 4; ++u)
        xv[u] = P2 ? ld_ca<VPL>(x + ((int64_t)c[u] * LPR + sub) * VPL)
                   : ld_ro<float, VPL>(x + ((int64_t)c[u] * LPR + sub) * VPL);
#pragma unroll
      for (int u = 0; u < 4; ++u) h[u].template fma<VPL>(xv[u], acc);
    }
  }
  LaneV<float, VPL> out;
#pragma unroll
  for (int q = 0; q < VPL; ++q) {
    if (first) { out.re[q] = acc.re[q]; out.im[q] = acc.im[q]; }
    else { out.re[q] = 2.f * acc.re[q] - prev.re[q]; out.im[q] = 2.f * acc.im[q] - prev.im[q]; }
  }
#pragma unroll
  for (int q = 0; q < VPL; ++q) {
    m0 += xs.re[q] * xs.re[q] + xs.im[q] * xs.im[q];
    if (first) m1 += xs.re[q] * out.re[q] + xs.im[q] * out.im[q];
    else m1 += xs.re[q] * prev.re[q] + xs.im[q] * prev.im[q];
  }
  if (gather) st_v<float, VPL>(y + me * VPL, out);
}

// Waits (thread 0) until waves 0 .. last are complete; the result is broadcast.
__device__ __forceinline__ bool fused_wait_waves(int32_t last, int32_t& seen, int32_t n_tiles,
                                                 const unsigned int* wave_cnt, int* err, int* ok_sh) {
  if (threadIdx.x == 0) {
    int ok = 1;
    uint32_t spins = 0;
    const int32_t G = (int32_t)gridDim.x;
    while (seen <= last) {
      const uint32_t target = (uint32_t)min(G, n_tiles - seen * G);
      if (ld_acquire_u32(wave_cnt + seen) >= target) { ++seen; continue; }
      if (++spins > kFuseWait) { atomicOr(err, 2); ok = 0; break; }
      __nanosleep(64);
    }
    *ok_sh = ok;
  }
  __syncthreads();
  return *ok_sh != 0;
}

template <int R, bool CPLX_H>
__global__ void __launch_bounds__(kStepThreads) kpm_fused2_kernel(
    int32_t n, int32_t n_tiles, int32_t tpt, const int32_t* __restrict__ soff, const int32_t* __restrict__ ecol,
    const float* __restrict__ eval, const float* __restrict__ diag, float2* A, float2* B,
    const int32_t* __restrict__ dep, const uint8_t* __restrict__ is_def, const int32_t* __restrict__ deferred,
    int32_t n_def, int32_t lag, unsigned int* wave_cnt, double* __restrict__ part1, double* __restrict__ part2,
    int first, int dot2, int* err) {
  constexpr int VPL = (R >= 2) ? 2 : 1;
  constexpr int LPR = R / VPL;
  static_assert(LPR >= 1 && LPR <= 32 && (32 % LPR) == 0, "R out of range");
  __shared__ int ok_sh;
  __shared__ double sh[4][kStepWarps];
  const int32_t G = (int32_t)gridDim.x;
  const int32_t c = (int32_t)blockIdx.x;
  float a0 = 0.f, a1 = 0.f, b0 = 0.f, b1 = 0.f;       // step s, step s + 1 partials
  int32_t seen = 0;                                     // waves known complete (thread 0)
  const int32_t n_waves = (n_tiles + G - 1) / G;
  for (int32_t k = 0;; ++k) {
    const int32_t t = c + k * G;
    if (t >= n_tiles + lag) break;
    if (t < n_tiles) {
      // phase 1: v_{s+1} of the tpt base tiles of task t into B
      for (int32_t u = 0; u < tpt; ++u)
        fused_rows<R, CPLX_H, false>(t * tpt + u, n, soff, ecol, eval, diag, A, B, B, first != 0, true, a0, a1);
      __syncthreads();
      if (threadIdx.x == 0) {
        __threadfence();
        atomicAdd(wave_cnt + k, 1u);
      }
    }
    const int32_t j = t - lag;
    if (j >= 0 && j < n_tiles && !is_def[j]) {
      // phase 2: v_{s+2}[j] into A, once every tile that j touches is through phase 1
      if (fused_wait_waves(dep[j] / G, seen, n_tiles, wave_cnt, err, &ok_sh))
        for (int32_t u = 0; u < tpt; ++u)
          fused_rows<R, CPLX_H, true>(j * tpt + u, n, soff, ecol, eval, diag, B, A, A, false, dot2 == 0, b0, b1);
    }
  }
  // deferred tiles: after every wave
  if (n_def > 0 && fused_wait_waves(n_waves - 1, seen, n_tiles, wave_cnt, err, &ok_sh)) {
    for (int32_t i = c; i < n_def; i += G)
      for (int32_t u = 0; u < tpt; ++u)
        fused_rows<R, CPLX_H, true>(deferred[i] * tpt + u, n, soff, ecol, eval, diag, B, A, A, false, dot2 == 0,
                                    b0, b1);
  }
  // per-CTA partials (FP64 above the thread)
  double d[4] = {(double)a0, (double)a1, (double)b0, (double)b1};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int q = 0; q < 4; ++q) d[q] += __shfl_xor_sync(0xffffffffu, d[q], o);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  __syncthreads();
  if (lane == 0)
#pragma unroll
    for (int q = 0; q < 4; ++q) sh[q][warp] = d[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int w = 0; w < kStepWarps; ++w)
#pragma unroll
      for (int q = 0; q < 4; ++q) s[q] += sh[q][w];
    part1[c] = s[0];
    part1[G + c] = s[1];
    part2[c] = s[2];
    part2[G + c] = s[3];
  }
}

}  // namespace tbk
