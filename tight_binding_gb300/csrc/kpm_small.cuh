// kpm_small.cuh — whole Chebyshev recursion in one launch for small systems.
//
// A 4,096-site lattice with 8 vectors (the reference's CPU-sized case) moves
// 512 KB per step: each step of the one-pass kernel is a few microseconds of
// launch and tail, so the solve is launch-bound.  Here one CTA owns one random
// vector for the whole solve: v_n and v_{n-1} live in shared memory (the
// recursion writes v_{n+1} over v_{n-1} in place), H~ is read through the
// read-only path (L1/L2-resident), and a __syncthreads separates the steps.
// Every row is computed with the same operations in the same order as the
// one-pass kernel (diagonal first, then the ELL entries), so the vectors are
// bit-identical to it; only the moment sums are grouped differently (per-warp
// FP64 sums, then the CTA's warps in a fixed order, per step and vector).
//
// Partials: part[(step * 2 + slot) * nblk + vector], the layout the fixed-order
// reduction of the multi-launch path reads (one chunk).
#pragma once

namespace tbk {

constexpr int kSmallThreads = 1024;

template <typename F, bool CPLX_H, bool BRAKET>
__global__ void __launch_bounds__(kSmallThreads) kpm_small_kernel(
    int32_t n, int32_t n_pad, int32_t n_steps, int32_t Rp, const int32_t* __restrict__ soff,
    const int32_t* __restrict__ ecol, const F* __restrict__ eval, const F* __restrict__ diag,
    const typename C2<F>::T* __restrict__ kets, const typename C2<F>::T* __restrict__ bras,
    double* __restrict__ part, int32_t nblk) {
  using CT = typename C2<F>::T;
  extern __shared__ __align__(16) unsigned char small_smem[];
  CT* va = reinterpret_cast<CT*>(small_smem);
  CT* vb = va + n_pad;
  __shared__ double wsum[2][2][kSmallThreads / 32];
  const int32_t r = blockIdx.x;                 // the vector this CTA owns
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int32_t i = threadIdx.x; i < n_pad; i += blockDim.x) {
    CT z;
    z.x = F(0);
    z.y = F(0);
    va[i] = i < n ? kets[(int64_t)i * Rp + r] : z;
    vb[i] = z;
  }
  __syncthreads();
  for (int32_t s = 0; s < n_steps; ++s) {
    const bool first = s == 0;
    const bool last_dot = !BRAKET && s == n_steps - 1 && s > 0;   // dots only, no product
    const CT* x = (s & 1) ? vb : va;
    CT* y = (s & 1) ? va : vb;                  // v_{s-1} on entry, v_{s+1} on exit
    double m0 = 0.0, m1 = 0.0;
    for (int32_t i = threadIdx.x; i < n; i += blockDim.x) {
      LaneV<F, 1> xs, prev, acc, out;
      xs.re[0] = x[i].x;
      xs.im[0] = x[i].y;
      prev.re[0] = y[i].x;
      prev.im[0] = y[i].y;
      if (!last_dot) {
        acc.re[0] = F(0);
        acc.im[0] = F(0);
        HVal<F, CPLX_H>::load(diag, i).template fma<1>(xs, acc);
        const int32_t sl = i >> 5, l = i & 31;
        const int32_t off = soff[sl];
        const int32_t w = (soff[sl + 1] - off) >> 5;
        for (int32_t k = 0; k < w; ++k) {
          const int32_t c = __ldg(ecol + off + l + (int64_t)k * 32);
          LaneV<F, 1> xv;
          xv.re[0] = x[c].x;
          xv.im[0] = x[c].y;
          HVal<F, CPLX_H>::load(eval, off + l + (int64_t)k * 32).template fma<1>(xv, acc);
        }
        if (first) {
          out = acc;
        } else {
          out.re[0] = F(2) * acc.re[0] - prev.re[0];
          out.im[0] = F(2) * acc.im[0] - prev.im[0];
        }
      } else {
        out = prev;
      }
      if constexpr (BRAKET) {
        const CT b = bras[(int64_t)i * Rp + r];
        m0 += static_cast<double>(b.x * out.re[0] + b.y * out.im[0]);
        if (first) m1 += static_cast<double>(b.x * xs.re[0] + b.y * xs.im[0]);
      } else {
        m0 += static_cast<double>(xs.re[0] * xs.re[0] + xs.im[0] * xs.im[0]);
        if (first) m1 += static_cast<double>(xs.re[0] * out.re[0] + xs.im[0] * out.im[0]);
        else m1 += static_cast<double>(xs.re[0] * prev.re[0] + xs.im[0] * prev.im[0]);
      }
      if (!last_dot) {
        CT o;
        o.x = out.re[0];
        o.y = out.im[0];
        y[i] = o;
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      m0 += __shfl_xor_sync(0xffffffffu, m0, o);
      m1 += __shfl_xor_sync(0xffffffffu, m1, o);
    }
    if (lane == 0) {
      wsum[s & 1][0][warp] = m0;
      wsum[s & 1][1][warp] = m1;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
        a += wsum[s & 1][0][q];
        b += wsum[s & 1][1][q];
      }
      part[((int64_t)s * 2 + 0) * nblk + r] = a;
      part[((int64_t)s * 2 + 1) * nblk + r] = b;
    }
  }
}

}  // namespace tbk
