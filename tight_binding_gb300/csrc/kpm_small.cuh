// kpm_small.cuh — whole Chebyshev recursion in one launch for small systems.
//
// A 4,096-site lattice with 8 vectors (the reference's CPU-sized case) moves
// 512 KB per step: each step of the one-pass kernel is a few microseconds of
// launch, gather latency and tail, so the solve is latency-bound.  Here one
// thread-block cluster owns one random vector for the whole solve.  The
// cluster's CTAs split the rows (rpc rows each, a power of two and a multiple
// of the 32-row ELL slices); each CTA keeps its rows of v_n and v_{n-1} and its
// slice of H~ (ELL columns, values, diagonal) in shared memory, reads
// neighbours owned by other CTAs through distributed shared memory, writes
// v_{n+1} over its v_{n-1} in place, and one cluster barrier separates the
// steps.  Nothing goes to DRAM between steps except two FP64 partials per CTA.
// Every row is computed with the same operations in the same order as the
// one-pass kernel (diagonal first, then the ELL entries), so the vectors take
// the same values; only the moment sums are grouped differently.
//
// Partials: part[(step * 2 + slot) * nblk + CTA], the layout the fixed-order
// reduction of the multi-launch path reads (one chunk).
//
// Opt-in (TBK_FLAG_PERSISTENT) where kpm_cta_kernel below does not apply.
// Measured on the 4,096-site, 8-vector case
// (M = 256): 0.84 ms FP64 and 0.57 ms complex64 per solve, against 0.71 ms and
// 0.58 ms for the per-step kernels replayed as a CUDA graph.  The steps stall
// on distributed-shared-memory reads and the cluster barrier (short-scoreboard
// and barrier stalls dominate), and FP64 work on 64 SMs meets GB300's slow
// FP64 pipe.
#pragma once
#include <cooperative_groups.h>

namespace tbk {

constexpr int kClusterMax = 8;          // portable cluster size
constexpr int kSmallThreadsMax = 1024;

// shared-memory layout of one CTA (bytes), shared by host and device
struct SmallLayout {
  int32_t rpc, lg_rpc, cs, threads;     // rows per CTA (2^lg_rpc), cluster size, threads per CTA
  int32_t max_ne;                       // largest ELL entry count of a CTA's slices
  int32_t vb;                           // bytes of one matrix value (F, or 2 F for complex H)
  int32_t csz;                          // bytes of one complex vector element
  __host__ __device__ int32_t off_x() const { return 0; }
  __host__ __device__ int32_t off_diag() const { return 2 * rpc * csz; }
  __host__ __device__ int32_t off_soff() const { return off_diag() + rpc * vb; }
  __host__ __device__ int32_t off_cols() const { return off_soff() + ((rpc / 32 + 1) * 4 + 15) / 16 * 16; }
  __host__ __device__ int32_t off_vals() const { return off_cols() + (max_ne * 4 + 15) / 16 * 16; }
  __host__ __device__ int32_t bytes() const { return off_vals() + (max_ne * vb + 15) / 16 * 16; }
};

template <typename F, bool CPLX_H, bool BRAKET>
__global__ void __launch_bounds__(kSmallThreadsMax) kpm_cluster_kernel(
    int32_t n, int32_t n_slices, int32_t n_steps, int32_t Rp, SmallLayout L, const int32_t* __restrict__ soff,
    const int32_t* __restrict__ ecol, const F* __restrict__ eval, const F* __restrict__ diag,
    const typename C2<F>::T* __restrict__ kets, const typename C2<F>::T* __restrict__ bras,
    double* __restrict__ part) {
  namespace cg = cooperative_groups;
  using CT = typename C2<F>::T;
  constexpr int VW = CPLX_H ? 2 : 1;    // F values per matrix value
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ double wsum[2][2][kSmallThreadsMax / 32];
  cg::cluster_group cl = cg::this_cluster();
  const int q = (int)cl.block_rank();
  const int32_t vec = blockIdx.x / L.cs;             // the random vector this cluster owns
  const int32_t row0 = q * L.rpc;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  CT* xa = reinterpret_cast<CT*>(sm + L.off_x());
  CT* xb = xa + L.rpc;
  F* dg = reinterpret_cast<F*>(sm + L.off_diag());
  int32_t* so = reinterpret_cast<int32_t*>(sm + L.off_soff());
  int32_t* cols = reinterpret_cast<int32_t*>(sm + L.off_cols());
  F* vals = reinterpret_cast<F*>(sm + L.off_vals());
  // this CTA's slices of H~ and rows of the kets
  const int32_t sl0 = min(row0 >> 5, n_slices);
  const int32_t nsl = L.rpc >> 5;
  const int32_t base = soff[sl0];
  const int32_t ne = soff[min(sl0 + nsl, n_slices)] - base;
  for (int32_t j = threadIdx.x; j <= nsl; j += blockDim.x) so[j] = soff[min(sl0 + j, n_slices)] - base;
  for (int32_t e = threadIdx.x; e < ne; e += blockDim.x) {
    cols[e] = ecol[base + e];
#pragma unroll
    for (int u = 0; u < VW; ++u) {
      if constexpr (is_dd<F>) {
        const float2 p = __ldg(reinterpret_cast<const float2*>(eval) + ((int64_t)base + e) * VW + u);
        vals[e * VW + u] = dd(p.x, p.y);
      } else {
        vals[e * VW + u] = __ldg(eval + ((int64_t)base + e) * VW + u);
      }
    }
  }
  for (int32_t li = threadIdx.x; li < L.rpc; li += blockDim.x) {
    const int32_t i = row0 + li;
    CT z;
    z.x = F(0);
    z.y = F(0);
#pragma unroll
    for (int u = 0; u < VW; ++u) {
      if (i < n) {
        if constexpr (is_dd<F>) {
          const float2 p = __ldg(reinterpret_cast<const float2*>(diag) + (int64_t)i * VW + u);
          dg[li * VW + u] = dd(p.x, p.y);
        } else {
          dg[li * VW + u] = __ldg(diag + (int64_t)i * VW + u);
        }
      } else {
        dg[li * VW + u] = F(0);
      }
    }
    xa[li] = i < n ? kets[(int64_t)i * Rp + vec] : z;
    xb[li] = z;
  }
  cl.sync();
  for (int32_t s = 0; s < n_steps; ++s) {
    const bool first = s == 0;
    const bool last_dot = !BRAKET && s == n_steps - 1 && s > 0;   // dots only, no product
    CT* x = (s & 1) ? xb : xa;
    CT* y = (s & 1) ? xa : xb;                  // v_{s-1} on entry, v_{s+1} on exit
    double m0 = 0.0, m1 = 0.0;
    for (int32_t li = threadIdx.x; li < L.rpc; li += blockDim.x) {
      if (row0 + li >= n) continue;
      LaneV<F, 1> xs, prev, acc, out;
      xs.re[0] = x[li].x;
      xs.im[0] = x[li].y;
      prev.re[0] = y[li].x;
      prev.im[0] = y[li].y;
      if (!last_dot) {
        acc.re[0] = F(0);
        acc.im[0] = F(0);
        HVal<F, CPLX_H>::load_smem(dg, li).template fma<1>(xs, acc);
        const int32_t l = li & 31;
        const int32_t off = so[li >> 5];
        const int32_t w = (so[(li >> 5) + 1] - off) >> 5;
        // predicated groups of 4 (as the one-pass kernel): a row's remote
        // neighbour reads are in flight together
        for (int32_t k = 0; k < w; k += 4) {
          int32_t c[4];
          HVal<F, CPLX_H> h[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const bool v = k + u < w;
            const int32_t e = off + l + (k + u) * 32;
            c[u] = v ? cols[e] : row0 + li;                          // padding: own row
            h[u] = v ? HVal<F, CPLX_H>::load_smem(vals, e) : HVal<F, CPLX_H>::zero();
          }
          LaneV<F, 1> xv[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const CT* xr = cl.map_shared_rank(x, (unsigned)(c[u] >> L.lg_rpc));
            const CT v = xr[c[u] & (L.rpc - 1)];
            xv[u].re[0] = v.x;
            xv[u].im[0] = v.y;
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) h[u].template fma<1>(xv[u], acc);
        }
        finish_acc<F, 1>(acc);
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
        const CT b = bras[(int64_t)(row0 + li) * Rp + vec];
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
        y[li] = o;
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
    cl.sync();                                   // step done everywhere: y becomes the next x
    if (threadIdx.x == 0) {
      double a = 0.0, b = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
        a += wsum[s & 1][0][w];
        b += wsum[s & 1][1][w];
      }
      part[((int64_t)s * 2 + 0) * gridDim.x + blockIdx.x] = a;
      part[((int64_t)s * 2 + 1) * gridDim.x + blockIdx.x] = b;
    }
  }
}

// One CTA per random complex64 vector for matrices with row classes
// (kpm_step.cuh's class form): the whole recursion of a vector in one SM's
// shared memory — v_n and v_{n-1} of every row, the diagonal, each row's class
// byte and the class table (84 KB for 4,096 sites) — with one CTA barrier
// between steps and no other SM involved.  Rows are computed as the step
// kernel's class form computes them (diagonal first, then the class's entries
// in order, whole groups of 4 over the zero-padded table), so the vectors
// take the same values; the moment sums are grouped per vector, in
// double-float trees on the FP32 pipe (one SM's FP64 rate would set the step
// time), with FP64 only for the step's result.  Templated on the vector
// precision, used for complex64.
struct CtaLayout {
  int32_t n, n_cls, w, csz, vb;           // rows, classes, entries per class, vector / matrix element bytes
  __host__ __device__ static int32_t up16(int32_t b) { return (b + 15) / 16 * 16; }
  __host__ __device__ int32_t off_x() const { return 0; }
  __host__ __device__ int32_t off_diag() const { return up16(2 * n * csz); }
  __host__ __device__ int32_t off_tval() const { return up16(off_diag() + n * vb); }
  __host__ __device__ int32_t off_toff() const { return up16(off_tval() + n_cls * w * vb); }
  __host__ __device__ int32_t off_tcnt() const { return off_toff() + n_cls * w * 4; }
  __host__ __device__ int32_t off_cls() const { return up16(off_tcnt() + n_cls * 4); }
  __host__ __device__ int32_t bytes() const { return up16(off_cls() + n); }
};
template <typename F>
__host__ __device__ constexpr int cta_threads() { return sizeof(F) == 4 ? 1024 : 512; }
__device__ __forceinline__ dd dd_of(float v) { return dd(v, 0.f); }
__device__ __forceinline__ dd dd_of(dd v) { return dd_norm(v); }   // TwoSum: an unnormalised Dot2 pair

template <typename F, bool CPLX_H, bool BRAKET>
__global__ void __launch_bounds__(cta_threads<F>()) kpm_cta_kernel(
    int32_t n_steps, int32_t Rp, CtaLayout L, const ClassTab ct, const F* __restrict__ diag,
    const typename C2<F>::T* __restrict__ kets, const typename C2<F>::T* __restrict__ bras,
    double* __restrict__ part) {
  using CT = typename C2<F>::T;
  constexpr int VW = CPLX_H ? 2 : 1;     // F values per matrix value
  constexpr int NT = cta_threads<F>();
  extern __shared__ __align__(16) unsigned char sm[];
  __shared__ dd wsum[2][2][NT / 32];
  const int32_t n = L.n, vec = blockIdx.x;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  CT* xa = reinterpret_cast<CT*>(sm + L.off_x());
  CT* xb = xa + n;
  F* dg = reinterpret_cast<F*>(sm + L.off_diag());
  F* tv = reinterpret_cast<F*>(sm + L.off_tval());
  int32_t* to = reinterpret_cast<int32_t*>(sm + L.off_toff());
  int32_t* tc = reinterpret_cast<int32_t*>(sm + L.off_tcnt());
  uint8_t* cl = sm + L.off_cls();
  {  // table, diagonal and class bytes as 4-byte words / bytes; the kets' column of this vector
    const int32_t ne = L.n_cls * L.w;
    const int32_t vw = ne * VW * (int32_t)sizeof(F) / 4, dw = n * VW * (int32_t)sizeof(F) / 4;
    const uint32_t* gv = static_cast<const uint32_t*>(ct.val);
    const uint32_t* gd = reinterpret_cast<const uint32_t*>(diag);
    for (int32_t q = threadIdx.x; q < vw; q += NT) reinterpret_cast<uint32_t*>(tv)[q] = __ldg(gv + q);
    for (int32_t q = threadIdx.x; q < ne; q += NT) to[q] = __ldg(ct.off + q);
    for (int32_t q = threadIdx.x; q < L.n_cls; q += NT) tc[q] = __ldg(ct.cnt + q);
    for (int32_t q = threadIdx.x; q < dw; q += NT) reinterpret_cast<uint32_t*>(dg)[q] = __ldg(gd + q);
    for (int32_t q = threadIdx.x; q < n; q += NT) {
      cl[q] = __ldg(ct.cls + q);
      xa[q] = kets[(int64_t)q * Rp + vec];
      CT z;
      z.x = F(0);
      z.y = F(0);
      xb[q] = z;
    }
  }
  __syncthreads();
  for (int32_t s = 0; s < n_steps; ++s) {
    const bool first = s == 0;
    const bool last_dot = !BRAKET && s == n_steps - 1 && s > 0;   // dots only, no product
    const CT* x = (s & 1) ? xb : xa;
    CT* y = (s & 1) ? xa : xb;                  // v_{s-1} on entry, v_{s+1} on exit
    F m0 = 0, m1 = 0;                           // this thread's rows (FP32 pipe; Dot2 for double-float)
    for (int32_t r = threadIdx.x; r < n; r += NT) {
      LaneV<F, 1> xs, prev, out;
      xs.re[0] = x[r].x;
      xs.im[0] = x[r].y;
      prev.re[0] = y[r].x;
      prev.im[0] = y[r].y;
      if (!last_dot) {
        LaneV<F, 1> acc;
        acc.re[0] = F(0);
        acc.im[0] = F(0);
        HVal<F, CPLX_H>::load_smem(dg, r).template fma<1>(xs, acc);
        const int32_t c = cl[r];
        const int32_t cnt = tc[c], tb = c * L.w;
        for (int32_t k = 0; k < cnt; k += 4) {
          HVal<F, CPLX_H> h[4];
          LaneV<F, 1> xv[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            // rows are verified equal to their class: r + offset is the row's
            // column; the clamp only keeps a bad table inside the vector
            const int32_t col = min(max(r + to[tb + k + u], 0), n - 1);
            h[u] = HVal<F, CPLX_H>::load_smem(tv, tb + k + u);
            xv[u].re[0] = x[col].x;
            xv[u].im[0] = x[col].y;
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) h[u].template fma<1>(xv[u], acc);
        }
        finish_acc<F, 1>(acc);
        if (first) out = acc;
        else recur_out<F, 1>(acc, prev, out);
      } else {
        out = prev;
      }
      if constexpr (BRAKET) {
        const CT bv = bras[(int64_t)r * Rp + vec];
        LaneV<F, 1> b;
        b.re[0] = bv.x;
        b.im[0] = bv.y;
        dot_acc<F, 1>(b, out, m0);
        if (first) dot_acc<F, 1>(b, xs, m1);
      } else {
        dot_acc<F, 1>(xs, xs, m0);
        if (first) dot_acc<F, 1>(xs, out, m1);
        else dot_acc<F, 1>(xs, prev, m1);
      }
      if (!last_dot) {
        CT o;
        o.x = out.re[0];
        o.y = out.im[0];
        y[r] = o;
      }
    }
    // sums of the vector: double-float trees on the FP32 pipe (GB300's FP64
    // rate on one SM would set the step time), FP64 only for the result
    dd a0 = dd_of(m0), a1 = dd_of(m1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      a0 = a0 + dd(__shfl_xor_sync(0xffffffffu, a0.hi, o), __shfl_xor_sync(0xffffffffu, a0.lo, o));
      a1 = a1 + dd(__shfl_xor_sync(0xffffffffu, a1.hi, o), __shfl_xor_sync(0xffffffffu, a1.lo, o));
    }
    if (lane == 0) {
      wsum[s & 1][0][warp] = a0;
      wsum[s & 1][1][warp] = a1;
    }
    __syncthreads();                             // step done: y becomes the next x
    if (warp == 0) {
      dd b0 = lane < NT / 32 ? wsum[s & 1][0][lane] : dd(0.f, 0.f);
      dd b1 = lane < NT / 32 ? wsum[s & 1][1][lane] : dd(0.f, 0.f);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        b0 = b0 + dd(__shfl_xor_sync(0xffffffffu, b0.hi, o), __shfl_xor_sync(0xffffffffu, b0.lo, o));
        b1 = b1 + dd(__shfl_xor_sync(0xffffffffu, b1.hi, o), __shfl_xor_sync(0xffffffffu, b1.lo, o));
      }
      if (lane == 0) {
        part[((int64_t)s * 2 + 0) * gridDim.x + blockIdx.x] = (double)b0;
        part[((int64_t)s * 2 + 1) * gridDim.x + blockIdx.x] = (double)b1;
      }
    }
  }
}

}  // namespace tbk
