// kpm_device.cuh — device helpers shared by the Chebyshev recursion kernels
// (kpm.cu, serving.cu): complex lane slices moved as one 64/128-bit access,
// Hamiltonian values (real or complex), L2 bulk prefetch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace tbk {

template <typename F> struct C2;
template <> struct C2<float> { using T = float2; };
template <> struct C2<double> { using T = double2; };

// Lane slice of a site's R vectors: VPL complex values moved as one access.
template <typename F, int VPL>
struct LaneV {
  F re[VPL], im[VPL];
};

template <typename F, int VPL>
__device__ __forceinline__ LaneV<F, VPL> ld_ro(const typename C2<F>::T* p) {
  LaneV<F, VPL> o;
  if constexpr (sizeof(F) == 4 && VPL == 2) {
    float4 q = __ldg(reinterpret_cast<const float4*>(p));
    o.re[0] = q.x; o.im[0] = q.y; o.re[1] = q.z; o.im[1] = q.w;
  } else {
    auto q = __ldg(p);
    o.re[0] = q.x; o.im[0] = q.y;
  }
  return o;
}
template <typename F, int VPL>
__device__ __forceinline__ LaneV<F, VPL> ld_stream(const typename C2<F>::T* p) {
  LaneV<F, VPL> o;
  if constexpr (sizeof(F) == 4 && VPL == 2) {
    float4 q = __ldcs(reinterpret_cast<const float4*>(p));
    o.re[0] = q.x; o.im[0] = q.y; o.re[1] = q.z; o.im[1] = q.w;
  } else {
    auto q = __ldcs(p);
    o.re[0] = q.x; o.im[0] = q.y;
  }
  return o;
}
template <typename F, int VPL>
__device__ __forceinline__ void st_v(typename C2<F>::T* p, const LaneV<F, VPL>& v) {
  if constexpr (sizeof(F) == 4 && VPL == 2) {
    *reinterpret_cast<float4*>(p) = make_float4(v.re[0], v.im[0], v.re[1], v.im[1]);
  } else {
    typename C2<F>::T q;
    q.x = v.re[0]; q.y = v.im[0];
    *p = q;
  }
}

template <typename F, int VPL>
__device__ __forceinline__ LaneV<F, VPL> ld_smem(const typename C2<F>::T* p) {
  LaneV<F, VPL> o;
  if constexpr (sizeof(F) == 4 && VPL == 2) {
    float4 q = *reinterpret_cast<const float4*>(p);
    o.re[0] = q.x; o.im[0] = q.y; o.re[1] = q.z; o.im[1] = q.w;
  } else {
    auto q = *p;
    o.re[0] = q.x; o.im[0] = q.y;
  }
  return o;
}

template <typename F, bool CPLX_H>
struct HVal;
template <typename F>
struct HVal<F, false> {
  F v;
  __device__ __forceinline__ static HVal load(const F* p, int64_t o) { return HVal{__ldg(p + o)}; }
  __device__ __forceinline__ static HVal load_smem(const F* p, int32_t o) { return HVal{p[o]}; }
  __device__ __forceinline__ static HVal zero() { return HVal{F(0)}; }
  template <int VPL>
  __device__ __forceinline__ void fma(const LaneV<F, VPL>& x, LaneV<F, VPL>& acc) const {
#pragma unroll
    for (int q = 0; q < VPL; ++q) { acc.re[q] = fma_(v, x.re[q], acc.re[q]); acc.im[q] = fma_(v, x.im[q], acc.im[q]); }
  }
  __device__ __forceinline__ static F fma_(F a, F b, F c) { return a * b + c; }
};
template <typename F>
struct HVal<F, true> {
  F r, i;
  __device__ __forceinline__ static HVal load(const F* p, int64_t o) {
    auto q = __ldg(reinterpret_cast<const typename C2<F>::T*>(p) + o);
    return HVal{q.x, q.y};
  }
  __device__ __forceinline__ static HVal load_smem(const F* p, int32_t o) {
    auto q = reinterpret_cast<const typename C2<F>::T*>(p)[o];
    return HVal{q.x, q.y};
  }
  __device__ __forceinline__ static HVal zero() { return HVal{F(0), F(0)}; }
  template <int VPL>
  __device__ __forceinline__ void fma(const LaneV<F, VPL>& x, LaneV<F, VPL>& acc) const {
#pragma unroll
    for (int q = 0; q < VPL; ++q) {
      acc.re[q] = r * x.re[q] + acc.re[q];
      acc.re[q] = -i * x.im[q] + acc.re[q];
      acc.im[q] = r * x.im[q] + acc.im[q];
      acc.im[q] = i * x.re[q] + acc.im[q];
    }
  }
};

template <typename F> struct VecW { static constexpr int max_vpl = (sizeof(F) == 4) ? 2 : 1; };

// Asynchronous bulk prefetch of [src, src+bytes) into L2 (no shared memory, no
// completion to wait for); bytes % 16 == 0 and src 16-byte aligned.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

}  // namespace tbk
