// kpm_device.cuh — device helpers shared by the Chebyshev recursion kernels
// (kpm.cu, serving.cu): complex lane slices moved as one 64/128-bit access,
// Hamiltonian values (real or complex), L2 bulk prefetch.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "tbk_internal.h"

namespace tbk {

// Double-float number: value = hi + lo (|lo| <= ulp(hi) / 2), about 48
// significant bits, computed on the FP32 pipe with error-free transformations
// (Knuth TwoSum, Dekker / FMA TwoProduct).  On GB300 the FP64 pipe is ~64x
// slower than FP32, so a recursion in this type runs at memory speed with
// FP64-class accuracy.  Every step uses the _rn intrinsics so that the compiler
// cannot contract a product and a sum into one FMA (which would break the
// error terms).
struct dd {
  float hi, lo;
  dd() = default;
  __host__ __device__ constexpr dd(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr dd(int v) : hi((float)v), lo(0.f) {}
  __device__ explicit dd(double v) {
    hi = __double2float_rn(v);
    lo = __double2float_rn(v - (double)hi);
  }
  __device__ explicit operator double() const { return (double)hi + (double)lo; }
};
__device__ __forceinline__ dd dd_fast_two_sum(float a, float b) {     // |a| >= |b|
  const float s = __fadd_rn(a, b);
  return dd(s, __fsub_rn(b, __fsub_rn(s, a)));
}
__device__ __forceinline__ dd operator+(dd a, dd b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float bb = __fsub_rn(s, a.hi);
  float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
  e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  return dd_fast_two_sum(s, e);
}
__device__ __forceinline__ dd operator-(dd a) { return dd(-a.hi, -a.lo); }
__device__ __forceinline__ dd operator-(dd a, dd b) { return a + (-b); }
__device__ __forceinline__ dd operator*(dd a, dd b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return dd_fast_two_sum(p, e);
}
__device__ __forceinline__ dd& operator+=(dd& a, dd b) { a = a + b; return a; }
// acc += h x for a row sum, accumulated unnormalised in the manner of Dot2
// (Ogita, Rump & Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput.
// 26(6), 2005): the product's leading term and its exact FMA error, the two
// cross terms, and the exact TwoSum error of the running sum all go into acc.lo
// with plain adds; acc.hi carries the running FP32 sum.  The dependency chain
// between entries is one add; dd_norm restores a normalised pair afterwards.
__device__ __forceinline__ void dd_fma_acc(dd h, dd x, dd& acc) {
  const float p = __fmul_rn(h.hi, x.hi);
  float e = __fmaf_rn(h.hi, x.hi, -p);
  e = __fmaf_rn(h.hi, x.lo, e);
  e = __fmaf_rn(h.lo, x.hi, e);
  const float s = __fadd_rn(acc.hi, p);
  const float bb = __fsub_rn(s, acc.hi);
  const float t = __fadd_rn(__fsub_rn(acc.hi, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  acc.hi = s;
  acc.lo = __fadd_rn(acc.lo, __fadd_rn(t, e));
}
// The same accumulation for two values that share the factor h (the real and
// imaginary parts of one vector element): Blackwell's packed f32x2 arithmetic
// does both halves in one instruction, each half rounded exactly as the scalar
// dd_fma_acc rounds it (the product is formed negated, np = (-h) x, so that
// e = fma(h, x, np) and s = acc - np need no separate negation; rounding is
// symmetric in sign, so every intermediate equals its scalar counterpart).
// hh / nhh / hl: (h.hi, h.hi), (-h.hi, -h.hi), (h.lo, h.lo) for a shared
// factor, or per-half factors for the cross terms of a complex product.
__device__ __forceinline__ uint64_t f2_pack(float a, float b) {
  uint64_t r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ void f2_unpack(uint64_t r, float& a, float& b) {
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
  uint64_t r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
  return r;
}
__device__ __forceinline__ uint64_t f2_fma(uint64_t a, uint64_t b, uint64_t c) {
  uint64_t r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
  return r;
}
__device__ __forceinline__ void dd_fma_acc2(uint64_t hh, uint64_t nhh, uint64_t hl, dd xa, dd xb, dd& acca,
                                            dd& accb) {
  const uint64_t xh = f2_pack(xa.hi, xb.hi), xl = f2_pack(xa.lo, xb.lo);
  const uint64_t ah = f2_pack(acca.hi, accb.hi), al = f2_pack(acca.lo, accb.lo);
  const uint64_t np = f2_mul(nhh, xh);                    // -p
  uint64_t e = f2_fma(hh, xh, np);                        // exact error of p
  e = f2_fma(hh, xl, e);
  e = f2_fma(hl, xh, e);
  const uint64_t s = f2_sub(ah, np);                      // acc.hi + p
  const uint64_t bb = f2_sub(s, ah);
  const uint64_t t = f2_sub(f2_sub(ah, f2_sub(s, bb)), f2_add(np, bb));   // TwoSum error: (ah - (s - bb)) + (p - bb)
  const uint64_t lo = f2_add(al, f2_add(t, e));
  f2_unpack(s, acca.hi, accb.hi);
  f2_unpack(lo, acca.lo, accb.lo);
}
__device__ __forceinline__ dd dd_norm(dd a) {            // TwoSum(hi, lo)
  const float s = __fadd_rn(a.hi, a.lo);
  const float bb = __fsub_rn(s, a.hi);
  return dd(s, __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(a.lo, bb)));
}
struct __align__(16) dd2 {
  dd x, y;
};
// round to FP32 once
__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(double v) { return __double2float_rn(v); }
__device__ __forceinline__ float to_f32(dd v) { return __fadd_rn(v.hi, v.lo); }

template <typename F> struct C2;
template <> struct C2<float> { using T = float2; };
template <> struct C2<double> { using T = double2; };
template <> struct C2<dd> { using T = dd2; };
template <typename F> constexpr bool is_dd = false;
template <> constexpr bool is_dd<dd> = true;

// Lane slice of a site's R vectors: VPL complex values moved as one access.
template <typename F, int VPL>
struct LaneV {
  F re[VPL], im[VPL];
};

template <typename F, int VPL>
__device__ __forceinline__ LaneV<F, VPL> ld_ro(const typename C2<F>::T* p) {
  LaneV<F, VPL> o;
  if constexpr (is_dd<F>) {
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      float4 q = __ldg(reinterpret_cast<const float4*>(p) + v);
      o.re[v] = dd(q.x, q.y); o.im[v] = dd(q.z, q.w);
    }
  } else if constexpr (sizeof(F) == 4 && VPL == 2) {
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
  if constexpr (is_dd<F>) {
#pragma unroll
    for (int v = 0; v < VPL; ++v) {
      float4 q = __ldcs(reinterpret_cast<const float4*>(p) + v);
      o.re[v] = dd(q.x, q.y); o.im[v] = dd(q.z, q.w);
    }
  } else if constexpr (sizeof(F) == 4 && VPL == 2) {
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
  if constexpr (is_dd<F>) {
#pragma unroll
    for (int u = 0; u < VPL; ++u)
      reinterpret_cast<float4*>(p)[u] = make_float4(v.re[u].hi, v.re[u].lo, v.im[u].hi, v.im[u].lo);
  } else if constexpr (sizeof(F) == 4 && VPL == 2) {
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
  __device__ __forceinline__ static HVal load(const F* p, int64_t o) {
    if constexpr (is_dd<F>) {
      const float2 q = __ldg(reinterpret_cast<const float2*>(p) + o);
      return HVal{dd(q.x, q.y)};
    } else {
      return HVal{__ldg(p + o)};
    }
  }
  __device__ __forceinline__ static HVal load_smem(const F* p, int32_t o) { return HVal{p[o]}; }
  __device__ __forceinline__ static HVal zero() { return HVal{F(0)}; }
  template <int VPL>
  __device__ __forceinline__ void fma(const LaneV<F, VPL>& x, LaneV<F, VPL>& acc) const {
    if constexpr (is_dd<F>) {
      // real and imaginary parts share v: one packed accumulation per element
      const uint64_t hh = f2_pack(v.hi, v.hi), nhh = f2_pack(-v.hi, -v.hi), hl = f2_pack(v.lo, v.lo);
#pragma unroll
      for (int q = 0; q < VPL; ++q) dd_fma_acc2(hh, nhh, hl, x.re[q], x.im[q], acc.re[q], acc.im[q]);
    } else {
#pragma unroll
      for (int q = 0; q < VPL; ++q) {
        acc.re[q] = fma_(v, x.re[q], acc.re[q]);
        acc.im[q] = fma_(v, x.im[q], acc.im[q]);
      }
    }
  }
  __device__ __forceinline__ static F fma_(F a, F b, F c) { return a * b + c; }
};
template <typename F>
struct HVal<F, true> {
  F r, i;
  __device__ __forceinline__ static HVal load(const F* p, int64_t o) {
    if constexpr (is_dd<F>) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(p) + o);
      return HVal{dd(q.x, q.y), dd(q.z, q.w)};
    } else {
      auto q = __ldg(reinterpret_cast<const typename C2<F>::T*>(p) + o);
      return HVal{q.x, q.y};
    }
  }
  __device__ __forceinline__ static HVal load_smem(const F* p, int32_t o) {
    auto q = reinterpret_cast<const typename C2<F>::T*>(p)[o];
    return HVal{q.x, q.y};
  }
  __device__ __forceinline__ static HVal zero() { return HVal{F(0), F(0)}; }
  template <int VPL>
  __device__ __forceinline__ void fma(const LaneV<F, VPL>& x, LaneV<F, VPL>& acc) const {
    if constexpr (is_dd<F>) {
      // (re, im) += r (x.re, x.im), then (re, im) += (-i x.im, i x.re): the
      // scalar order of both components, two packed accumulations
      const uint64_t rh = f2_pack(r.hi, r.hi), nrh = f2_pack(-r.hi, -r.hi), rl = f2_pack(r.lo, r.lo);
      const uint64_t ih = f2_pack(-i.hi, i.hi), nih = f2_pack(i.hi, -i.hi), il = f2_pack(-i.lo, i.lo);
#pragma unroll
      for (int q = 0; q < VPL; ++q) {
        dd_fma_acc2(rh, nrh, rl, x.re[q], x.im[q], acc.re[q], acc.im[q]);
        dd_fma_acc2(ih, nih, il, x.im[q], x.re[q], acc.re[q], acc.im[q]);
      }
    } else {
#pragma unroll
      for (int q = 0; q < VPL; ++q) {
        acc.re[q] = r * x.re[q] + acc.re[q];
        acc.re[q] = -i * x.im[q] + acc.re[q];
        acc.im[q] = r * x.im[q] + acc.im[q];
        acc.im[q] = i * x.re[q] + acc.im[q];
      }
    }
  }
};

// out = 2 acc - prev for the lane's elements.  Double-float: both parts of an
// element in packed f32x2 arithmetic; 2 acc is exact, so the scalar dd(2) *
// acc is the pair's TwoSum (2 hi, 2 lo), and the subtraction is the scalar
// dd addition of -prev, operation for operation: the same values.
__device__ __forceinline__ void dd_out2(dd ar, dd ai, dd pr, dd pi, dd& outr, dd& outi) {
  const uint64_t neg = f2_pack(-1.f, -1.f);
  const uint64_t h = f2_add(f2_pack(ar.hi, ai.hi), f2_pack(ar.hi, ai.hi));
  const uint64_t l = f2_add(f2_pack(ar.lo, ai.lo), f2_pack(ar.lo, ai.lo));
  const uint64_t s = f2_add(h, l);                             // fast TwoSum (|h| >= |l|)
  const uint64_t sl = f2_sub(l, f2_sub(s, h));
  const uint64_t yh = f2_mul(neg, f2_pack(pr.hi, pi.hi)), yl = f2_mul(neg, f2_pack(pr.lo, pi.lo));
  const uint64_t s2 = f2_add(s, yh);                           // the dd addition
  const uint64_t bb = f2_sub(s2, s);
  uint64_t e = f2_add(f2_sub(s, f2_sub(s2, bb)), f2_sub(yh, bb));
  e = f2_add(e, f2_add(sl, yl));
  const uint64_t o = f2_add(s2, e);
  const uint64_t ol = f2_sub(e, f2_sub(o, s2));
  f2_unpack(o, outr.hi, outi.hi);
  f2_unpack(ol, outr.lo, outi.lo);
}
template <typename F, int VPL>
__device__ __forceinline__ void recur_out(const LaneV<F, VPL>& acc, const LaneV<F, VPL>& prev, LaneV<F, VPL>& out) {
#pragma unroll
  for (int q = 0; q < VPL; ++q) {
    if constexpr (is_dd<F>) {
      dd_out2(acc.re[q], acc.im[q], prev.re[q], prev.im[q], out.re[q], out.im[q]);
    } else {
      out.re[q] = F(2) * acc.re[q] - prev.re[q];
      out.im[q] = F(2) * acc.im[q] - prev.im[q];
    }
  }
}
// m += Re sum_q conj(a_q) b_q over the lane's elements.  Double-float: the
// terms accumulate unnormalised in the manner of Dot2 (dd_fma_acc), which the
// final conversion (double) hi + (double) lo takes exactly.
template <typename F, int VPL>
__device__ __forceinline__ void dot_acc(const LaneV<F, VPL>& a, const LaneV<F, VPL>& b, F& m) {
#pragma unroll
  for (int q = 0; q < VPL; ++q) {
    if constexpr (is_dd<F>) {
      dd_fma_acc(a.re[q], b.re[q], m);
      dd_fma_acc(a.im[q], b.im[q], m);
    } else {
      m += a.re[q] * b.re[q] + a.im[q] * b.im[q];
    }
  }
}

// a row sum built by HVal::fma, ready for use: double-float sums are
// normalised (no-op for float and double)
template <typename F, int VPL>
__device__ __forceinline__ void finish_acc(LaneV<F, VPL>& acc) {
  if constexpr (is_dd<F>) {
#pragma unroll
    for (int q = 0; q < VPL; ++q) {
      acc.re[q] = dd_norm(acc.re[q]);
      acc.im[q] = dd_norm(acc.im[q]);
    }
  }
}

template <typename F> struct VecW { static constexpr int max_vpl = (sizeof(F) == 4) ? 2 : 1; };
// double-float: two vectors per lane (two 16-byte accesses) as for complex64,
// twice the rows per warp and so twice the gathers in flight per warp
template <> struct VecW<dd> { static constexpr int max_vpl = 2; };

// Asynchronous bulk prefetch of [src, src+bytes) into L2 (no shared memory, no
// completion to wait for); bytes % 16 == 0 and src 16-byte aligned.
__device__ __forceinline__ void bulk_prefetch_l2(const void* src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(src), "r"(bytes) : "memory");
}

}  // namespace tbk
