// kpm_step.cuh — the one-pass recursion step kernel and its launch templates.
// Instantiated per vector precision in kpm_step_f32.cu, kpm_step_f64.cu and
// kpm_step_dd.cu (compiled in parallel); everything else calls
// launch_step_prec / occupancy_prec.
#pragma once
#include <cuda_runtime.h>

#include "kpm_device.cuh"
#include "tbk_internal.h"

namespace tbk {

constexpr int kStepThreads = 256;
constexpr int kStepWarps = kStepThreads / 32;

// Row classes of a translation-invariant matrix (EllDev::cls*): class of each
// row, and per class its entry count, column offsets (column - row) and values
// in the recursion's precision, w entries per class.
struct ClassTab {
  const uint8_t* cls = nullptr;
  const int32_t* cnt = nullptr;
  const int32_t* off = nullptr;
  const void* val = nullptr;
  int32_t n_cls = 0, w = 0;
};
// shared-memory table of the class form: values, offsets, counts
template <typename F, bool CPLX_H>
constexpr int class_value_bytes() { return (CPLX_H ? 2 : 1) * (int)sizeof(F); }
template <typename F, bool CPLX_H>
inline size_t class_smem_bytes(const ClassTab& ct) {
  const size_t ne = (size_t)ct.n_cls * ct.w;
  return ne * class_value_bytes<F, CPLX_H>() + ne * 4 + (size_t)ct.n_cls * 4;
}

// One recursion step over all rows, x = v_s, y = v_{s-1} on entry.
//   FIRST: y = H x                    else: y = 2 H x - y  (v_{s+1} over v_{s-1})
//   doubling (BRAKET false): part[0] += <x|x>; part[1] += <x|y_in> (= <v_s|v_{s-1}>),
//                            FIRST: part[1] += <x|H x> (= <v_0|v_1>)
//   braket:                  part[0] += <b|v_{s+1}>;  FIRST also part[1] += <b|x>
//   gather == 0: no product at all (the last doubling step only needs the dots).
//   KST: 3 = add c v to the output (a Clenshaw step of a Chebyshev expansion,
//   ks.addc / ks.addv); otherwise also write complex64 K-tiled stores (Kubo
//   blocks, KStore): 1 = the output into one store; 2 = per column group the
//   output or V x for an
//   operator V with H's ELL structure, formed from the same gathered x (the
//   operator product of the previous block fused into the step), so that the
//   two sides of a Kubo pair can run as one recursion of twice the width.  A
//   template parameter because even an untaken runtime branch there costs the
//   moments recursion ~8% of its bandwidth.
//   KST = 4: a plain step whose moments nothing reads (the Kubo recursion
//   ahead of an operator product).  Only KST = 0 forms the moment sums.
//   PIPE: rows wider than one group of 4 gathers (ELL width > 4, e.g. FCC's
//   12 neighbours) load the next group's columns while this group's gathers
//   are in flight: 4 dependent memory round trips per 12-neighbour row instead
//   of 6 (1.8x on the FCC Kubo recursion).  Narrow rows keep the plain loop,
//   whose extra predicated loads would cost the honeycomb recursion 8%.
//   CLS: rows of a translation-invariant matrix come in a few classes (ct);
//   each neighbour is row + offset from the class table in shared memory and
//   its value comes from there too, so no column index or value is loaded and
//   the only index read (the row's class byte) is issued one grid-stride
//   iteration ahead.  Same entries in the same order as the ELL: the same sums.
template <typename F, int R, bool CPLX_H, bool FIRST, bool BRAKET, int KST = 0, bool PIPE = false, bool CLS = false>
__global__ void __launch_bounds__(kStepThreads) kpm_step_kernel(
    int32_t n, int32_t n_tiles, const int32_t* __restrict__ soff, const int32_t* __restrict__ ecol,
    const F* __restrict__ eval, const F* __restrict__ diag, const typename C2<F>::T* __restrict__ x,
    typename C2<F>::T* y, const typename C2<F>::T* pv, const typename C2<F>::T* __restrict__ bras,
    double* __restrict__ part, int store, int reverse, int gather, int pf_dist, const KStore ks, const ClassTab ct) {
  using CT = typename C2<F>::T;
  constexpr int VPL = (R >= VecW<F>::max_vpl) ? VecW<F>::max_vpl : 1;
  constexpr int LPR = R / VPL;             // lanes per row
  constexpr int RPW = 32 / LPR;            // rows per warp
  constexpr int ROWS_PER_TILE = RPW * kStepWarps;
  static_assert(LPR >= 1 && LPR <= 32 && (32 % LPR) == 0, "R out of range");
  using Acc = F;                           // per-thread sums in the vector precision

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane % LPR;
  Acc m0 = 0, m1 = 0;
  static_assert(!(CLS && (PIPE || KST == 2)), "class form: no column pipeline, no operator products");

  // class form: the table in shared memory (4-byte words: values, offsets, counts)
  extern __shared__ __align__(16) unsigned char cls_smem[];
  const F* s_val = reinterpret_cast<const F*>(cls_smem);
  const int32_t* s_off = nullptr;
  const int32_t* s_cnt = nullptr;
  uint32_t c_next = 0;                     // class of this thread's row in the next iteration
  if constexpr (CLS) {
    const int32_t ne = ct.n_cls * ct.w;
    const int32_t vw = ne * (class_value_bytes<F, CPLX_H>() / 4);
    uint32_t* sw = reinterpret_cast<uint32_t*>(cls_smem);
    const uint32_t* gv = static_cast<const uint32_t*>(ct.val);
    for (int32_t q = threadIdx.x; q < vw; q += blockDim.x) sw[q] = gv[q];
    for (int32_t q = threadIdx.x; q < ne; q += blockDim.x) sw[vw + q] = (uint32_t)ct.off[q];
    for (int32_t q = threadIdx.x; q < ct.n_cls; q += blockDim.x) sw[vw + ne + q] = (uint32_t)ct.cnt[q];
    s_off = reinterpret_cast<const int32_t*>(sw + vw);
    s_cnt = reinterpret_cast<const int32_t*>(sw + vw + ne);
    __syncthreads();
    const int32_t t0 = blockIdx.x;
    if (t0 < n_tiles) {
      const int32_t r0 = (reverse ? (n_tiles - 1 - t0) : t0) * ROWS_PER_TILE + warp * RPW + lane / LPR;
      if (r0 < n) c_next = __ldg(ct.cls + r0);
    }
  }

  for (int32_t t = blockIdx.x; t < n_tiles; t += gridDim.x) {
    const uint32_t c_cur = c_next;
    if constexpr (CLS) {
      const int32_t tn = t + (int32_t)gridDim.x;
      c_next = 0;
      if (tn < n_tiles) {
        const int32_t rn = (reverse ? (n_tiles - 1 - tn) : tn) * ROWS_PER_TILE + warp * RPW + lane / LPR;
        if (rn < n) c_next = __ldg(ct.cls + rn);
      }
    }
    const int32_t tile = reverse ? (n_tiles - 1 - t) : t;
    if (pf_dist > 0 && threadIdx.x == 0) {
      // bring the streams of the tile this CTA reaches pf_dist iterations later
      // into L2 ahead of time: its own rows of v_n and v_{n-1} (and the bras)
      const int32_t tf = t + pf_dist * (int32_t)gridDim.x;
      if (tf < n_tiles) {
        const int32_t tilef = reverse ? (n_tiles - 1 - tf) : tf;
        const int64_t rf = (int64_t)tilef * ROWS_PER_TILE;
        const int32_t nr = (int32_t)min((int64_t)ROWS_PER_TILE, (int64_t)n - rf);
        if (nr > 0) {
          const uint32_t vb = (uint32_t)nr * (uint32_t)(R * sizeof(CT));
          if ((vb & 15u) == 0) {
            bulk_prefetch_l2(x + rf * R, vb);
            if (!FIRST) bulk_prefetch_l2(pv + rf * R, vb);
            if (BRAKET) bulk_prefetch_l2(bras + rf * R, vb);
          }
          if constexpr (!CLS) {
            if (gather) {
              // and the ELL columns and values of its slices, so that the rows'
              // column loads find them in L2 (slice offsets are whole 32-entry
              // columns: 128-byte aligned, whole 128-byte multiples)
              constexpr uint32_t VB = (CPLX_H ? 2u : 1u) * (uint32_t)sizeof(F);
              const int32_t s0 = (int32_t)(rf >> 5), s1 = (int32_t)((rf + nr - 1) >> 5);
              const int32_t o0 = soff[s0], o1 = soff[s1 + 1];
              if (o1 > o0) {
                bulk_prefetch_l2(ecol + o0, (uint32_t)(o1 - o0) * 4u);
                bulk_prefetch_l2(reinterpret_cast<const char*>(eval) + (int64_t)o0 * VB, (uint32_t)(o1 - o0) * VB);
              }
            }
          }
        }
      }
    }
    const int32_t r = tile * ROWS_PER_TILE + warp * RPW + lane / LPR;
    if (r >= n) continue;
    const int64_t me = (int64_t)r * LPR + sub;
    const LaneV<F, VPL> xs = ld_ro<F, VPL>(x + me * VPL);
    LaneV<F, VPL> prev;
    if constexpr (!FIRST) prev = ld_stream<F, VPL>(pv + me * VPL);   // pv == y: in place
    LaneV<F, VPL> acc, vacc;
#pragma unroll
    for (int q = 0; q < VPL; ++q) { acc.re[q] = 0; acc.im[q] = 0; }
    // column group of this lane (its VPL columns never straddle two groups)
    const int grp = (KST == 2 && ks.halves == 2 && sub * VPL >= R / 2) ? 1 : 0;
    const F* vval = nullptr;
    const F* vdiag = nullptr;
    if constexpr (KST == 2) {
      const void* vv = grp ? ks.vval[1] : ks.vval[0];      // selects, not an indexed parameter array
      const void* vd = grp ? ks.vdiag[1] : ks.vdiag[0];
      vval = vv ? static_cast<const F*>(vv) : eval;
      vdiag = vd ? static_cast<const F*>(vd) : diag;
#pragma unroll
      for (int q = 0; q < VPL; ++q) { vacc.re[q] = 0; vacc.im[q] = 0; }
    }
    if (gather && CLS) {
      HVal<F, CPLX_H>::load(diag, r).template fma<VPL>(xs, acc);
      const int32_t cnt = s_cnt[c_cur];
      const int32_t tb = (int32_t)c_cur * ct.w;
      // a class's tail entries up to the table width (a multiple of 4) are
      // (offset 0, value 0): 0 x (own row), exactly what a predicated-off entry
      // adds.  FP32 vectors take whole groups without predicates (fewer
      // instructions and registers); the wider types keep the predicates,
      // whose unconditional form holds more gathers in registers
      constexpr bool WHOLE = sizeof(F) == 4;
      for (int k = 0; k < cnt; k += 4) {
        HVal<F, CPLX_H> h[4];
        LaneV<F, VPL> xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const bool v = WHOLE || k + u < cnt;
          // rows are verified equal to their class, so r + offset is the
          // row's column; the clamp only keeps a bad table inside the block
          const int32_t c = v ? min(max(r + s_off[tb + k + u], 0), n - 1) : r;
          h[u] = v ? HVal<F, CPLX_H>::load_smem(s_val, tb + k + u) : HVal<F, CPLX_H>::zero();
          xv[u] = v ? ld_ro<F, VPL>(x + ((int64_t)c * LPR + sub) * VPL) : xs;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) h[u].template fma<VPL>(xv[u], acc);
      }
    } else if (gather) {
      HVal<F, CPLX_H>::load(diag, r).template fma<VPL>(xs, acc);
      if constexpr (KST == 2) HVal<F, CPLX_H>::load(vdiag, r).template fma<VPL>(xs, vacc);
      const int32_t s = r >> 5, l = r & 31;
      const int32_t off = soff[s];
      const int32_t w = (soff[s + 1] - off) >> 5;
      const int32_t* cp = ecol + off + l;
      // all of a row's gathers in flight together: predicated groups of 4
      int32_t cn[4];
      if constexpr (PIPE) {
#pragma unroll
        for (int u = 0; u < 4; ++u) cn[u] = u < w ? __ldg(cp + u * 32) : r;
      }
      for (int k = 0; k < w; k += 4) {
        int32_t c[4];
        HVal<F, CPLX_H> h[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          const bool v = k + u < w;
          if constexpr (PIPE) c[u] = cn[u];
          else c[u] = v ? __ldg(cp + (k + u) * 32) : r;             // padding: own row
          h[u] = v ? HVal<F, CPLX_H>::load(eval, off + l + (int64_t)(k + u) * 32) : HVal<F, CPLX_H>::zero();
        }
        if constexpr (PIPE) {                                       // next group's columns
#pragma unroll
          for (int u = 0; u < 4; ++u) cn[u] = k + 4 + u < w ? __ldg(cp + (k + 4 + u) * 32) : r;
        }
        LaneV<F, VPL> xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) xv[u] = ld_ro<F, VPL>(x + ((int64_t)c[u] * LPR + sub) * VPL);
#pragma unroll
        for (int u = 0; u < 4; ++u) h[u].template fma<VPL>(xv[u], acc);
        if constexpr (KST == 2) {
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const HVal<F, CPLX_H> hv = k + u < w ? HVal<F, CPLX_H>::load(vval, off + l + (int64_t)(k + u) * 32)
                                                 : HVal<F, CPLX_H>::zero();
            hv.template fma<VPL>(xv[u], vacc);
          }
        }
      }
    }
    finish_acc<F, VPL>(acc);
    if constexpr (KST == 2) finish_acc<F, VPL>(vacc);
    LaneV<F, VPL> out;
    if constexpr (FIRST) out = acc;
    else recur_out<F, VPL>(acc, prev, out);
    if constexpr (KST == 3) {
      // Clenshaw step of a Chebyshev expansion: b_k = 2 H b_{k+1} - b_{k+2} + c_k v
      const LaneV<F, VPL> vv = ld_ro<F, VPL>(static_cast<const CT*>(ks.addv) + me * VPL);
      const F cr = F(ks.addc[0]), ci = F(ks.addc[1]);
#pragma unroll
      for (int q = 0; q < VPL; ++q) {
        out.re[q] = out.re[q] + (cr * vv.re[q] - ci * vv.im[q]);
        out.im[q] = out.im[q] + (cr * vv.im[q] + ci * vv.re[q]);
      }
    }
    // moment partial sums (before the store, from registers only); steps that
    // feed stores, expansions or an operator product need none
    if constexpr (KST != 0) {
    } else if constexpr (BRAKET) {
      const LaneV<F, VPL> b = ld_ro<F, VPL>(bras + me * VPL);
      dot_acc<F, VPL>(b, out, m0);
      if constexpr (FIRST) dot_acc<F, VPL>(b, xs, m1);
    } else {
      dot_acc<F, VPL>(xs, xs, m0);
      if constexpr (FIRST) dot_acc<F, VPL>(xs, out, m1);
      else dot_acc<F, VPL>(xs, prev, m1);
    }
    if (store) st_v<F, VPL>(y + me * VPL, out);
    if constexpr (KST == 1) {
      // block km[0] of the K-tiled store: one rounding per value
#pragma unroll
      for (int q = 0; q < VPL; ++q) {
        const int64_t k = (int64_t)r * R + sub * VPL + q;
        ks.store[0][((k >> 4) * ks.kM + ks.km[0]) * 16 + (k & 15)] = make_float2(to_f32(out.re[q]), to_f32(out.im[q]));
      }
    } else if constexpr (KST == 2) {
      const int32_t kmg = grp ? ks.km[1] : ks.km[0];
      if (kmg >= 0) {
        const int32_t Rg = R / ks.halves;
        const LaneV<F, VPL>& sv = (grp ? ks.usev[1] : ks.usev[0]) ? vacc : out;
        float2* dst = grp ? ks.store[1] : ks.store[0];
#pragma unroll
        for (int q = 0; q < VPL; ++q) {
          const int64_t k = (int64_t)r * Rg + sub * VPL + q - grp * Rg;
          dst[((k >> 4) * ks.kM + kmg) * 16 + (k & 15)] = make_float2(to_f32(sv.re[q]), to_f32(sv.im[q]));
        }
      }
    }
  }
  // FP64 from here on: warp shuffle, then across the CTA's warps
  double d0 = (double)m0, d1 = (double)m1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    d0 += __shfl_xor_sync(0xffffffffu, d0, o);
    d1 += __shfl_xor_sync(0xffffffffu, d1, o);
  }
  __shared__ double sh[2][kStepWarps];
  if (lane == 0) { sh[0][warp] = d0; sh[1][warp] = d1; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
#pragma unroll
    for (int q = 0; q < kStepWarps; ++q) { a += sh[0][q]; b += sh[1][q]; }
    part[blockIdx.x] = a;
    part[gridDim.x + blockIdx.x] = b;
  }
}


// ----------------------------------------------------------------- dispatch
struct StepArgs {
  int32_t n, n_tiles, n_slices;
  int* err;
  const int32_t* soff;
  const int32_t* ecol;
  const void* eval;
  const void* diag;
  const void* x;
  void* y;
  const void* pv;      // v_{n-1}; equal to y for the in-place recursion
  const void* bras;
  double* part;
  int store, reverse, gather, pf_dist;
  KStore ks;                   // optional complex64 K-tiled stores (Kubo blocks)
  int kst = 0;                 // 0 moments, 1 output into ks.store[0], 2 per-group output / V x,
                               // 3 Clenshaw term, 4 plain step without moment sums
  bool pipe = false;           // ELL wider than 4: pipelined column loads
  bool cls = false;            // row classes (ct) instead of the ELL's columns and values
  ClassTab ct;
};

template <typename F, int R, bool CPLX_H, bool CLS>
inline int launch_step_r(const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  using CT = typename C2<F>::T;
  const size_t smem = CLS ? class_smem_bytes<F, CPLX_H>(a.ct) : 0;
  auto x = static_cast<const CT*>(a.x);
  auto y = static_cast<CT*>(a.y);
  auto pv = static_cast<const CT*>(a.pv ? a.pv : a.y);
  auto b = static_cast<const CT*>(a.bras);
  auto ev = static_cast<const F*>(a.eval);
  auto dg = static_cast<const F*>(a.diag);
#define TBK_STEP(FI, BR, KS)                                                                          \
  do {                                                                                                \
    if constexpr (CLS)                                                                                \
      kpm_step_kernel<F, R, CPLX_H, FI, BR, KS, false, true><<<grid, kStepThreads, smem, st>>>(       \
          a.n, a.n_tiles, a.soff, a.ecol, ev, dg, x, y, pv, b, a.part, a.store, a.reverse, a.gather, a.pf_dist, a.ks, \
          a.ct);                                                                                      \
    else if (a.pipe)                                                                                  \
      kpm_step_kernel<F, R, CPLX_H, FI, BR, KS, true><<<grid, kStepThreads, 0, st>>>(                 \
          a.n, a.n_tiles, a.soff, a.ecol, ev, dg, x, y, pv, b, a.part, a.store, a.reverse, a.gather, a.pf_dist, a.ks, \
          a.ct);                                                                                      \
    else                                                                                              \
      kpm_step_kernel<F, R, CPLX_H, FI, BR, KS, false><<<grid, kStepThreads, 0, st>>>(                \
          a.n, a.n_tiles, a.soff, a.ecol, ev, dg, x, y, pv, b, a.part, a.store, a.reverse, a.gather, a.pf_dist, a.ks, \
          a.ct);                                                                                      \
  } while (0)
  if (a.kst != 0) {
    if (braket) return fail(TBK_ERR_UNSUPPORTED, "K-tiled store with a braket step");
    constexpr int VPLR = (R >= VecW<F>::max_vpl) ? VecW<F>::max_vpl : 1;
    if (a.kst == 2 && a.ks.halves == 2 && (R / 2) % VPLR != 0)
      return fail(TBK_ERR_UNSUPPORTED, "column groups narrower than a lane's vectors");
    if (a.kst == 3) {
      if (first) return fail(TBK_ERR_UNSUPPORTED, "Clenshaw term on a first step");
      TBK_STEP(false, false, 3);
    } else if (a.kst == 4) {
      if (first) TBK_STEP(true, false, 4); else TBK_STEP(false, false, 4);
    } else if (a.kst == 2) {
      if constexpr (CLS) return fail(TBK_ERR_UNSUPPORTED, "operator products in the class form");
      else { if (first) TBK_STEP(true, false, 2); else TBK_STEP(false, false, 2); }
    }
    else { if (first) TBK_STEP(true, false, 1); else TBK_STEP(false, false, 1); }
  } else if (first) { if (braket) TBK_STEP(true, true, 0); else TBK_STEP(true, false, 0); }
  else { if (braket) TBK_STEP(false, true, 0); else TBK_STEP(false, false, 0); }
#undef TBK_STEP
  TBK_CHECK_LAUNCH();
  return TBK_OK;
}

template <typename F, bool CPLX_H, bool CLS = false>
inline int launch_step(int R, const StepArgs& a, bool first, bool braket, int grid, cudaStream_t st) {
  switch (R) {
    case 1: return launch_step_r<F, 1, CPLX_H, CLS>(a, first, braket, grid, st);
    case 2: return launch_step_r<F, 2, CPLX_H, CLS>(a, first, braket, grid, st);
    case 4: return launch_step_r<F, 4, CPLX_H, CLS>(a, first, braket, grid, st);
    case 8: return launch_step_r<F, 8, CPLX_H, CLS>(a, first, braket, grid, st);
    case 16: return launch_step_r<F, 16, CPLX_H, CLS>(a, first, braket, grid, st);
    case 32: return launch_step_r<F, 32, CPLX_H, CLS>(a, first, braket, grid, st);
    case 64:
      if constexpr (sizeof(F) == 4) return launch_step_r<F, 64, CPLX_H, CLS>(a, first, braket, grid, st);
      break;
  }
  return fail(TBK_ERR_UNSUPPORTED, "chunk width %d not instantiated", R);
}


template <typename F, bool CPLX_H, int R, bool CLS = false>
inline int occupancy_blocks(size_t smem = 0) {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kpm_step_kernel<F, R, CPLX_H, false, false, 0, false, CLS>,
                                                kStepThreads, smem);
  return nb > 0 ? nb : 1;
}

template <typename F, bool CLS>
inline int occupancy_r(bool cplx, int R, size_t smem) {
  switch (R) {
    case 1: return cplx ? occupancy_blocks<F, true, 1, CLS>(smem) : occupancy_blocks<F, false, 1, CLS>(smem);
    case 2: return cplx ? occupancy_blocks<F, true, 2, CLS>(smem) : occupancy_blocks<F, false, 2, CLS>(smem);
    case 4: return cplx ? occupancy_blocks<F, true, 4, CLS>(smem) : occupancy_blocks<F, false, 4, CLS>(smem);
    case 8: return cplx ? occupancy_blocks<F, true, 8, CLS>(smem) : occupancy_blocks<F, false, 8, CLS>(smem);
    case 16: return cplx ? occupancy_blocks<F, true, 16, CLS>(smem) : occupancy_blocks<F, false, 16, CLS>(smem);
    default: return cplx ? occupancy_blocks<F, true, 32, CLS>(smem) : occupancy_blocks<F, false, 32, CLS>(smem);
  }
}

// per-precision entry points (TBK_PREC_*); a.cls selects the class form
int launch_step_prec(int prec, bool cplx, int R, const StepArgs& a, bool first, bool braket, int grid,
                     cudaStream_t st);
int occupancy_prec(int prec, bool cplx, int R);
// CTAs per SM of the class-form kernel with its shared-memory table
int occupancy_cls_prec(int prec, bool cplx, int R, size_t smem);
// the class table of a matrix in a precision (ct.n_cls == 0: no class form)
ClassTab class_tab(const EllDev& E, int prec);
size_t class_smem(const EllDev& E, int prec);

}  // namespace tbk
