// serving.cu — many density-of-states solves advanced together.
//
// No counterpart in the reference: each of its solves is one call of
// density_of_states_seq (TB/functions.h:15-32), whose moments come from
// Cheb_first_kind_seq_braket (TB/numerics_cuda.cu:190-255).  Here a request is
// a lattice spec plus bounds, M, R, seed and precision, and
//   - the admission thread takes requests in FIFO order while the HBM budget
//     holds their build peak, builds H~ = (H - b)/a and the sliced ELL on its
//     own stream with stream-ordered (pool) allocations, keeps only what the
//     recursion reads and seeds the random-phase kets;
//   - the round thread moves built requests into the running set (bounded by
//     the bytes one step moves) and advances the set S steps per round.  A
//     round is one CUDA graph: per (precision, width) group a chain of S step
//     launches over the slabs of all the group's requests (the chains of
//     different groups run concurrently), then the reduction of the per-slab
//     moment partials and the moment assembly of the requests that finish,
//     written straight into pinned host memory.  Graphs are cached per group
//     set; what changes from round to round (which requests, at which step)
//     lives in a device table copied in before the launch.
// A request's rows are cut into tiles (one CTA's work) of kSrvWarps slabs;
// each slab (a fixed set of the tile's rows) is one warp's work and one moment
// partial, and the slab partials of a request are summed in slab order.  So a
// request's moments depend only on the request, never on what runs beside it.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "host_model.h"
#include "kpm_device.cuh"
#include "tbk_internal.h"

namespace tbk {
namespace {

constexpr int kSrvThreads = 256;
constexpr int kSrvWarps = kSrvThreads / 32;
constexpr int kIterPerSlab = 8;        // warp iterations (512 B of v_s each) per slab
// group code = ((prec * 8 + log2(width)) * 2 + complex) * 2 + class form, prec < 3
constexpr int kGroups = 96;
using GroupMask = unsigned __int128;
inline GroupMask group_bit(int code) { return (GroupMask)1 << code; }

struct SLane {                      // up to 64 vectors of one request (device view)
  const int32_t* soff;              // ELL slice offsets; class form: entry count per class
  const int32_t* ecol;              // ELL columns; class form: column offsets per class
  const void* eval;                 // ELL values; class form: values per class
  const void* diag;
  const uint8_t* cls;               // class form: class of each row
  void* va;                         // v_s for even s
  void* vb;                         // v_s for odd s
  int32_t n, n_steps, s0, req;
  // the lane's slab partials are part[slab_begin ..+ n_slabs): kSrvWarps per
  // tile (its first tile is slab_begin / kSrvWarps), the last tile's slabs
  // past the rows hold zeros; slab_rows rows per slab
  int32_t slab_begin, n_slabs, slab_rows, cls_w;   // cls_w: class form, entries per class
  int32_t n_cls, pad;               // class form: classes
};
struct STile {                      // kSrvWarps slabs of one lane, from row row0
  int32_t lane, row0;
};
struct SReq {
  double* sums;                     // [2 * n_steps] step sums
  double* mu;                       // pinned host result, device-visible
  int32_t lane0, n_lanes, s0, n_steps, n_mom, finishing;
};
struct SHdr {
  int32_t grp_begin[kGroups];       // a group's tiles: tiles[grp_begin .. + grp_count)
  int32_t grp_count[kGroups];
  int32_t n_lanes, n_tiles, n_reqs, pad;
};

// complex element size cs = 8 (complex64) or 16 (complex128); width R
__host__ __device__ constexpr int srv_vpl(int cs, int R) { return (cs == 8 && R >= 2) ? 2 : 1; }
__host__ __device__ constexpr int srv_rows_per_warp(int cs, int R) { return 32 / (R / srv_vpl(cs, R)); }
// Rows per slab: eight warp iterations, 4 KB of v_s (a tile: kSrvWarps slabs).
// The slab is the unit of one moment partial, so this fixes the summation
// order; it depends on (cs, R) alone.
inline int srv_iters_per_slab() {
  static const int it = [] {
    const char* e = getenv("TBK_SERVE_SLAB_ITERS");             // tuning override
    const int v = e ? atoi(e) : 0;
    return v >= 1 && v <= 256 ? v : kIterPerSlab;
  }();
  return it;
}
inline int srv_slab_rows(int cs, int R, int64_t) { return srv_rows_per_warp(cs, R) * srv_iters_per_slab(); }

// One doubling recursion step (step j of the round) over the tiles of group g.
// A lane's rows are cut into tiles of kSrvWarps slabs (kSrvWarps * slab_rows
// rows); a CTA takes a tile, and warp w's slab is the tile's row groups w,
// w + kSrvWarps, w + 2 kSrvWarps, ... (RPW rows each), so that at each warp
// iteration the CTA's warps read consecutive rows (whole DRAM pages) together.
// A slab is one moment partial: one warp's per-lane sums over its rows, then a
// fixed shuffle tree; slab w of the lane's k-th tile is partial k kSrvWarps + w.
// With s = s0 + j the lane's step, x = v_s and y = v_{s-1} on entry:
//   s == 0:         y = H x,             partials <x|x>, <x|y>
//   0 < s < last:   y = 2 H x - y,       partials <x|x>, <x|y_in>
//   s == last:      no product, no store, partials <x|x>, <x|y_in>
// which are the step sums of the doubling identities mu_2s = 2<v_s|v_s> - mu_0,
// mu_2s-1 = 2<v_s|v_s-1> - mu_1.
// The lane's pointers live in a per-CTA shared slot, re-read at each use so
// that they hold no registers across the gathers (complex64 groups fit 6 CTAs
// per SM in the class form, 5 in the ELL form, wider types 4); a CTA reloads
// the slot only when its next tile belongs to another lane.
// CLS (groups whose H~ has row classes): the slot also holds the lane's class
// table (entry counts, column offsets, values), where the streamed vector rows
// cannot evict it; a row's neighbours are row + offset, its values come from
// the table, and the only index it loads (its class byte) is issued one warp
// iteration ahead.  Same entries in the same order as the ELL: the same sums.
template <typename F, int R, bool CPLX_H, bool CLS>
__global__ void __launch_bounds__(kSrvThreads, sizeof(F) == 4 ? (CLS ? 6 : 5) : 4) srv_step_kernel(
    const SHdr* __restrict__ hdr, const SLane* __restrict__ lanes, const STile* __restrict__ tiles, int32_t g,
    int32_t j, int32_t reverse, int32_t pf_dist, double* __restrict__ part, int32_t slab_cap) {
  using CT = typename C2<F>::T;
  constexpr int CS = (int)sizeof(CT);
  constexpr int VPL = srv_vpl(CS, R);
  constexpr int LPR = R / VPL;
  constexpr int RPW = 32 / LPR;
  constexpr int STRIDE = RPW * kSrvWarps;                      // rows per CTA warp iteration
  static_assert(LPR >= 1 && LPR <= 32 && (32 % LPR) == 0, "width out of range");
  constexpr int VW = (CPLX_H ? 2 : 1) * (int)sizeof(F) / 4;    // 4-byte words per class-table value
  // class table: values, then offsets, then counts, at fixed word offsets
  __shared__ __align__(16) uint32_t tab[CLS ? kMaxClassEntries * (VW + 1) + kMaxClasses : 1];
  const F* s_val = reinterpret_cast<const F*>(tab);
  const int32_t* s_off = reinterpret_cast<const int32_t*>(tab + kMaxClassEntries * VW);
  const int32_t* s_cnt = reinterpret_cast<const int32_t*>(tab + kMaxClassEntries * (VW + 1));
  struct TP {
    const CT* x;
    CT* y;
    const int32_t* soff;
    const int32_t* ecol;
    const F* eval;
    const F* diag;
    const uint8_t* cls;
    int32_t n, w, s, ns, rows;
  };
  __shared__ TP tp;
  volatile TP* vt = &tp;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int sub = lane % LPR;
  const int32_t begin = hdr->grp_begin[g], cnt = hdr->grp_count[g];
  int32_t cur = -1;                                            // the lane whose slot the CTA holds
  for (int32_t t = blockIdx.x; t < cnt; t += gridDim.x) {
    const int32_t ti = begin + (reverse ? cnt - 1 - t : t);
    const STile tl = tiles[ti];
    if (tl.lane != cur) {                                      // uniform over the CTA
      __syncthreads();                                         // nobody reads the previous slot any more
      const SLane* L = lanes + tl.lane;
      if constexpr (CLS) {
        const int32_t ne = L->n_cls * L->cls_w;
        const uint32_t* gv = static_cast<const uint32_t*>(L->eval);
        for (int32_t q = threadIdx.x; q < ne * VW; q += kSrvThreads) tab[q] = __ldg(gv + q);
        for (int32_t q = threadIdx.x; q < ne; q += kSrvThreads)
          tab[kMaxClassEntries * VW + q] = (uint32_t)__ldg(L->ecol + q);
        for (int32_t q = threadIdx.x; q < L->n_cls; q += kSrvThreads)
          tab[kMaxClassEntries * (VW + 1) + q] = (uint32_t)__ldg(L->soff + q);
      }
      if (threadIdx.x == 0) {
        const int32_t sl = L->s0 + j;
        tp.x = static_cast<const CT*>((sl & 1) ? L->vb : L->va);
        tp.y = static_cast<CT*>((sl & 1) ? L->va : L->vb);
        tp.soff = L->soff;
        tp.ecol = L->ecol;
        tp.eval = static_cast<const F*>(L->eval);
        tp.diag = static_cast<const F*>(L->diag);
        tp.cls = L->cls;
        tp.n = L->n;
        tp.w = L->cls_w;
        tp.s = sl;
        tp.ns = L->n_steps;
        tp.rows = L->slab_rows * kSrvWarps;
      }
      __syncthreads();
      cur = tl.lane;
    }
    if (pf_dist > 0 && threadIdx.x == 0) {
      // rows into L2 in bulk: pf_dist 1, this tile's v_s (its warps' later
      // iterations and gathers find it there; v_{s-1} as well measured slower
      // on large requests, 120 MB per wave in flight); 2, v_s and v_{s-1} of
      // the tile this CTA takes one wave later
      const int32_t tf = pf_dist == 2 ? t + (int32_t)gridDim.x : t;
      if (tf < cnt) {
        const STile sf = tiles[begin + (reverse ? cnt - 1 - tf : tf)];
        const SLane* Lf = lanes + sf.lane;
        const int32_t sfs = Lf->s0 + j;
        const int32_t nr = min(Lf->slab_rows * kSrvWarps, Lf->n - sf.row0);
        if (sfs < Lf->n_steps && nr > 0) {
          const uint32_t nb = (uint32_t)nr * (uint32_t)(R * CS);
          if ((nb & 15u) == 0) {
            const CT* xf = static_cast<const CT*>((sfs & 1) ? Lf->vb : Lf->va);
            const CT* pf = static_cast<const CT*>((sfs & 1) ? Lf->va : Lf->vb);
            bulk_prefetch_l2(xf + (int64_t)sf.row0 * R, nb);
            if (sfs > 0 && pf_dist == 2) bulk_prefetch_l2(pf + (int64_t)sf.row0 * R, nb);
          }
        }
      }
    }
    const int32_t s = vt->s, ns = vt->ns;
    if (s >= ns) continue;                                     // the lane's recursion ended before this step
    const bool first = s == 0;
    const bool dot_only = s == ns - 1 && s > 0;
    const int32_t rend = min(tl.row0 + vt->rows, vt->n);
    F m0 = 0, m1 = 0;
    uint32_t c_next = 0;                                       // class form: class of this lane's next row
    if constexpr (CLS) {
      const int32_t r0 = tl.row0 + warp * RPW + lane / LPR;
      if (r0 < rend) c_next = __ldg(vt->cls + r0);
    }
    for (int32_t rb = tl.row0 + warp * RPW; rb < rend; rb += STRIDE) {
      const int32_t r = rb + lane / LPR;
      if (r >= rend) break;
      const uint32_t cr = c_next;
      if constexpr (CLS) c_next = r + STRIDE < rend ? __ldg(vt->cls + r + STRIDE) : 0u;
      const int64_t me = (int64_t)r * LPR + sub;
      const LaneV<F, VPL> xs = ld_ro<F, VPL>(vt->x + me * VPL);
      LaneV<F, VPL> prev;
      if (!first) {
        prev = ld_stream<F, VPL>(vt->y + me * VPL);
      } else {
#pragma unroll
        for (int q = 0; q < VPL; ++q) { prev.re[q] = 0; prev.im[q] = 0; }
      }
      LaneV<F, VPL> acc;
#pragma unroll
      for (int q = 0; q < VPL; ++q) { acc.re[q] = 0; acc.im[q] = 0; }
      if (!dot_only && CLS) {
        HVal<F, CPLX_H>::load(vt->diag, r).template fma<VPL>(xs, acc);
        const int32_t kc = s_cnt[cr];
        const int32_t tb = (int32_t)cr * vt->w;
        const int32_t n = vt->n;
        // zero tail entries up to the table width (a multiple of 4): FP32
        // vectors take whole groups without predicates, as the moments kernel
        constexpr bool WHOLE = sizeof(F) == 4;
        for (int k = 0; k < kc; k += 4) {
          const CT* xp = vt->x;
          HVal<F, CPLX_H> h[4];
          LaneV<F, VPL> xv[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const bool v = WHOLE || k + u < kc;
            // rows are verified equal to their class: r + offset is the row's
            // column; the clamp only keeps a bad table inside the block
            const int32_t c = v ? min(max(r + s_off[tb + k + u], 0), n - 1) : r;
            h[u] = v ? HVal<F, CPLX_H>::load_smem(s_val, tb + k + u) : HVal<F, CPLX_H>::zero();
            xv[u] = v ? ld_ro<F, VPL>(xp + ((int64_t)c * LPR + sub) * VPL) : xs;
          }
#pragma unroll
          for (int u = 0; u < 4; ++u) h[u].template fma<VPL>(xv[u], acc);
        }
      } else if (!dot_only) {
        HVal<F, CPLX_H>::load(vt->diag, r).template fma<VPL>(xs, acc);
        const int32_t sidx = r >> 5, l = r & 31;
        const int32_t* so = vt->soff;
        const int32_t off = so[sidx];
        const int32_t w = (so[sidx + 1] - off) >> 5;
        for (int k = 0; k < w; k += 4) {
          const int32_t* cp = vt->ecol + off + l;
          const F* ev = vt->eval;
          int32_t c[4];
          HVal<F, CPLX_H> h[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            const bool v = k + u < w;
            c[u] = v ? __ldg(cp + (k + u) * 32) : r;
            h[u] = v ? HVal<F, CPLX_H>::load(ev, off + l + (int64_t)(k + u) * 32) : HVal<F, CPLX_H>::zero();
          }
          const CT* xp = vt->x;
          LaneV<F, VPL> xv[4];
#pragma unroll
          for (int u = 0; u < 4; ++u) xv[u] = ld_ro<F, VPL>(xp + ((int64_t)c[u] * LPR + sub) * VPL);
#pragma unroll
          for (int u = 0; u < 4; ++u) h[u].template fma<VPL>(xv[u], acc);
        }
      }
      finish_acc<F, VPL>(acc);
      LaneV<F, VPL> out;
      if (first) out = acc;
      else recur_out<F, VPL>(acc, prev, out);
      dot_acc<F, VPL>(xs, xs, m0);
      if (first) dot_acc<F, VPL>(xs, out, m1);
      else dot_acc<F, VPL>(xs, prev, m1);
      if (!dot_only) st_v<F, VPL>(vt->y + me * VPL, out);
    }
    __syncwarp();
    // slab partial in FP64: a fixed shuffle tree, lane 0 writes (an empty
    // slab of a lane's last tile writes zeros)
    double d0 = (double)m0, d1 = (double)m1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      d0 += __shfl_xor_sync(0xffffffffu, d0, o);
      d1 += __shfl_xor_sync(0xffffffffu, d1, o);
    }
    if (lane == 0) {
      double* pp = part + ((int64_t)j * slab_cap + (int64_t)ti * kSrvWarps + warp) * 2;
      pp[0] = d0;
      pp[1] = d1;
    }
  }
}

// Step sums of every running request: one CTA per (request, step of the
// round); thread k adds slabs k, k+256, ... of each lane in order, then a fixed
// tree in shared memory; thread 0 writes.
constexpr int kReduceThreads = 256;
__global__ void __launch_bounds__(kReduceThreads) srv_reduce_kernel(
    const SHdr* __restrict__ hdr, const SLane* __restrict__ lanes, const SReq* __restrict__ reqs,
    const double* __restrict__ part, int32_t slab_cap, int32_t S) {
  __shared__ double sh[2][kReduceThreads];
  const int32_t total = hdr->n_reqs * S;
  for (int32_t w = blockIdx.x; w < total; w += gridDim.x) {
    const int32_t q = w / S, j = w - q * S;
    const SReq rq = reqs[q];
    const int32_t s = rq.s0 + j;
    if (s >= rq.n_steps) continue;               // uniform over the CTA
    double t0 = 0.0, t1 = 0.0;
    for (int32_t c = 0; c < rq.n_lanes; ++c) {
      const SLane& L = lanes[rq.lane0 + c];
      const double* p = part + ((int64_t)j * slab_cap + L.slab_begin) * 2;
      double a0 = 0.0, a1 = 0.0;
      for (int32_t k = threadIdx.x; k < L.n_slabs; k += kReduceThreads) { a0 += p[2 * k]; a1 += p[2 * k + 1]; }
      sh[0][threadIdx.x] = a0;
      sh[1][threadIdx.x] = a1;
      __syncthreads();
      for (int o = kReduceThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
          sh[0][threadIdx.x] += sh[0][threadIdx.x + o];
          sh[1][threadIdx.x] += sh[1][threadIdx.x + o];
        }
        __syncthreads();
      }
      t0 += sh[0][0];
      t1 += sh[1][0];
      __syncthreads();
    }
    if (threadIdx.x == 0) { rq.sums[2 * s] = t0; rq.sums[2 * s + 1] = t1; }
  }
}

// mu_k of the requests that finish in this round, from their step sums
// (step 0: mu_0, mu_1; step s: <v_s|v_s>, <v_s|v_s-1>), into pinned host memory.
__global__ void srv_finish_kernel(const SHdr* __restrict__ hdr, const SReq* __restrict__ reqs) {
  for (int32_t q = blockIdx.x; q < hdr->n_reqs; q += gridDim.x) {
    const SReq rq = reqs[q];
    if (!rq.finishing) continue;
    const double* sums = rq.sums;
    const double mu0 = sums[0], mu1 = sums[1];
    for (int32_t k = threadIdx.x; k < rq.n_mom; k += blockDim.x) {
      double v;
      if (k == 0) v = mu0;
      else if (k == 1) v = mu1;
      else if (k & 1) v = 2.0 * sums[2 * ((k + 1) >> 1) + 1] - mu1;
      else v = 2.0 * sums[2 * (k >> 1)] - mu0;
      rq.mu[k] = v;
    }
  }
}

// Synthetic width-4 ELL for the launch-shape tuner: row r couples to r +- 1 and
// r +- 257 (mod n), value 0.25, diagonal 0.1 (a 2D-like gather pattern).
template <typename F>
__global__ void srv_synth_ell_kernel(int32_t n, int32_t n_slices, int32_t* soff, int32_t* ecol, F* eval, F* diag) {
  const int32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r <= n_slices && r >= 0) soff[r] = r * 32 * 4;
  if (r >= n_slices * 32) return;
  const int32_t s = r >> 5, l = r & 31;
  const int32_t d[4] = {1, n - 1, 257 % n, n - 257 % n};
  for (int k = 0; k < 4; ++k) {
    const int64_t e = (int64_t)s * 32 * 4 + k * 32 + l;
    ecol[e] = r < n ? (int32_t)(((int64_t)r + d[k]) % n) : r;
    eval[e] = r < n ? F(0.25) : F(0);
  }
  diag[r] = r < n ? F(0.1) : F(0);
}

struct LaunchArgs {
  const SHdr* hdr;
  const SLane* lanes;
  const STile* tiles;
  double* part;
  int32_t code, j, reverse, pf, slab_cap, grid;
};
template <typename F, int R, bool C, bool K>
int srv_launch(const LaunchArgs& a, cudaStream_t st) {
  srv_step_kernel<F, R, C, K><<<a.grid, kSrvThreads, 0, st>>>(a.hdr, a.lanes, a.tiles, a.code, a.j, a.reverse, a.pf,
                                                             a.part, a.slab_cap);
  TBK_CHECK_LAUNCH();
  return TBK_OK;
}
template <typename F, int R, bool C, bool K>
int srv_occ() {
  int nb = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, srv_step_kernel<F, R, C, K>, kSrvThreads, 0);
  return nb > 0 ? nb : 1;
}
// tiles of a lane of n rows (slab_rows rows per slab)
inline int32_t srv_lane_tiles(int32_t n, int32_t slab_rows) {
  const int64_t tr = (int64_t)slab_rows * kSrvWarps;
  return (int32_t)(((int64_t)n + tr - 1) / tr);
}
using LaunchFn = int (*)(const LaunchArgs&, cudaStream_t);
using OccFn = int (*)();
struct GroupFns {
  LaunchFn launch = nullptr;
  OccFn occ = nullptr;
};
template <typename F, bool C, bool K>
GroupFns fns_for(int rc) {
  switch (rc) {
    case 1: return {srv_launch<F, 1, C, K>, srv_occ<F, 1, C, K>};
    case 2: return {srv_launch<F, 2, C, K>, srv_occ<F, 2, C, K>};
    case 4: return {srv_launch<F, 4, C, K>, srv_occ<F, 4, C, K>};
    case 8: return {srv_launch<F, 8, C, K>, srv_occ<F, 8, C, K>};
    case 16: return {srv_launch<F, 16, C, K>, srv_occ<F, 16, C, K>};
    case 32: return {srv_launch<F, 32, C, K>, srv_occ<F, 32, C, K>};
    case 64:
      if constexpr (sizeof(F) == 4) return {srv_launch<F, 64, C, K>, srv_occ<F, 64, C, K>};
      break;
  }
  return {};
}
int code_prec(int code) { return code >> 5; }
int code_width(int code) { return 1 << ((code >> 2) & 7); }
bool code_cplx(int code) { return (code & 2) != 0; }
bool code_cls(int code) { return (code & 1) != 0; }
int group_code(int prec, int rc, bool cplx, bool cls) {
  int lg = 0;
  while ((1 << lg) < rc) ++lg;
  return (((prec * 8) + lg) * 2 + (cplx ? 1 : 0)) * 2 + (cls ? 1 : 0);
}
template <typename F>
GroupFns fns_prec(int rc, bool c, bool k) {
  if (k) return c ? fns_for<F, true, true>(rc) : fns_for<F, false, true>(rc);
  return c ? fns_for<F, true, false>(rc) : fns_for<F, false, false>(rc);
}
GroupFns group_fns(int code) {
  const int rc = code_width(code);
  const bool c = code_cplx(code), k = code_cls(code);
  if (code_prec(code) == TBK_PREC_MIXED) return fns_prec<float>(rc, c, k);
  if (code_prec(code) == TBK_PREC_DD) return fns_prec<dd>(rc, c, k);
  return fns_prec<double>(rc, c, k);
}
int width_for(int prec, int R) {
  const int rmax = prec == TBK_PREC_MIXED ? 64 : 32;
  int rc = 1;
  while (rc < R && rc < rmax) rc <<= 1;
  return rc;
}
int32_t steps_for(int32_t n_mom) { return n_mom <= 2 ? 1 : n_mom / 2 + 1; }

using Clock = std::chrono::steady_clock;

struct Footprint {
  int64_t peak = 0, resident = 0, step_bytes = 0;
};

int check_request(const tbk_request* q) {
  if (!q || !q->lattice) return fail(TBK_ERR_INVALID, "request: null argument");
  if (q->kind < TBK_REQ_DOS || q->kind > TBK_REQ_KUBO_GREENWOOD) return fail(TBK_ERR_INVALID, "unknown request kind %d", q->kind);
  if (q->kind != TBK_REQ_DOS) {
    const int dim = q->lattice->cell.dim;
    for (int k = 0; k < 2; ++k)
      if (q->axis[k] < 0 || q->axis[k] >= dim) return fail(TBK_ERR_INVALID, "Error: axis out of range.");
    if (q->kernel < 0 || q->kernel > 5) return fail(TBK_ERR_INVALID, "unknown kernel %d", q->kernel);
  }
  if (q->n_mom < 2) return fail(TBK_ERR_INVALID, "n must be greater than or equal to 2");
  if (q->R < 1) return fail(TBK_ERR_INVALID, "R must be >= 1");
  if (q->precision != TBK_PREC_MIXED && q->precision != TBK_PREC_FP64 && q->precision != TBK_PREC_DD)
    return fail(TBK_ERR_INVALID, "unknown precision %d", q->precision);
  if (q->build_mode < 0 || q->build_mode > 2) return fail(TBK_ERR_INVALID, "unknown build mode %d", q->build_mode);
  if (!(q->e_max > q->e_min)) return fail(TBK_ERR_INVALID, "spectral bounds need e_max > e_min");
  if (q->lattice->total < 1) return fail(TBK_ERR_INVALID, "empty lattice");
  if (q->lattice->total > INT32_MAX / 2) return fail(TBK_ERR_UNSUPPORTED, "lattice too large for int32 indices");
  return TBK_OK;
}

// Bytes the request holds at each phase of its build and once resident.  Entry
// bounds: a site of atom a has at most deg(a) = #hopping terms touching a
// off-diagonal entries, plus the diagonal.
static_assert(sizeof(tbk_request) == 96, "tbk_request layout is part of the C ABI");

int kubo_chunk(int R) {
  int c = 1;
  while (c < R && c < 32) c <<= 1;
  return c;
}

Footprint footprint_of(const tbk_request& q, const tbk_lattice_s& L);

// Conductivity request: matrices (H, H~, two position diagonals, two
// commutators, their ELLs), both stored block sides at the chunk width that
// fits the budget, the work blocks and the mu_nm accumulators.
Footprint kubo_footprint(const tbk_request& q, const tbk_lattice_s& L, double budget, int* chunk) {
  tbk_request d = q;
  d.kind = TBK_REQ_DOS;
  d.precision = TBK_PREC_DD;
  const Footprint base = footprint_of(d, L);          // one matrix built, rescaled and in ELL form
  const int64_t Np = (L.total + 31) / 32 * 32;
  const int64_t M = q.n_mom;
  int rc = kubo_chunk(q.R);
  auto total = [&](int c) {
    const int64_t stores = 2 * M * (Np * c + 16) * 8;
    const int64_t work = 12 * Np * c * 16;
    return 4 * base.peak + stores + work + 4 * M * M * 16 + (64 << 20);
  };
  while (rc > 1 && (double)total(rc) > budget) rc >>= 1;
  *chunk = rc;
  Footprint f;
  f.peak = total(rc);
  f.resident = f.peak;
  f.step_bytes = 0;
  return f;
}

Footprint footprint_of(const tbk_request& q, const tbk_lattice_s& L) {
  const Cell& C = L.cell;
  const int64_t N = L.total;
  const int64_t cells = C.n_atoms > 0 ? N / C.n_atoms : 0;
  int64_t per_cell = 0;
  int64_t maxdeg = 0;
  for (int a = 0; a < C.n_atoms; ++a) {
    int64_t d = 0;
    for (const auto& h : C.hops) d += (h.from == a) + (h.to == a);
    per_cell += d + 1;
    maxdeg = std::max(maxdeg, d);
  }
  const bool mixed = q.precision == TBK_PREC_MIXED;
  const int64_t vs = q.is_complex ? 2 : 1;
  const int64_t hs = mixed ? 4 : 8;
  const int64_t nnz = cells * per_cell;
  const int64_t Np = (N + 31) / 32 * 32, NS = Np / 32;
  const int64_t E = Np * maxdeg + 32;
  auto csc = [&](int64_t z) { return 4 * (N + 2) + (z + 1) * (4 + 8 * vs); };
  int64_t fields = 8 * (N + 1) + 65536;
  if (L.gauge_kind == GAUGE_SITES) fields += 24 * N;
  if (L.scalar_kind == SCALAR_SITES) fields += 8 * N;
  if (!L.removed.empty()) fields += 9 * N;
  const int64_t build = csc(nnz) + fields;
  const int64_t rescale = csc(nnz) + csc(nnz + N) + 8 * (N + 1);
  // FP64 and FP32 values, plus the double-float copy for double-float requests
  const int64_t vals = q.precision == TBK_PREC_DD ? 20 : 12;
  const int64_t ell_all = 8 * (NS + 1) + (E + 32) * (4 + vals * vs) + Np * vals * vs;
  const int64_t ell = csc(nnz + N) + 12 * (N + 1) + 12 * (nnz + N + 1) + ell_all;
  const int64_t ell_keep = 4 * (NS + 1) + (E + 32) * (4 + hs * vs) + Np * hs * vs;
  const int rc = width_for(q.precision, q.R);
  const int64_t lanes = (q.R + rc - 1) / rc;
  const int64_t cs = mixed ? 8 : 16;
  const int64_t vec = lanes * 2 * Np * rc * cs;
  const int64_t resident = ell_keep + vec + 16 * (int64_t)steps_for(q.n_mom);
  Footprint f;
  f.peak = std::max({build, rescale, ell, resident});
  f.peak += f.peak / 32 + (2 << 20);                     // allocation rounding
  f.resident = resident;
  // bytes one full step moves: x, v_{n-1}, y and the matrix (as the recursion counts them)
  f.step_bytes = lanes * (3 * N * rc * cs + (E * (4 + hs * vs) + Np * hs * vs));
  return f;
}

struct Arena {   // first-fit allocator over the pinned result array (in doubles)
  std::map<int64_t, int64_t> free_;
  void init(int64_t n) { free_.clear(); if (n > 0) free_[0] = n; }
  bool can_take(int64_t n) const {
    for (const auto& kv : free_) if (kv.second >= n) return true;
    return false;
  }
  int64_t take(int64_t n) {
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= n) {
        const int64_t off = it->first, len = it->second;
        free_.erase(it);
        if (len > n) free_[off + n] = len - n;
        return off;
      }
    }
    return -1;
  }
  void give(int64_t off, int64_t n) {
    auto it = free_.emplace(off, n).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) { it->second += nx->second; free_.erase(nx); }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) { pv->second += it->second; free_.erase(it); }
    }
  }
};

enum { ST_QUEUED = 0, ST_BUILDING, ST_READY, ST_RUNNING, ST_DONE, ST_FAILED };

struct SrvRequest {
  int64_t ticket = 0;
  tbk_lattice_s lat;
  tbk_request q{};
  Footprint fp;
  int state = ST_QUEUED;
  int status = TBK_OK;
  std::string err;
  int64_t reserved = 0;
  tbk_sparse_s* Ht = nullptr;
  std::vector<DevBuf> vec;           // va, vb per lane
  DevBuf sums;
  int64_t mu_off = -1;
  int32_t rc = 0, cs = 0, n_lanes = 0, n_steps = 0, s0 = 0, code = 0, n = 0, slab_rows = 0;
  int32_t kubo_rc = 0;               // conductivity requests: vectors per stored chunk
  double step_bytes = 0.0;           // algorithmic bytes of one full step
  double mat_bytes = 0.0, vec_bytes = 0.0;
  std::vector<double> mu;
  double t_submit = 0, t_build0 = 0, t_ready = 0, t_done = 0;
  ~SrvRequest() { delete Ht; }
  void release_device() {
    delete Ht;
    Ht = nullptr;
    vec.clear();
    sums.release();
  }
};

struct Round {
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::vector<SrvRequest*> finishing;
  double bytes = 0.0;
  int64_t launches = 0;
};

}  // namespace
}  // namespace tbk

using namespace tbk;

struct tbk_server_s {
  int dev = 0;
  int sms = 152;
  int S = 16;
  // class form for requests whose H~ has row classes (the default;
  // TBK_SERVE_CLASSES=0 at create keeps every request in the ELL form)
  bool classes = true;
  double budget = 120e9, step_budget = 2e9;
  int max_resident = 4096;
  cudaStream_t st_loop = nullptr, st_admit = nullptr;
  cudaStream_t side[kGroups] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kGroups] = {};
  cudaMemPool_t pool = nullptr;
  AsyncAllocCtx actx;
  // round tables: one device copy, two pinned host staging copies
  int32_t cap_lanes = 0, cap_tiles = 0, cap_reqs = 0;
  size_t off_lanes = 0, off_tiles = 0, off_reqs = 0, tab_bytes = 0;
  DevBuf dtab, part;
  char* stage[2] = {nullptr, nullptr};
  cudaEvent_t copy_ev[2] = {nullptr, nullptr};
  bool copy_pending[2] = {false, false};
  std::map<std::pair<GroupMask, int>, cudaGraphExec_t> graphs;   // key: (group mask, round length)
  // launch shapes per group code
  int grid[kGroups] = {};
  int pf[kGroups] = {};
  double tune_ms[kGroups] = {};
  bool tuned[kGroups] = {};
  // requests
  std::mutex mu;
  // graph capture and device builds never overlap: a build's first launch of a
  // kernel may load its module, which CUDA refuses while any stream captures
  std::mutex capture_mu;
  std::condition_variable cv_admit, cv_loop, cv_done;
  std::deque<SrvRequest*> queued, ready;
  std::unordered_map<int64_t, std::unique_ptr<SrvRequest>> all;
  int64_t next_ticket = 1;
  bool stop = false;
  bool broken = false;
  std::string broken_msg;
  int64_t reserved = 0, peak_reserved = 0;
  int32_t n_held = 0, peak_held = 0;     // requests holding device memory
  double* arena_host = nullptr;
  int64_t arena_len = 0;
  Arena arena;
  // counters
  int64_t n_done = 0, n_failed = 0, n_rounds = 0, n_graphs = 0, n_launches = 0;
  double busy_ms = 0.0, bytes = 0.0, updates = 0.0, build_ms = 0.0;
  int64_t overshoot = INT64_MIN;
  Clock::time_point epoch;
  std::thread th_admit, th_loop;

  double now_ms() const { return std::chrono::duration<double, std::milli>(Clock::now() - epoch).count(); }
};

namespace tbk {
namespace {

void finish_request(tbk_server_s* S, SrvRequest* r, int status, const std::string& msg) {
  // caller holds S->mu
  if (r->mu_off >= 0) { S->arena.give(r->mu_off, r->q.n_mom); r->mu_off = -1; }
  r->release_device();
  if (r->reserved) {
    S->reserved -= r->reserved;
    r->reserved = 0;
    S->n_held -= 1;
  }
  r->status = status;
  r->err = msg;
  r->state = status == TBK_OK ? ST_DONE : ST_FAILED;
  r->t_done = S->now_ms();
  if (status == TBK_OK) ++S->n_done;
  else ++S->n_failed;
}

// ------------------------------------------------------------------ admission
int build_request(tbk_server_s* S, SrvRequest* r) {
  cudaStream_t st = S->st_admit;
  const tbk_request& q = r->q;
  TBK_CUDA(cudaStreamSynchronize(st));
  size_t used0 = 0, zero = 0;
  cudaMemPoolGetAttribute(S->pool, cudaMemPoolAttrUsedMemCurrent, &used0);
  cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrUsedMemHigh, &zero);
  tbk_sparse H = nullptr, Ht = nullptr;
  TBK_TRY(tbk_build_hamiltonian(&H, &r->lat, q.build_mode, q.extend, q.is_complex, st));
  const double a = (q.e_max - q.e_min) / 2.0, b = (q.e_max + q.e_min) / 2.0;
  int s = tbk_sparse_rescale(&Ht, H, a, b, st);
  delete H;
  if (s != TBK_OK) return s;
  r->Ht = Ht;
  TBK_TRY(ensure_ell(Ht, st));
  // keep what the recursion reads: the ELL (or the row classes) in the request's precision
  Ht->col_ptr.release();
  Ht->row_idx.release();
  Ht->values.release();
  if (S->classes) TBK_TRY(ensure_classes(Ht, st));
  const bool mixed = q.precision == TBK_PREC_MIXED;
  const bool cls = Ht->ell.cls_state == 1;
  if (q.precision == TBK_PREC_DD) TBK_TRY(ensure_ell_dd(Ht, st));
  if (q.precision != TBK_PREC_FP64) { Ht->ell.val64.release(); Ht->ell.diag64.release(); Ht->ell.cls_v64.release(); }
  if (!mixed) { Ht->ell.val32.release(); Ht->ell.diag32.release(); Ht->ell.cls_v32.release(); }
  if (q.precision != TBK_PREC_DD) Ht->ell.cls_vdd.release();
  if (cls) {                                  // the class form reads no ELL columns or values
    Ht->ell.col.release();
    Ht->ell.val64.release();
    Ht->ell.val32.release();
    Ht->ell.valdd.release();
  }
  r->n = Ht->rows;
  r->rc = width_for(q.precision, q.R);
  r->cs = mixed ? 8 : 16;
  r->n_lanes = (q.R + r->rc - 1) / r->rc;
  r->n_steps = steps_for(q.n_mom);
  r->code = group_code(q.precision, r->rc, Ht->ell.cplx != 0, cls);
  r->slab_rows = srv_slab_rows(r->cs, r->rc, r->n);
  const int64_t Np = (int64_t)Ht->ell.n_slices * 32;
  const size_t blk = (size_t)Np * r->rc * r->cs;
  r->vec.resize(2 * (size_t)r->n_lanes);
  for (int32_t c = 0; c < r->n_lanes; ++c) {
    TBK_TRY(r->vec[2 * c].alloc(blk));
    TBK_TRY(r->vec[2 * c + 1].alloc(blk));
    TBK_CUDA(cudaMemsetAsync(r->vec[2 * c].p, 0, blk, st));
    TBK_CUDA(cudaMemsetAsync(r->vec[2 * c + 1].p, 0, blk, st));
    TBK_TRY(random_block_any(q.precision, r->n, q.R, c * r->rc, r->rc, q.seed, r->vec[2 * c].p, st));
  }
  TBK_TRY(r->sums.alloc(sizeof(double) * 2 * (size_t)r->n_steps));
  TBK_CUDA(cudaStreamSynchronize(st));
  size_t high = 0;
  cudaMemPoolGetAttribute(S->pool, cudaMemPoolAttrUsedMemHigh, &high);
  const int64_t over = (int64_t)high - (int64_t)used0 - r->fp.peak;
  const EllDev& E = Ht->ell;
  int64_t held = (int64_t)(E.slice_off.bytes + E.col.bytes + E.val32.bytes + E.val64.bytes + E.valdd.bytes +
                           E.diag32.bytes + E.diag64.bytes + E.diagdd.bytes + E.cls.bytes + E.cls_cnt.bytes +
                           E.cls_off.bytes + E.cls_v32.bytes + E.cls_v64.bytes + E.cls_vdd.bytes + r->sums.bytes);
  for (auto& v : r->vec) held += (int64_t)v.bytes;
  const double hv = (mixed ? 4.0 : 8.0) * (E.cplx ? 2.0 : 1.0);
  // algorithmic matrix bytes of a step: the class byte and diagonal of each
  // row (class form) or the ELL columns, values and diagonal
  r->mat_bytes = cls ? (double)E.n_rows * (1.0 + hv)
                     : (double)E.n_entries * (4.0 + hv) + (double)E.n_rows * hv + 4.0 * (E.n_slices + 1);
  r->vec_bytes = (double)r->n * r->rc * r->cs;
  r->step_bytes = r->n_lanes * (3.0 * r->vec_bytes + r->mat_bytes);
  std::lock_guard<std::mutex> lk(S->mu);
  S->overshoot = std::max(S->overshoot, over);
  S->reserved += held - r->reserved;
  r->reserved = held;
  return TBK_OK;
}

// A conductivity request end to end on the admission stream: H~, the
// velocity commutators, mu_nm of tbk_kubo_mu with the stored blocks inside the
// request's reservation.
int run_kubo_request(tbk_server_s* S, SrvRequest* r) {
  cudaStream_t st = S->st_admit;
  const tbk_request& q = r->q;
  tbk_sparse H = nullptr, Ht = nullptr, X[2] = {nullptr, nullptr}, V[2] = {nullptr, nullptr};
  auto cleanup = [&] {
    for (tbk_sparse m : {H, Ht, X[0], X[1], V[0], V[1]}) if (m) tbk_sparse_destroy(m);
  };
  int s = tbk_build_hamiltonian(&H, &r->lat, q.build_mode, q.extend, q.is_complex, st);
  const double a = (q.e_max - q.e_min) / 2.0, b = (q.e_max + q.e_min) / 2.0;
  if (s == TBK_OK) s = tbk_sparse_rescale(&Ht, H, a, b, st);
  const int nops = q.kind == TBK_REQ_KUBO_BASTIN ? 2 : 1;
  for (int k = 0; k < nops && s == TBK_OK; ++k) {
    s = tbk_build_position(&X[k], &r->lat, q.axis[k], st);
    if (s == TBK_OK) s = tbk_sparse_commutator(&V[k], Ht, X[k], st);   // X H~ - H~ X
  }
  if (s != TBK_OK) {
    cleanup();
    return s;
  }
  const int32_t M = q.n_mom;
  r->mu.assign(2 * (size_t)M * M, 0.0);
  const int32_t flags = TBK_MU_TENSOR | (q.precision == TBK_PREC_MIXED ? TBK_MU_MIXED_RECURSION
                                         : q.precision == TBK_PREC_DD   ? TBK_MU_DD_RECURSION
                                                                        : 0);
  const double n_pad = (double)((Ht->rows + 31) / 32 * 32);
  const double stores_gb = 2.0 * M * (n_pad * r->kubo_rc + 16) * 8.0 / 1e9;
  if (q.kind == TBK_REQ_KUBO_BASTIN)
    s = tbk_kubo_mu(Ht, nullptr, nullptr, V[0], V[1], M, q.R, q.seed, nullptr, q.kernel, q.kernel_p0, q.kernel_p1,
                    flags, stores_gb, r->mu.data(), st);
  else
    s = tbk_kubo_mu(Ht, V[0], V[0], nullptr, nullptr, M, q.R, q.seed, nullptr, q.kernel, q.kernel_p0, q.kernel_p1,
                    flags, stores_gb, r->mu.data(), st);
  cleanup();
  return s;
}

void admit_main(tbk_server_s* S) {
  cudaSetDevice(S->dev);
  tl_async_alloc = &S->actx;
  for (;;) {
    SrvRequest* r = nullptr;
    {
      std::unique_lock<std::mutex> lk(S->mu);
      S->cv_admit.wait(lk, [&] {
        if (S->stop) return true;
        if (S->queued.empty()) return false;
        SrvRequest* h = S->queued.front();
        return S->reserved + h->fp.peak <= (int64_t)S->budget && S->n_held < S->max_resident &&
               (h->q.kind != TBK_REQ_DOS || S->arena.can_take(h->q.n_mom));
      });
      if (S->stop) break;
      r = S->queued.front();
      S->queued.pop_front();
      if (r->q.kind == TBK_REQ_DOS) r->mu_off = S->arena.take(r->q.n_mom);
      r->reserved = r->fp.peak;
      S->reserved += r->reserved;
      S->peak_reserved = std::max(S->peak_reserved, S->reserved);
      S->n_held += 1;
      S->peak_held = std::max(S->peak_held, S->n_held);
      r->state = ST_BUILDING;
      r->t_build0 = S->now_ms();
    }
    int s;
    {
      std::lock_guard<std::mutex> cap(S->capture_mu);
      if (S->broken) s = TBK_ERR_CUDA;
      else if (r->q.kind != TBK_REQ_DOS) s = run_kubo_request(S, r);
      else s = build_request(S, r);
    }
    const std::string msg = s == TBK_OK ? std::string() : std::string(tbk_last_error());
    if (r->q.kind != TBK_REQ_DOS) {                  // conductivity: done (or failed) here
      {
        std::lock_guard<std::mutex> lk(S->mu);
        r->t_ready = S->now_ms();
        S->build_ms += r->t_ready - r->t_build0;
        finish_request(S, r, s, s == TBK_OK ? std::string() : (S->broken ? S->broken_msg : msg));
      }
      S->cv_done.notify_all();
      S->cv_admit.notify_all();
      continue;
    }
    {
      std::lock_guard<std::mutex> lk(S->mu);
      r->t_ready = S->now_ms();
      S->build_ms += r->t_ready - r->t_build0;
      if (s == TBK_OK) {
        r->state = ST_READY;
        S->ready.push_back(r);
      } else {
        finish_request(S, r, s, S->broken ? S->broken_msg : msg);
      }
    }
    if (s == TBK_OK) S->cv_loop.notify_one();
    else { S->cv_done.notify_all(); S->cv_admit.notify_all(); }
  }
  cudaStreamSynchronize(S->st_admit);
  tl_async_alloc = nullptr;
}

// ------------------------------------------------------------------ rounds
int ensure_tables(tbk_server_s* S, int32_t lanes, int32_t tiles, int32_t reqs) {
  if (lanes <= S->cap_lanes && tiles <= S->cap_tiles && reqs <= S->cap_reqs && S->dtab.p) return TBK_OK;
  const int32_t cl = std::max(lanes, std::max(64, S->cap_lanes * 2));
  const int32_t cs = std::max(tiles, std::max(1024, S->cap_tiles * 2));
  const int32_t cr = std::max(reqs, std::max(64, S->cap_reqs * 2));
  auto up = [](size_t x) { return (x + 255) & ~(size_t)255; };
  S->off_lanes = up(sizeof(SHdr));
  S->off_tiles = S->off_lanes + up(sizeof(SLane) * cl);
  S->off_reqs = S->off_tiles + up(sizeof(STile) * cs);
  S->tab_bytes = S->off_reqs + up(sizeof(SReq) * cr);
  // graphs hold the old addresses
  for (auto& kv : S->graphs) cudaGraphExecDestroy(kv.second);
  S->graphs.clear();
  for (int b = 0; b < 2; ++b) {
    if (S->copy_pending[b]) { TBK_CUDA(cudaEventSynchronize(S->copy_ev[b])); S->copy_pending[b] = false; }
    if (S->stage[b]) cudaFreeHost(S->stage[b]);
    S->stage[b] = nullptr;
    TBK_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&S->stage[b]), S->tab_bytes, cudaHostAllocDefault));
  }
  TBK_TRY(S->dtab.alloc(S->tab_bytes));
  TBK_TRY(S->part.alloc(sizeof(double) * 2 * (size_t)cs * kSrvWarps * S->S));   // one partial pair per slab
  S->cap_lanes = cl;
  S->cap_tiles = cs;
  S->cap_reqs = cr;
  return TBK_OK;
}

int capture_graph(tbk_server_s* S, GroupMask mask, int steps, cudaGraphExec_t* out) {
  const std::pair<GroupMask, int> key(mask, steps);
  auto it = S->graphs.find(key);
  if (it != S->graphs.end()) { *out = it->second; return TBK_OK; }
  std::lock_guard<std::mutex> cap(S->capture_mu);
  cudaStream_t st = S->st_loop;
  const char* base = S->dtab.as<char>();
  LaunchArgs a;
  a.hdr = reinterpret_cast<const SHdr*>(base);
  a.lanes = reinterpret_cast<const SLane*>(base + S->off_lanes);
  a.tiles = reinterpret_cast<const STile*>(base + S->off_tiles);
  a.part = S->part.as<double>();
  a.slab_cap = S->cap_tiles * kSrvWarps;
  TBK_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
  int rc = TBK_OK;
  cudaError_t e = cudaEventRecord(S->ev_fork, st);
  for (int code = 0; code < kGroups && e == cudaSuccess && rc == TBK_OK; ++code) {
    if (!(mask & group_bit(code))) continue;
    const GroupFns fn = group_fns(code);
    if (!fn.launch) { rc = fail(TBK_ERR_UNSUPPORTED, "group %d not instantiated", code); break; }
    cudaStream_t sd = S->side[code];
    e = cudaStreamWaitEvent(sd, S->ev_fork, 0);
    a.code = code;
    a.grid = S->grid[code];
    a.pf = S->pf[code];
    for (int j = 0; j < steps && e == cudaSuccess && rc == TBK_OK; ++j) {
      a.j = j;
      a.reverse = j & 1;
      rc = fn.launch(a, sd);
    }
    if (e == cudaSuccess) e = cudaEventRecord(S->ev_join[code], sd);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, S->ev_join[code], 0);
  }
  if (e == cudaSuccess && rc == TBK_OK) {
    srv_reduce_kernel<<<S->sms * 8, kReduceThreads, 0, st>>>(a.hdr, a.lanes, reinterpret_cast<const SReq*>(base + S->off_reqs),
                                                 a.part, a.slab_cap, steps);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && rc == TBK_OK) {
    srv_finish_kernel<<<S->sms, 256, 0, st>>>(a.hdr, reinterpret_cast<const SReq*>(base + S->off_reqs));
    e = cudaGetLastError();
  }
  cudaGraph_t g = nullptr;
  cudaError_t e2 = cudaStreamEndCapture(st, &g);
  if (rc != TBK_OK) { if (g) cudaGraphDestroy(g); return rc; }
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return fail(TBK_ERR_CUDA, "round capture: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
  }
  cudaGraphExec_t x = nullptr;
  e = cudaGraphInstantiate(&x, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) return fail(TBK_ERR_CUDA, "round instantiate: %s", cudaGetErrorString(e));
  S->graphs[key] = x;
  ++S->n_graphs;
  *out = x;
  return TBK_OK;
}

int reap(tbk_server_s* S, Round& rd) {
  TBK_CUDA(cudaEventSynchronize(rd.ev1));
  float ms = 0.f;
  cudaEventElapsedTime(&ms, rd.ev0, rd.ev1);
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->busy_ms += ms;
    S->bytes += rd.bytes;
    S->n_launches += rd.launches;
    ++S->n_rounds;
    for (SrvRequest* r : rd.finishing) {
      r->mu.assign(S->arena_host + r->mu_off, S->arena_host + r->mu_off + r->q.n_mom);
      S->updates += (double)r->n * r->q.R * r->q.n_mom;
      finish_request(S, r, TBK_OK, std::string());
    }
  }
  cudaEventDestroy(rd.ev0);
  cudaEventDestroy(rd.ev1);
  rd.ev0 = rd.ev1 = nullptr;
  if (!rd.finishing.empty()) { S->cv_done.notify_all(); S->cv_admit.notify_all(); }
  return TBK_OK;
}

// Plans and launches one round over `run`; requests that finish move to rd.finishing.
int launch_round(tbk_server_s* S, std::vector<SrvRequest*>& run, std::deque<Round>& inflight, int64_t round_id) {
  std::vector<SrvRequest*> order(run);
  std::stable_sort(order.begin(), order.end(), [](SrvRequest* a, SrvRequest* b) { return a->code < b->code; });
  // round length: S, or the next power of two covering the longest remainder
  // (so that a lone short tail does not run empty launches)
  int32_t left = 0;
  for (SrvRequest* r : run) left = std::max(left, r->n_steps - r->s0);
  int32_t RS = 1;
  while (RS < left && RS < S->S) RS <<= 1;
  RS = std::min(RS, S->S);
  int32_t n_lanes = 0, n_tiles = 0;
  for (SrvRequest* r : order) {
    n_lanes += r->n_lanes;
    n_tiles += r->n_lanes * srv_lane_tiles(r->n, r->slab_rows);
  }
  const int32_t n_reqs = (int32_t)order.size();
  if (n_lanes > S->cap_lanes || n_tiles > S->cap_tiles || n_reqs > S->cap_reqs || !S->dtab.p) {
    while (!inflight.empty()) { TBK_TRY(reap(S, inflight.front())); inflight.pop_front(); }
    TBK_TRY(ensure_tables(S, n_lanes, n_tiles, n_reqs));
  }
  const int b = (int)(round_id & 1);
  if (S->copy_pending[b]) { TBK_CUDA(cudaEventSynchronize(S->copy_ev[b])); S->copy_pending[b] = false; }
  char* hb = S->stage[b];
  SHdr* hdr = reinterpret_cast<SHdr*>(hb);
  SLane* lanes = reinterpret_cast<SLane*>(hb + S->off_lanes);
  STile* tiles = reinterpret_cast<STile*>(hb + S->off_tiles);
  SReq* reqs = reinterpret_cast<SReq*>(hb + S->off_reqs);
  memset(hdr, 0, sizeof(SHdr));
  Round rd;
  GroupMask mask = 0;
  int32_t li = 0, si = 0;
  for (int32_t qi = 0; qi < n_reqs; ++qi) {
    SrvRequest* r = order[qi];
    const int code = r->code;
    if (!(mask & group_bit(code))) { mask |= group_bit(code); hdr->grp_begin[code] = si; }
    const int32_t sr = r->slab_rows;
    const int32_t steps = std::min(RS, r->n_steps - r->s0);
    SReq& q = reqs[qi];
    q.sums = r->sums.as<double>();
    q.mu = S->arena_host + r->mu_off;
    q.lane0 = li;
    q.n_lanes = r->n_lanes;
    q.s0 = r->s0;
    q.n_steps = r->n_steps;
    q.n_mom = r->q.n_mom;
    q.finishing = r->s0 + RS >= r->n_steps ? 1 : 0;
    const EllDev& E = r->Ht->ell;
    for (int32_t c = 0; c < r->n_lanes; ++c) {
      SLane& L = lanes[li];
      const int pq = r->q.precision;
      if (code_cls(r->code)) {
        L.soff = E.cls_cnt.as<int32_t>();
        L.ecol = E.cls_off.as<int32_t>();
        L.eval = pq == TBK_PREC_MIXED ? E.cls_v32.p : pq == TBK_PREC_DD ? E.cls_vdd.p : E.cls_v64.p;
        L.cls = E.cls.as<uint8_t>();
        L.cls_w = E.cls_w;
        L.n_cls = E.n_cls;
      } else {
        L.soff = E.slice_off.as<int32_t>();
        L.ecol = E.col.as<int32_t>();
        L.eval = pq == TBK_PREC_MIXED ? E.val32.p : pq == TBK_PREC_DD ? E.valdd.p : E.val64.p;
        L.cls = nullptr;
        L.cls_w = 0;
        L.n_cls = 0;
      }
      L.diag = pq == TBK_PREC_MIXED ? E.diag32.p : pq == TBK_PREC_DD ? E.diagdd.p : E.diag64.p;
      L.va = r->vec[2 * c].p;
      L.vb = r->vec[2 * c + 1].p;
      L.n = r->n;
      L.n_steps = r->n_steps;
      L.s0 = r->s0;
      L.req = qi;
      const int32_t nt = srv_lane_tiles(r->n, sr);
      L.slab_begin = si * kSrvWarps;
      L.n_slabs = nt * kSrvWarps;
      L.slab_rows = sr;
      for (int32_t k = 0; k < nt; ++k) tiles[si + k] = STile{li, k * sr * kSrvWarps};
      si += nt;
      ++li;
    }
    hdr->grp_count[code] = si - hdr->grp_begin[code];
    // algorithmic bytes of this request's steps in the round
    for (int32_t j = 0; j < steps; ++j) {
      const int32_t s = r->s0 + j;
      const bool dot_only = s == r->n_steps - 1 && s > 0;
      double bb = r->vec_bytes + (s > 0 ? r->vec_bytes : 0.0) + (dot_only ? 0.0 : r->vec_bytes + r->mat_bytes);
      rd.bytes += bb * r->n_lanes;
    }
    if (q.finishing) rd.finishing.push_back(r);
  }
  hdr->n_lanes = li;
  hdr->n_tiles = si;
  hdr->n_reqs = n_reqs;
  cudaGraphExec_t gx = nullptr;
  TBK_TRY(capture_graph(S, mask, RS, &gx));
  cudaStream_t st = S->st_loop;
  char* db = S->dtab.as<char>();
  TBK_CUDA(cudaMemcpyAsync(db, hb, sizeof(SHdr), cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemcpyAsync(db + S->off_lanes, lanes, sizeof(SLane) * li, cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemcpyAsync(db + S->off_tiles, tiles, sizeof(STile) * si, cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemcpyAsync(db + S->off_reqs, reqs, sizeof(SReq) * n_reqs, cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaEventRecord(S->copy_ev[b], st));
  S->copy_pending[b] = true;
  TBK_CUDA(cudaEventCreate(&rd.ev0));
  TBK_CUDA(cudaEventCreate(&rd.ev1));
  TBK_CUDA(cudaEventRecord(rd.ev0, st));
  TBK_CUDA(cudaGraphLaunch(gx, st));
  TBK_CUDA(cudaEventRecord(rd.ev1, st));
  int groups = 0;
  for (int c = 0; c < kGroups; ++c) groups += (int)((mask >> c) & 1u);
  rd.launches = (int64_t)groups * RS + 2;
  // advance: who is left for the next round
  std::vector<SrvRequest*> next;
  for (SrvRequest* r : run) {
    r->s0 += RS;
    if (r->s0 < r->n_steps) next.push_back(r);
  }
  run.swap(next);
  inflight.push_back(std::move(rd));
  return TBK_OK;
}

void fail_all(tbk_server_s* S, std::vector<SrvRequest*>& run, std::deque<Round>& inflight, const std::string& msg) {
  std::lock_guard<std::mutex> lk(S->mu);
  S->broken = true;
  S->broken_msg = msg;
  for (SrvRequest* r : run) finish_request(S, r, TBK_ERR_CUDA, msg);
  run.clear();
  for (Round& rd : inflight) {
    for (SrvRequest* r : rd.finishing) finish_request(S, r, TBK_ERR_CUDA, msg);
    if (rd.ev0) cudaEventDestroy(rd.ev0);
    if (rd.ev1) cudaEventDestroy(rd.ev1);
  }
  inflight.clear();
  while (!S->ready.empty()) { finish_request(S, S->ready.front(), TBK_ERR_CUDA, msg); S->ready.pop_front(); }
}

void loop_main(tbk_server_s* S) {
  cudaSetDevice(S->dev);
  std::vector<SrvRequest*> run;
  std::deque<Round> inflight;
  int64_t round_id = 0;
  for (;;) {
    {
      std::unique_lock<std::mutex> lk(S->mu);
      if (run.empty() && inflight.empty())
        S->cv_loop.wait(lk, [&] { return S->stop || !S->ready.empty(); });
      if (S->stop && inflight.empty()) break;
      if (!S->stop) {
        double step = 0.0;
        for (SrvRequest* r : run) step += r->step_bytes;
        while (!S->ready.empty() && (run.empty() || step + S->ready.front()->step_bytes <= S->step_budget)) {
          SrvRequest* r = S->ready.front();
          S->ready.pop_front();
          r->state = ST_RUNNING;
          step += r->step_bytes;
          run.push_back(r);
        }
      }
    }
    if (!run.empty() && !S->stop) {
      const int rc = launch_round(S, run, inflight, round_id++);
      if (rc != TBK_OK) {
        fail_all(S, run, inflight, tbk_last_error());
        S->cv_done.notify_all();
        S->cv_admit.notify_all();
        continue;
      }
    }
    // keep one round queued behind the running one; wait for the older
    const size_t keep = (run.empty() || S->stop) ? 0 : 1;
    while (inflight.size() > keep) {
      const int rc = reap(S, inflight.front());
      inflight.pop_front();
      if (rc != TBK_OK) { fail_all(S, run, inflight, tbk_last_error()); break; }
    }
  }
  // stop: what is still running fails
  std::lock_guard<std::mutex> lk(S->mu);
  for (SrvRequest* r : run) finish_request(S, r, TBK_ERR_INVALID, "server stopped");
}

// Times each candidate launch shape of every real group on a synthetic width-4
// operator of ~256 MB per vector block — two blocks exceed the 129 MB L2, as
// the requests that dominate the traffic do, so that the L2 prefetch mode
// is chosen on DRAM streams (TBK_SERVE_TUNE_MB overrides) — and keeps
// the fastest (grid, prefetch mode: none, the tile's own v_s rows, or the
// next wave's tile).  Each width is tuned twice: through
// the synthetic ELL, and in the class form with the same couplings as one
// class (offsets +-1, +-257, clamped at the ends of the block); the complex-H
// group of the same width and form takes the same shape.
int autotune(tbk_server_s* S) {
  cudaStream_t st = S->st_loop;
  cudaEvent_t e0, e1;
  TBK_CUDA(cudaEventCreate(&e0));
  TBK_CUDA(cudaEventCreate(&e1));
  int rc_all = TBK_OK;
  for (int prec = 0; prec < 3 && rc_all == TBK_OK; ++prec) {
    for (int rc = 4; rc <= (prec == TBK_PREC_MIXED ? 64 : 32) && rc_all == TBK_OK; rc <<= 1) {
      const int cs = prec == TBK_PREC_MIXED ? 8 : 16;
      int64_t tune_mb = 256;
      if (const char* ev = getenv("TBK_SERVE_TUNE_MB")) tune_mb = std::max(1, atoi(ev));   // tuning override
      int32_t n = (int32_t)((tune_mb << 20) / ((int64_t)rc * cs));
      const int sr = srv_slab_rows(cs, rc, n);
      const int32_t tr = sr * kSrvWarps;                      // rows per tile
      n = std::max(tr, n / tr * tr);
      const int32_t ns = n / 32, n_tile = n / tr;
      DevBuf soff, ecol, eval, diag, va, vb, tab, prt, ccnt, coff, cval, cls;
      const size_t fs = prec == TBK_PREC_MIXED ? 4 : 8;
      if ((rc_all = soff.alloc(4 * (size_t)(ns + 1))) || (rc_all = ecol.alloc(4 * 128 * (size_t)ns)) ||
          (rc_all = eval.alloc(fs * 128 * (size_t)ns)) || (rc_all = diag.alloc(fs * 32 * (size_t)ns)) ||
          (rc_all = va.alloc((size_t)n * rc * cs)) || (rc_all = vb.alloc((size_t)n * rc * cs)) ||
          (rc_all = prt.alloc(sizeof(double) * 2 * (size_t)n_tile * kSrvWarps)) || (rc_all = ccnt.alloc(sizeof(int32_t))) ||
          (rc_all = coff.alloc(4 * sizeof(int32_t))) || (rc_all = cval.alloc(4 * fs)) ||
          (rc_all = cls.alloc((size_t)n)))
        break;
      const int T = 256;
      if (prec == TBK_PREC_MIXED)
        srv_synth_ell_kernel<float><<<(ns * 32 + T) / T, T, 0, st>>>(n, ns, soff.as<int32_t>(), ecol.as<int32_t>(),
                                                                    eval.as<float>(), diag.as<float>());
      else if (prec == TBK_PREC_DD)
        srv_synth_ell_kernel<dd><<<(ns * 32 + T) / T, T, 0, st>>>(n, ns, soff.as<int32_t>(), ecol.as<int32_t>(),
                                                                 eval.as<dd>(), diag.as<dd>());
      else
        srv_synth_ell_kernel<double><<<(ns * 32 + T) / T, T, 0, st>>>(n, ns, soff.as<int32_t>(), ecol.as<int32_t>(),
                                                                     eval.as<double>(), diag.as<double>());
      TBK_CUDA(cudaGetLastError());
      {
        const int32_t hc = 4, ho[4] = {1, -1, 257, -257};
        const float v32[4] = {0.25f, 0.25f, 0.25f, 0.25f};
        const double v64[4] = {0.25, 0.25, 0.25, 0.25};
        const float vdd[8] = {0.25f, 0.f, 0.25f, 0.f, 0.25f, 0.f, 0.25f, 0.f};   // (hi, lo) pairs
        const void* hv = prec == TBK_PREC_MIXED ? (const void*)v32 : prec == TBK_PREC_DD ? (const void*)vdd
                                                                                        : (const void*)v64;
        TBK_CUDA(cudaMemcpyAsync(ccnt.p, &hc, sizeof(hc), cudaMemcpyHostToDevice, st));
        TBK_CUDA(cudaMemcpyAsync(coff.p, ho, sizeof(ho), cudaMemcpyHostToDevice, st));
        TBK_CUDA(cudaMemcpyAsync(cval.p, hv, 4 * fs, cudaMemcpyHostToDevice, st));
        TBK_CUDA(cudaMemsetAsync(cls.p, 0, cls.bytes, st));
      }
      TBK_CUDA(cudaMemsetAsync(vb.p, 0, vb.bytes, st));
      TBK_TRY(random_block_any(prec, n, rc, 0, rc, 7, va.p, st));
      const size_t off_l = (sizeof(SHdr) + 255) & ~(size_t)255, off_s = off_l + ((sizeof(SLane) + 255) & ~(size_t)255);
      TBK_TRY(tab.alloc(off_s + sizeof(STile) * (size_t)n_tile));
      for (int form = 0; form < 2; ++form) {
        const bool cf = form == 1;
        const int code = group_code(prec, rc, false, cf);
        const GroupFns fn = group_fns(code);
        // table: one lane at step 1 of a long recursion, all its tiles in group `code`
        std::vector<char> h(off_s + sizeof(STile) * (size_t)n_tile, 0);
        SHdr* hd = reinterpret_cast<SHdr*>(h.data());
        hd->grp_begin[code] = 0;
        hd->grp_count[code] = n_tile;
        hd->n_lanes = 1;
        hd->n_tiles = n_tile;
        SLane* L = reinterpret_cast<SLane*>(h.data() + off_l);
        L->soff = cf ? ccnt.as<int32_t>() : soff.as<int32_t>();
        L->ecol = cf ? coff.as<int32_t>() : ecol.as<int32_t>();
        L->eval = cf ? cval.p : eval.p;
        L->cls = cf ? cls.as<uint8_t>() : nullptr;
        L->cls_w = cf ? 4 : 0;
        L->n_cls = cf ? 1 : 0;
        L->diag = diag.p;
        L->va = va.p;
        L->vb = vb.p;
        L->n = n;
        L->n_steps = 1 << 30;
        L->s0 = 1;
        L->slab_begin = 0;
        L->n_slabs = n_tile * kSrvWarps;
        L->slab_rows = sr;
        STile* tl = reinterpret_cast<STile*>(h.data() + off_s);
        for (int32_t k = 0; k < n_tile; ++k) tl[k] = STile{0, k * tr};
        TBK_CUDA(cudaMemcpyAsync(tab.p, h.data(), h.size(), cudaMemcpyHostToDevice, st));
        TBK_CUDA(cudaStreamSynchronize(st));
        LaunchArgs a;
        a.hdr = tab.as<SHdr>();
        a.lanes = reinterpret_cast<const SLane*>(tab.as<char>() + off_l);
        a.tiles = reinterpret_cast<const STile*>(tab.as<char>() + off_s);
        a.part = prt.as<double>();
        a.slab_cap = n_tile * kSrvWarps;
        a.code = code;
        a.j = 0;
        const int occ = fn.occ();
        const int grids[4] = {S->sms, 2 * S->sms, 4 * S->sms, occ * S->sms};
        double best = 1e30;
        for (int gi = 0; gi < 4; ++gi) {
          if (grids[gi] > occ * S->sms) continue;
          for (int pf = 0; pf <= 2; ++pf) {
            a.grid = grids[gi];
            a.pf = pf;
            for (int w = 0; w < 2; ++w) { a.reverse = w & 1; TBK_TRY(fn.launch(a, st)); }
            TBK_CUDA(cudaEventRecord(e0, st));
            for (int w = 0; w < 6; ++w) { a.reverse = w & 1; TBK_TRY(fn.launch(a, st)); }
            TBK_CUDA(cudaEventRecord(e1, st));
            TBK_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (ms / 6.0 < best) {
              best = ms / 6.0;
              S->grid[code] = a.grid;
              S->pf[code] = pf;
            }
          }
        }
        S->tune_ms[code] = best;
        S->tuned[code] = true;
        const int cc = group_code(prec, rc, true, cf);
        S->grid[cc] = S->grid[code];
        S->pf[cc] = S->pf[code];
      }
      TBK_CUDA(cudaStreamSynchronize(st));
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return rc_all;
}

void server_free(tbk_server_s* S) {
  if (S->st_loop) cudaStreamSynchronize(S->st_loop);
  if (S->st_admit) cudaStreamSynchronize(S->st_admit);
  for (auto& kv : S->all) kv.second->release_device();
  S->all.clear();
  for (auto& kv : S->graphs) cudaGraphExecDestroy(kv.second);
  S->graphs.clear();
  S->dtab.release();
  S->part.release();
  if (S->st_admit) cudaStreamSynchronize(S->st_admit);
  cudaDeviceSynchronize();
  for (int b = 0; b < 2; ++b) {
    if (S->stage[b]) cudaFreeHost(S->stage[b]);
    if (S->copy_ev[b]) cudaEventDestroy(S->copy_ev[b]);
  }
  if (S->arena_host) cudaFreeHost(S->arena_host);
  for (int g = 0; g < kGroups; ++g) {
    if (S->side[g]) cudaStreamDestroy(S->side[g]);
    if (S->ev_join[g]) cudaEventDestroy(S->ev_join[g]);
  }
  if (S->ev_fork) cudaEventDestroy(S->ev_fork);
  if (S->st_loop) cudaStreamDestroy(S->st_loop);
  if (S->st_admit) cudaStreamDestroy(S->st_admit);
  if (S->pool) cudaMemPoolDestroy(S->pool);
  delete S;
}

}  // namespace
}  // namespace tbk

extern "C" {

int tbk_request_footprint(const tbk_request* req, int64_t* build_peak_bytes, int64_t* resident_bytes) {
  TBK_TRY(check_request(req));
  int rc = 1;
  const Footprint f = req->kind == TBK_REQ_DOS ? footprint_of(*req, *req->lattice)
                                               : kubo_footprint(*req, *req->lattice, 120e9, &rc);
  if (build_peak_bytes) *build_peak_bytes = f.peak;
  if (resident_bytes) *resident_bytes = f.resident;
  return TBK_OK;
}

int tbk_server_create(tbk_server* out, const tbk_server_config* cfg) {
  if (!out) return fail(TBK_ERR_INVALID, "tbk_server_create: null argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) {
    cudaGetLastError();
    return fail(TBK_ERR_CUDA, "tbk_server_create: no CUDA device");
  }
  auto* S = new tbk_server_s();
  if (const char* e = getenv("TBK_SERVE_CLASSES")) S->classes = atoi(e) != 0;
  S->epoch = Clock::now();
  if (cfg) {
    if (cfg->budget_gb > 0) S->budget = cfg->budget_gb * 1e9;
    if (cfg->steps_per_round > 0) S->S = cfg->steps_per_round;
    if (cfg->max_resident > 0) S->max_resident = cfg->max_resident;
    if (cfg->step_gb > 0) S->step_budget = cfg->step_gb * 1e9;
  }
  const int arena_mb = (cfg && cfg->result_arena_mb > 0) ? cfg->result_arena_mb : 64;
  cudaGetDevice(&S->dev);
  S->sms = sm_count();
  auto bad = [&](cudaError_t e, const char* what) {
    int c = fail(TBK_ERR_CUDA, "tbk_server_create: %s: %s", what, cudaGetErrorString(e));
    server_free(S);
    return c;
  };
  cudaError_t e;
  if ((e = cudaStreamCreateWithFlags(&S->st_loop, cudaStreamNonBlocking)) != cudaSuccess) return bad(e, "stream");
  // builds run beside saturating rounds: their short kernels take SMs first
  int prio_lo = 0, prio_hi = 0;
  cudaDeviceGetStreamPriorityRange(&prio_lo, &prio_hi);
  if ((e = cudaStreamCreateWithPriority(&S->st_admit, cudaStreamNonBlocking, prio_hi)) != cudaSuccess)
    return bad(e, "stream");
  for (int g = 0; g < kGroups; ++g) {
    if ((e = cudaStreamCreateWithFlags(&S->side[g], cudaStreamNonBlocking)) != cudaSuccess) return bad(e, "stream");
    if ((e = cudaEventCreateWithFlags(&S->ev_join[g], cudaEventDisableTiming)) != cudaSuccess) return bad(e, "event");
  }
  if ((e = cudaEventCreateWithFlags(&S->ev_fork, cudaEventDisableTiming)) != cudaSuccess) return bad(e, "event");
  for (int b = 0; b < 2; ++b)
    if ((e = cudaEventCreateWithFlags(&S->copy_ev[b], cudaEventDisableTiming)) != cudaSuccess) return bad(e, "event");
  cudaMemPoolProps props;
  memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = S->dev;
  if ((e = cudaMemPoolCreate(&S->pool, &props)) != cudaSuccess) return bad(e, "memory pool");
  uint64_t keep = UINT64_MAX;
  cudaMemPoolSetAttribute(S->pool, cudaMemPoolAttrReleaseThreshold, &keep);
  S->actx.pool = S->pool;
  S->actx.stream = S->st_admit;
  S->arena_len = (int64_t)arena_mb * (1 << 20) / (int64_t)sizeof(double);
  if ((e = cudaHostAlloc(reinterpret_cast<void**>(&S->arena_host), sizeof(double) * S->arena_len,
                         cudaHostAllocMapped | cudaHostAllocPortable)) != cudaSuccess)
    return bad(e, "pinned result arena");
  S->arena.init(S->arena_len);
  for (int code = 0; code < kGroups; ++code) {
    const GroupFns fn = group_fns(code);
    S->grid[code] = fn.occ ? fn.occ() * S->sms : S->sms;
    S->pf[code] = 0;                     // untuned: no L2 prefetch (the tuner may pick one)
  }
  if (cfg && cfg->autotune) {
    const int s = autotune(S);
    if (s != TBK_OK) { server_free(S); return s; }
  }
  {
    const int s = ensure_tables(S, 64, 4096, 64);
    if (s != TBK_OK) { server_free(S); return s; }
  }
  S->th_admit = std::thread(admit_main, S);
  S->th_loop = std::thread(loop_main, S);
  *out = S;
  return TBK_OK;
}

void tbk_server_destroy(tbk_server S) {
  if (!S) return;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    S->stop = true;
  }
  S->cv_admit.notify_all();
  S->cv_loop.notify_all();
  if (S->th_admit.joinable()) S->th_admit.join();
  if (S->th_loop.joinable()) S->th_loop.join();
  {
    std::lock_guard<std::mutex> lk(S->mu);
    for (SrvRequest* r : S->queued) finish_request(S, r, TBK_ERR_INVALID, "server stopped");
    S->queued.clear();
    for (SrvRequest* r : S->ready) finish_request(S, r, TBK_ERR_INVALID, "server stopped");
    S->ready.clear();
  }
  S->cv_done.notify_all();
  server_free(S);
}

int tbk_server_submit(tbk_server S, const tbk_request* req, int64_t* ticket) {
  if (!S || !ticket) return fail(TBK_ERR_INVALID, "tbk_server_submit: null argument");
  *ticket = 0;
  TBK_TRY(check_request(req));
  auto r = std::make_unique<SrvRequest>();
  r->lat = *req->lattice;
  r->q = *req;
  r->q.lattice = nullptr;
  if (req->kind == TBK_REQ_DOS) {
    r->fp = footprint_of(*req, r->lat);
  } else {
    int rc = 1;
    r->fp = kubo_footprint(*req, r->lat, S->budget, &rc);
    r->kubo_rc = rc;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  if (S->broken) return fail(TBK_ERR_CUDA, "server failed: %s", S->broken_msg.c_str());
  if (S->stop) return fail(TBK_ERR_INVALID, "server stopped");
  if (r->fp.peak > (int64_t)S->budget)
    return fail(TBK_ERR_BUDGET, "request needs %lld bytes at its build peak, budget %.0f", (long long)r->fp.peak,
                S->budget);
  if (r->q.kind == TBK_REQ_DOS && r->q.n_mom > S->arena_len)
    return fail(TBK_ERR_BUDGET, "n_mom %d exceeds the result arena", r->q.n_mom);
  r->ticket = S->next_ticket++;
  r->t_submit = S->now_ms();
  *ticket = r->ticket;
  S->queued.push_back(r.get());
  S->all.emplace(r->ticket, std::move(r));
  S->cv_admit.notify_one();
  return TBK_OK;
}

int tbk_server_poll(tbk_server S, int64_t ticket, int32_t wait_ms, double* mu_out, double* times_ms) {
  if (!S) return fail(TBK_ERR_INVALID, "tbk_server_poll: null server");
  if (wait_ms < 0) return fail(TBK_ERR_INVALID, "wait_ms must be >= 0");
  std::unique_lock<std::mutex> lk(S->mu);
  auto it = S->all.find(ticket);
  if (it == S->all.end()) return fail(TBK_ERR_INVALID, "unknown ticket %lld", (long long)ticket);
  SrvRequest* r = it->second.get();
  S->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms),
                      [&] { return r->state == ST_DONE || r->state == ST_FAILED; });
  if (r->state != ST_DONE && r->state != ST_FAILED) return TBK_PENDING;
  if (times_ms) {
    times_ms[0] = (r->t_build0 > 0 ? r->t_build0 : r->t_done) - r->t_submit;
    times_ms[1] = r->t_build0 > 0 ? r->t_ready - r->t_build0 : 0.0;
    times_ms[2] = r->t_ready > 0 ? r->t_done - r->t_ready : 0.0;
    times_ms[3] = r->t_done - r->t_submit;
  }
  if (r->state == ST_FAILED) {
    const int st = r->status;
    const std::string msg = r->err;
    S->all.erase(it);
    return fail(st, "%s", msg.c_str());
  }
  if (mu_out) memcpy(mu_out, r->mu.data(), sizeof(double) * r->mu.size());
  S->all.erase(it);
  return TBK_OK;
}

int tbk_server_stats(tbk_server S, double* out, int32_t n) {
  if (!S || !out) return fail(TBK_ERR_INVALID, "tbk_server_stats: null argument");
  std::lock_guard<std::mutex> lk(S->mu);
  const double v[14] = {(double)S->n_done, (double)S->n_failed, (double)S->n_rounds, (double)S->n_graphs,
                        S->busy_ms, S->bytes, S->updates, (double)S->n_launches, S->budget,
                        (double)S->peak_reserved, (double)S->reserved, S->build_ms, (double)S->peak_held,
                        S->overshoot == INT64_MIN ? 0.0 : (double)S->overshoot};
  for (int32_t i = 0; i < n && i < 14; ++i) out[i] = v[i];
  return TBK_OK;
}

int tbk_server_tuning(tbk_server S, int32_t max_rows, double* rows) {
  if (!S || !rows) return fail(TBK_ERR_INVALID, "tbk_server_tuning: null argument");
  int k = 0;
  for (int code = 0; code < kGroups && k < max_rows; ++code) {
    if (!S->tuned[code]) continue;
    double* r = rows + 6 * k;
    r[0] = code_prec(code);
    r[1] = code_width(code);
    r[2] = code_cls(code) ? 1 : 0;
    r[3] = S->grid[code];
    r[4] = S->pf[code];
    r[5] = S->tune_ms[code];
    ++k;
  }
  return k;
}

}  // extern "C"
