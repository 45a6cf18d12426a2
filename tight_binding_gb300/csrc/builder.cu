// builder.cu — device-side lattice -> sparse Hamiltonian builder and the sparse
// transformations on the path (rescale, velocity commutator, sliced-ELL).
//
// The reference builds a triplet list on the host and calls Eigen's
// setFromTriplets (TB/lattice.h:216-305).  Here every CSC column is produced
// by one thread that enumerates exactly the triplets that land in it:
//   (a) direct triplets (row, col=j, t) of hoppings ending on site j, and
//   (b) conjugate triplets (col=j ... ) of hoppings starting on site j,
// sorts them by (row, position in the reference's triplet list) and sums
// duplicates in that order — which is setFromTriplets' semantics (sorted inner
// indices, duplicates summed in insertion order, explicit zeros kept).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "host_model.h"
#include "tbk_internal.h"

namespace tbk {

// ------------------------------------------------------------------ scans
constexpr int kScanThreads = 512;
constexpr int kScanItems = 4;
constexpr int kScanTile = kScanThreads * kScanItems;

template <typename T>
__global__ void __launch_bounds__(kScanThreads) scan_tile_kernel(const T* __restrict__ in, T* __restrict__ out,
                                                                 T* __restrict__ block_sums, int64_t n) {
  __shared__ T sh[kScanThreads];
  int64_t base = (int64_t)blockIdx.x * kScanTile + (int64_t)threadIdx.x * kScanItems;
  T v[kScanItems];
  T local = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : T(0);
    local += v[k];
  }
  sh[threadIdx.x] = local;
  __syncthreads();
  for (int off = 1; off < kScanThreads; off <<= 1) {
    T add = threadIdx.x >= off ? sh[threadIdx.x - off] : T(0);
    __syncthreads();
    sh[threadIdx.x] += add;
    __syncthreads();
  }
  T run = sh[threadIdx.x] - local;  // exclusive prefix of this thread
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) out[base + k] = run;
    run += v[k];
  }
  if (threadIdx.x == kScanThreads - 1 && block_sums) block_sums[blockIdx.x] = sh[threadIdx.x];
}

template <typename T>
__global__ void scan_add_kernel(T* __restrict__ out, const T* __restrict__ offs, int64_t n) {
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] += offs[i / kScanTile];
}

template <typename T>
static int exclusive_scan(const T* in, T* out, int64_t n, cudaStream_t st) {
  if (n <= 0) return TBK_OK;
  int64_t nb = (n + kScanTile - 1) / kScanTile;
  if (nb == 1) {
    scan_tile_kernel<T><<<1, kScanThreads, 0, st>>>(in, out, nullptr, n);
    TBK_CHECK_LAUNCH();
    return TBK_OK;
  }
  DevBuf sums, offs;
  TBK_TRY(sums.alloc(sizeof(T) * nb));
  TBK_TRY(offs.alloc(sizeof(T) * nb));
  scan_tile_kernel<T><<<(unsigned)nb, kScanThreads, 0, st>>>(in, out, sums.as<T>(), n);
  TBK_CHECK_LAUNCH();
  TBK_TRY(exclusive_scan<T>(sums.as<T>(), offs.as<T>(), nb, st));
  scan_add_kernel<T><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, offs.as<T>(), n);
  TBK_CHECK_LAUNCH();
  // keep the temporaries alive until the kernels ran
  TBK_CUDA(cudaStreamSynchronize(st));
  return TBK_OK;
}

template <typename T>
static int scan_with_total(const T* in, T* out, int64_t n, cudaStream_t st, T* total) {
  TBK_TRY(exclusive_scan<T>(in, out, n, st));
  if (total) {
    T last_in = 0, last_out = 0;
    if (n > 0) {
      TBK_CUDA(cudaMemcpyAsync(&last_in, in + n - 1, sizeof(T), cudaMemcpyDeviceToHost, st));
      TBK_CUDA(cudaMemcpyAsync(&last_out, out + n - 1, sizeof(T), cudaMemcpyDeviceToHost, st));
      TBK_CUDA(cudaStreamSynchronize(st));
    }
    *total = last_in + last_out;
  }
  return TBK_OK;
}

int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t st, int32_t* total) {
  return scan_with_total<int32_t>(in, out, n, st, total);
}
int exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t st, int64_t* total) {
  return scan_with_total<int64_t>(in, out, n, st, total);
}

int sm_count() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 152;
  }
  return sms;
}

// ------------------------------------------------------------------ ELL structure comparison
__global__ void diff_i32_kernel(int64_t n, const int32_t* __restrict__ a, const int32_t* __restrict__ b,
                                int* __restrict__ flag) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (a[i] != b[i]) *flag = 1;
}

int same_ell_structure(tbk_sparse_s* A, tbk_sparse_s* B, bool* same, cudaStream_t st) {
  *same = false;
  TBK_TRY(ensure_ell(A, st));
  TBK_TRY(ensure_ell(B, st));
  const EllDev& a = A->ell;
  const EllDev& b = B->ell;
  if (a.n_rows != b.n_rows || a.n_slices != b.n_slices || a.n_entries != b.n_entries || a.cplx != b.cplx)
    return TBK_OK;
  DevBuf flag;
  TBK_TRY(flag.alloc(sizeof(int)));
  TBK_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), st));
  const int g = 4 * sm_count();
  diff_i32_kernel<<<g, 256, 0, st>>>((int64_t)a.n_slices + 1, a.slice_off.as<int32_t>(), b.slice_off.as<int32_t>(),
                                     flag.as<int>());
  TBK_CHECK_LAUNCH();
  if (a.n_entries > 0) {
    diff_i32_kernel<<<g, 256, 0, st>>>(a.n_entries, a.col.as<int32_t>(), b.col.as<int32_t>(), flag.as<int>());
    TBK_CHECK_LAUNCH();
  }
  int h = 1;
  TBK_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  *same = h == 0;
  return TBK_OK;
}

// ------------------------------------------------------------------ vacancies
__global__ void keep_flags_kernel(int64_t n, const uint8_t* __restrict__ removed, int32_t* __restrict__ keep) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    keep[i] = removed[i] ? 0 : 1;
}
__global__ void scatter_comp_kernel(int64_t n, const uint8_t* __restrict__ removed, const int32_t* __restrict__ pos,
                                    int32_t* __restrict__ comp, int32_t* __restrict__ inv) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    if (removed[i]) {
      comp[i] = -1;
    } else {
      comp[i] = pos[i];
      inv[pos[i]] = (int32_t)i;
    }
  }
}

// bare -> compressed site map (comp, -1 where removed) and compressed -> bare
// (inv) from the removal mask: keep flags, exclusive scan, scatter
int compact_sites(const uint8_t* removed_host, int64_t n, DevBuf* comp, DevBuf* inv, int32_t* kept, cudaStream_t st) {
  DevBuf mask, keep, pos;
  TBK_TRY(mask.alloc(n));
  TBK_TRY(keep.alloc(sizeof(int32_t) * n));
  TBK_TRY(pos.alloc(sizeof(int32_t) * n));
  TBK_TRY(comp->alloc(sizeof(int32_t) * n));
  TBK_TRY(inv->alloc(sizeof(int32_t) * (n + 1)));
  TBK_CUDA(cudaMemcpyAsync(mask.p, removed_host, n, cudaMemcpyHostToDevice, st));
  const int g = std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 8 * sm_count()));
  keep_flags_kernel<<<g, 256, 0, st>>>(n, mask.as<uint8_t>(), keep.as<int32_t>());
  TBK_CHECK_LAUNCH();
  TBK_TRY(exclusive_scan_i32(keep.as<int32_t>(), pos.as<int32_t>(), n, st, kept));
  scatter_comp_kernel<<<g, 256, 0, st>>>(n, mask.as<uint8_t>(), pos.as<int32_t>(), comp->as<int32_t>(),
                                         inv->as<int32_t>());
  TBK_CHECK_LAUNCH();
  return TBK_OK;
}

// ------------------------------------------------------------------ builder
constexpr int kMaxCand = 64;   // triplets landing in one CSC column

struct DevHop {
  int32_t from, to;
  int32_t v[3];
  int32_t pad;
  double tr, ti;
};

struct BuildParams {
  int32_t dim, n_atoms, n_hops, mode, is_complex;
  int32_t span[3], extend[3];
  int64_t stride[3];            // bare index strides (atom fastest)
  int32_t n_cols;               // matrix size (= total_number)
  int32_t n_kept;               // columns carrying entries (vacancies compress)
  double bases[9];
  int32_t gauge_kind, scalar_kind;
  double gauge_linear[12];
  double disorder_W;
  uint64_t disorder_seed;
  const DevHop* hops;
  const double* pos;            // n_atoms x 3
  const double* gauge_sites;    // total x 3
  const double* scalar_sites;   // total
  const int32_t* comp;          // bare -> compressed (-1 removed), or null
  const int32_t* inv;           // compressed -> bare, or null
  int32_t* warn_flag;           // imaginary part discarded (real Scalar)
  int32_t vel_axis;             // >= 0: bond-displacement velocity along this axis instead of H
  double vel_scale;
};

__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

// t * exp(i A(r_from) . d_hop) and the on-site scalar field, evaluated operation
// by operation as the oracle does (no fused multiply-add).
__device__ void hop_value(const BuildParams& P, const DevHop& h, const int32_t* iv, int64_t rb,
                          bool same_site, double& tr, double& ti) {
  tr = h.tr;
  ti = h.ti;
  if (P.mode == TBK_BUILD_BARE) return;
  if (P.gauge_kind != GAUGE_NONE) {
    double A[3], d[3];
    if (P.gauge_kind == GAUGE_LINEAR) {
      double rf[3];
      for (int x = 0; x < 3; ++x) {
        double s = 0.0;
        for (int c = 0; c < P.dim; ++c) s = dadd(s, dmul(P.bases[c * 3 + x], (double)iv[c]));
        rf[x] = dadd(P.pos[h.from * 3 + x], s);
      }
      for (int x = 0; x < 3; ++x) {
        double s = 0.0;
        for (int y = 0; y < 3; ++y) s = dadd(s, dmul(P.gauge_linear[3 * x + y], rf[y]));
        A[x] = dadd(s, P.gauge_linear[9 + x]);
      }
    } else {
      for (int x = 0; x < 3; ++x) A[x] = P.gauge_sites[3 * rb + x];
    }
    for (int x = 0; x < 3; ++x) {
      double s = 0.0;
      for (int c = 0; c < P.dim; ++c) s = dadd(s, dmul(P.bases[c * 3 + x], (double)h.v[c]));
      d[x] = dadd(dadd(-P.pos[h.from * 3 + x], s), P.pos[h.to * 3 + x]);
    }
    double phi = dadd(dadd(dmul(A[0], d[0]), dmul(A[1], d[1])), dmul(A[2], d[2]));
    double sn, cs;
    sincos(phi, &sn, &cs);
    double nr = __dsub_rn(dmul(tr, cs), dmul(ti, sn));
    double ni = dadd(dmul(tr, sn), dmul(ti, cs));
    tr = nr;
    ti = ni;
  }
  if (same_site) {
    if (P.scalar_kind == SCALAR_SITES) tr = dadd(tr, P.scalar_sites[rb]);
    else if (P.scalar_kind == SCALAR_DISORDER)
      tr = dadd(tr, dmul(P.disorder_W, __dsub_rn(u01(P.disorder_seed, kDisorderStream, (uint64_t)rb), 0.5)));
  }
}

struct Cand {
  int32_t row;
  int64_t key;
  double re, im;
};

// Enumerates the triplets of CSC column j; returns the count (or -1 on overflow).
// component vel_axis of the hop's bond vector r_to - r_from (minimum image:
// the hop's own lattice vector, whatever the periodic wrap)
__device__ double bond_component(const BuildParams& P, const DevHop& h) {
  const int x = P.vel_axis;
  double s = 0.0;
  for (int c = 0; c < P.dim; ++c) s = dadd(s, dmul(P.bases[c * 3 + x], (double)h.v[c]));
  return dadd(dadd(-P.pos[h.from * 3 + x], s), P.pos[h.to * 3 + x]);
}

__device__ int column_candidates(const BuildParams& P, int32_t j, Cand* c, bool want_values) {
  if (j >= P.n_kept) return 0;
  int64_t bare = P.inv ? P.inv[j] : j;
  int32_t a = (int32_t)(bare % P.n_atoms);
  int64_t cell = bare / P.n_atoms;
  int32_t cj[3] = {0, 0, 0};
  {
    int64_t rem = cell;
    for (int x = P.dim - 1; x >= 0; --x) { cj[x] = (int32_t)(rem % P.span[x]); rem /= P.span[x]; }
  }
  const bool periodic = P.mode == TBK_BUILD_PERIODIC_BARE;
  int n = 0;
  for (int hi = 0; hi < P.n_hops; ++hi) {
    const DevHop h = P.hops[hi];
    // (a) direct triplet of hop hi started in cell iv = cj - delta, ending here
    if (h.to == a) {
      int32_t iv[3] = {0, 0, 0};
      bool ok = true;
      for (int x = 0; x < P.dim; ++x) {
        int32_t t = cj[x] - h.v[x];
        if (periodic && P.extend[x]) t = ((t % P.span[x]) + P.span[x]) % P.span[x];
        else if (t < 0 || t >= P.span[x]) ok = false;
        iv[x] = t;
      }
      if (ok) {
        int64_t rb = h.from;
        int64_t lin = 0;
        for (int x = 0; x < P.dim; ++x) { rb += iv[x] * P.stride[x]; lin = lin * P.span[x] + iv[x]; }
        int32_t row = (int32_t)rb;
        if (P.comp) { row = P.comp[rb]; if (row < 0) ok = false; }
        if (ok) {
          if (n >= kMaxCand) return -1;
          c[n].row = row;
          c[n].key = (lin * P.n_hops + hi) * 2;
          if (want_values) {
            double tr, ti;
            const bool vel = P.vel_axis >= 0;
            hop_value(P, h, iv, rb, !vel && rb == bare, tr, ti);
            if (vel) {                                   // (x_row - x_col) t with row = from, col = to
              const double f = dmul(-bond_component(P, h), P.vel_scale);
              tr = dmul(tr, f);
              ti = dmul(ti, f);
            }
            if (!P.is_complex) { if (fabs(ti) > 1e-10) atomicOr(P.warn_flag, 1); ti = 0.0; }
            c[n].re = tr;
            c[n].im = ti;
          }
          ++n;
        }
      }
    }
    // (b) conjugate triplet of hop hi started here (cell cj, atom a)
    if (h.from == a) {
      int32_t tv[3] = {0, 0, 0};
      bool ok = true;
      for (int x = 0; x < P.dim; ++x) {
        int32_t t = cj[x] + h.v[x];
        if (periodic && P.extend[x]) t = ((t % P.span[x]) + P.span[x]) % P.span[x];
        else if (t < 0 || t >= P.span[x]) ok = false;
        tv[x] = t;
      }
      if (ok) {
        int64_t cb = h.to;
        for (int x = 0; x < P.dim; ++x) cb += tv[x] * P.stride[x];
        if (cb == bare) continue;                      // on-site: no conjugate triplet
        int32_t row = (int32_t)cb;
        if (P.comp) { row = P.comp[cb]; if (row < 0) continue; }
        if (n >= kMaxCand) return -1;
        int64_t lin = cell;
        c[n].row = row;
        c[n].key = (lin * P.n_hops + hi) * 2 + 1;
        if (want_values) {
          double tr, ti;
          hop_value(P, h, cj, bare, false, tr, ti);
          if (P.vel_axis >= 0) {                         // row = to, col = from: + bond
            const double f = dmul(bond_component(P, h), P.vel_scale);
            tr = dmul(tr, f);
            ti = dmul(ti, f);
          }
          if (!P.is_complex) { if (fabs(ti) > 1e-10) atomicOr(P.warn_flag, 1); ti = 0.0; }
          c[n].re = tr;
          c[n].im = -ti;
        }
        ++n;
      }
    }
  }
  // insertion sort by (row, key)
  for (int i = 1; i < n; ++i) {
    Cand x = c[i];
    int k = i - 1;
    while (k >= 0 && (c[k].row > x.row || (c[k].row == x.row && c[k].key > x.key))) { c[k + 1] = c[k]; --k; }
    c[k + 1] = x;
  }
  return n;
}

__global__ void build_count_kernel(BuildParams P, int32_t* __restrict__ cnt, int32_t* __restrict__ err) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= P.n_cols) return;
  Cand c[kMaxCand];
  int n = column_candidates(P, j, c, false);
  if (n < 0) { atomicOr(err, 1); cnt[j] = 0; return; }
  int u = 0;
  for (int i = 0; i < n; ++i) u += (i == 0 || c[i].row != c[i - 1].row) ? 1 : 0;
  cnt[j] = u;
}

__global__ void build_fill_kernel(BuildParams P, const int32_t* __restrict__ col_ptr,
                                  int32_t* __restrict__ row_idx, double* __restrict__ val) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= P.n_cols) return;
  Cand c[kMaxCand];
  int n = column_candidates(P, j, c, true);
  if (n < 0) return;
  int64_t o = col_ptr[j];
  for (int i = 0; i < n;) {
    double sr = c[i].re, si = c[i].im;
    int k = i + 1;
    while (k < n && c[k].row == c[i].row) { sr = dadd(sr, c[k].re); si = dadd(si, c[k].im); ++k; }
    row_idx[o] = c[i].row;
    if (P.is_complex) { val[2 * o] = sr; val[2 * o + 1] = si; }
    else val[o] = sr;
    ++o;
    i = k;
  }
}

// ------------------------------------------------------------- rescale
__global__ void rescale_count_kernel(int32_t n, const int32_t* __restrict__ cp, const int32_t* __restrict__ ri,
                                     int32_t* __restrict__ cnt) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int32_t b = cp[j], e = cp[j + 1];
  bool has = false;
  for (int32_t p = b; p < e; ++p) has = has || ri[p] == j;
  cnt[j] = (e - b) + (has ? 0 : 1);
}

__global__ void rescale_fill_kernel(int32_t n, const int32_t* __restrict__ cp, const int32_t* __restrict__ ri,
                                    const double* __restrict__ v, int cplx, double a, double b,
                                    const int32_t* __restrict__ ocp, int32_t* __restrict__ ori,
                                    double* __restrict__ ov) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  int64_t k = ocp[j];
  bool done = false;
  auto put_diag_only = [&]() {
    ori[k] = j;
    if (cplx) { ov[2 * k] = __ddiv_rn(__dsub_rn(0.0, b), a); ov[2 * k + 1] = __ddiv_rn(__dsub_rn(0.0, 0.0), a); }
    else ov[k] = __ddiv_rn(__dsub_rn(0.0, b), a);
    ++k;
    done = true;
  };
  for (int32_t p = cp[j]; p < cp[j + 1]; ++p) {
    int32_t r = ri[p];
    if (!done && r > j) put_diag_only();
    ori[k] = r;
    double sub = (r == j) ? b : 0.0;
    if (r == j) done = true;
    if (cplx) { ov[2 * k] = __ddiv_rn(__dsub_rn(v[2 * p], sub), a); ov[2 * k + 1] = __ddiv_rn(__dsub_rn(v[2 * p + 1], 0.0), a); }
    else ov[k] = __ddiv_rn(__dsub_rn(v[p], sub), a);
    ++k;
  }
  if (!done) put_diag_only();
}

// ------------------------------------------------------------- commutator
__global__ void diag_extract_kernel(int32_t n, const int32_t* __restrict__ cp, const int32_t* __restrict__ ri,
                                    const double* __restrict__ v, int cplx, double* __restrict__ x) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double d = 0.0;
  for (int32_t p = cp[j]; p < cp[j + 1]; ++p)
    if (ri[p] == j) d = cplx ? v[2 * p] : v[p];
  x[j] = d;
}

__global__ void commutator_kernel(int32_t n, const int32_t* __restrict__ cp, const int32_t* __restrict__ ri,
                                  const double* __restrict__ v, int cplx, const double* __restrict__ x,
                                  double* __restrict__ ov) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  double xj = x[j];
  for (int32_t p = cp[j]; p < cp[j + 1]; ++p) {
    double xi = x[ri[p]];
    if (cplx) {
      ov[2 * p] = __dsub_rn(__dmul_rn(xi, v[2 * p]), __dmul_rn(v[2 * p], xj));
      ov[2 * p + 1] = __dsub_rn(__dmul_rn(xi, v[2 * p + 1]), __dmul_rn(v[2 * p + 1], xj));
    } else {
      ov[p] = __dsub_rn(__dmul_rn(xi, v[p]), __dmul_rn(v[p], xj));
    }
  }
}

// ------------------------------------------------------------- CSC -> rows -> sliced ELL
__global__ void row_count_kernel(int64_t nnz, const int32_t* __restrict__ ri, int32_t* __restrict__ cnt) {
  int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < nnz) atomicAdd(&cnt[ri[p]], 1);
}

__global__ void row_scatter_kernel(int32_t n, const int32_t* __restrict__ cp, const int32_t* __restrict__ ri,
                                   const int32_t* __restrict__ rp, int32_t* __restrict__ cur,
                                   int32_t* __restrict__ rc, int64_t* __restrict__ src) {
  int32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  for (int32_t p = cp[j]; p < cp[j + 1]; ++p) {
    int32_t i = ri[p];
    int32_t s = atomicAdd(&cur[i], 1);
    rc[rp[i] + s] = j;
    src[rp[i] + s] = p;
  }
}

__global__ void row_sort_kernel(int32_t n, const int32_t* __restrict__ rp, int32_t* __restrict__ rc,
                                int64_t* __restrict__ src) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t b = rp[i], e = rp[i + 1];
  for (int32_t p = b + 1; p < e; ++p) {
    int32_t c = rc[p];
    int64_t s = src[p];
    int32_t q = p - 1;
    while (q >= b && rc[q] > c) { rc[q + 1] = rc[q]; src[q + 1] = src[q]; --q; }
    rc[q + 1] = c;
    src[q + 1] = s;
  }
}

__global__ void slice_width_kernel(int32_t n, int32_t n_slices, const int32_t* __restrict__ rp,
                                   const int32_t* __restrict__ rc, int32_t* __restrict__ width32) {
  int32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n_slices) return;
  int32_t w = 0;
  for (int l = 0; l < 32; ++l) {
    int32_t i = s * 32 + l;
    if (i >= n) break;
    int32_t cnt = 0;
    for (int32_t p = rp[i]; p < rp[i + 1]; ++p) cnt += rc[p] != i ? 1 : 0;
    w = max(w, cnt);
  }
  width32[s] = w * 32;
}

__global__ void ell_fill_kernel(int32_t n, const int32_t* __restrict__ rp, const int32_t* __restrict__ rc,
                                const int64_t* __restrict__ src, const double* __restrict__ v, int in_cplx, int cplx,
                                const int32_t* __restrict__ soff, int32_t* __restrict__ ecol,
                                double* __restrict__ e64, float* __restrict__ e32,
                                double* __restrict__ d64, float* __restrict__ d32) {
  int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int32_t s = i >> 5, l = i & 31;
  int64_t base = soff[s];
  int32_t w = (soff[s + 1] - soff[s]) >> 5;
  int k = 0;
  double dr = 0.0, di = 0.0;
  for (int32_t p = rp[i]; p < rp[i + 1]; ++p) {
    int64_t q = src[p];
    double vr = in_cplx ? v[2 * q] : v[q];
    double vi = in_cplx ? v[2 * q + 1] : 0.0;
    if (rc[p] == i) { dr += vr; di += vi; continue; }   // a CSC holds at most one diagonal entry per column
    int64_t o = base + (int64_t)k * 32 + l;
    ecol[o] = rc[p];
    if (cplx) { e64[2 * o] = vr; e64[2 * o + 1] = vi; e32[2 * o] = __double2float_rn(vr); e32[2 * o + 1] = __double2float_rn(vi); }
    else { e64[o] = vr; e32[o] = __double2float_rn(vr); }
    ++k;
  }
  for (; k < w; ++k) {
    int64_t o = base + (int64_t)k * 32 + l;
    ecol[o] = i;
    if (cplx) { e64[2 * o] = 0.0; e64[2 * o + 1] = 0.0; e32[2 * o] = 0.f; e32[2 * o + 1] = 0.f; }
    else { e64[o] = 0.0; e32[o] = 0.f; }
  }
  if (cplx) { d64[2 * i] = dr; d64[2 * i + 1] = di; d32[2 * i] = __double2float_rn(dr); d32[2 * i + 1] = __double2float_rn(di); }
  else { d64[i] = dr; d32[i] = __double2float_rn(dr); }
}

// flag = 1 when any imaginary part of a complex value array is nonzero (or NaN)
__global__ void imag_nonzero_kernel(int64_t nnz, const double* __restrict__ v, int* __restrict__ flag) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < nnz; q += (int64_t)gridDim.x * blockDim.x)
    if (!(v[2 * q + 1] == 0.0)) { atomicOr(flag, 1); return; }
}

// Rows of the slice tail beyond n (n not a multiple of 32) still need valid
// padding so that kernels may read a full slice.
__global__ void ell_tail_kernel(int32_t n, int32_t n_slices, const int32_t* __restrict__ soff,
                                int32_t* __restrict__ ecol, double* __restrict__ e64, float* __restrict__ e32,
                                int cplx) {
  int32_t l = threadIdx.x;
  int32_t s = n_slices - 1;
  int32_t i = s * 32 + l;
  if (i < n || l >= 32) return;
  int64_t base = soff[s];
  int32_t w = (soff[s + 1] - soff[s]) >> 5;
  for (int k = 0; k < w; ++k) {
    int64_t o = base + (int64_t)k * 32 + l;
    ecol[o] = 0;
    if (cplx) { e64[2 * o] = 0.0; e64[2 * o + 1] = 0.0; e32[2 * o] = 0.f; e32[2 * o + 1] = 0.f; }
    else { e64[o] = 0.0; e32[o] = 0.f; }
  }
}

int ensure_ell(tbk_sparse_s* A, cudaStream_t st) {
  if (A->ell_ready) return TBK_OK;
  if (A->rows != A->cols) return fail(TBK_ERR_INVALID, "recursion needs a square matrix (%d x %d)", A->rows, A->cols);
  const int32_t n = A->rows;
  const int in_cplx = A->is_complex;
  // a complex matrix whose imaginary parts are all zero gets a real ELL: the
  // products are the same (only the sign of an exact zero can differ) and the
  // recursion streams half the matrix bytes
  int cplx = in_cplx;
  if (in_cplx && A->nnz > 0) {
    DevBuf flag;
    TBK_TRY(flag.alloc(sizeof(int)));
    TBK_CUDA(cudaMemsetAsync(flag.p, 0, sizeof(int), st));
    const int64_t blocks = std::min<int64_t>((A->nnz + 255) / 256, 65535);
    imag_nonzero_kernel<<<(unsigned)blocks, 256, 0, st>>>(A->nnz, A->values.as<double>(), flag.as<int>());
    TBK_CHECK_LAUNCH();
    int h = 1;
    TBK_CUDA(cudaMemcpyAsync(&h, flag.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    TBK_CUDA(cudaStreamSynchronize(st));
    cplx = h ? 1 : 0;
  }
  EllDev& E = A->ell;
  E.cplx = cplx;
  E.n_rows = n;
  E.n_slices = (n + 31) / 32;
  DevBuf cnt, rp, cur, rc, src, w32;
  TBK_TRY(cnt.alloc(sizeof(int32_t) * (n + 1)));
  TBK_TRY(rp.alloc(sizeof(int32_t) * (n + 1)));
  TBK_TRY(cur.alloc(sizeof(int32_t) * (n + 1)));
  TBK_TRY(rc.alloc(sizeof(int32_t) * (A->nnz + 1)));
  TBK_TRY(src.alloc(sizeof(int64_t) * (A->nnz + 1)));
  TBK_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (n + 1), st));
  TBK_CUDA(cudaMemsetAsync(cur.p, 0, sizeof(int32_t) * (n + 1), st));
  const int T = 256;
  if (A->nnz > 0) {
    row_count_kernel<<<(unsigned)((A->nnz + T - 1) / T), T, 0, st>>>(A->nnz, A->row_idx.as<int32_t>(), cnt.as<int32_t>());
    TBK_CHECK_LAUNCH();
  }
  int32_t total = 0;
  TBK_TRY(exclusive_scan_i32(cnt.as<int32_t>(), rp.as<int32_t>(), n + 1, st, &total));
  row_scatter_kernel<<<(n + T - 1) / T, T, 0, st>>>(n, A->col_ptr.as<int32_t>(), A->row_idx.as<int32_t>(),
                                                     rp.as<int32_t>(), cur.as<int32_t>(), rc.as<int32_t>(),
                                                     src.as<int64_t>());
  TBK_CHECK_LAUNCH();
  row_sort_kernel<<<(n + T - 1) / T, T, 0, st>>>(n, rp.as<int32_t>(), rc.as<int32_t>(), src.as<int64_t>());
  TBK_CHECK_LAUNCH();
  TBK_TRY(w32.alloc(sizeof(int32_t) * (E.n_slices + 1)));
  TBK_CUDA(cudaMemsetAsync(w32.p, 0, sizeof(int32_t) * (E.n_slices + 1), st));
  slice_width_kernel<<<(E.n_slices + T - 1) / T, T, 0, st>>>(n, E.n_slices, rp.as<int32_t>(), rc.as<int32_t>(),
                                                               w32.as<int32_t>());
  TBK_CHECK_LAUNCH();
  TBK_TRY(E.slice_off.alloc(sizeof(int32_t) * (E.n_slices + 1)));
  int32_t n_entries = 0;
  TBK_TRY(exclusive_scan_i32(w32.as<int32_t>(), E.slice_off.as<int32_t>(), E.n_slices + 1, st, &n_entries));
  E.n_entries = n_entries;
  const size_t vs = cplx ? 2 : 1;
  TBK_TRY(E.col.alloc(sizeof(int32_t) * (n_entries + 32)));
  TBK_TRY(E.val64.alloc(sizeof(double) * vs * (n_entries + 32)));
  TBK_TRY(E.val32.alloc(sizeof(float) * vs * (n_entries + 32)));
  TBK_TRY(E.diag64.alloc(sizeof(double) * vs * (E.n_slices * 32)));
  TBK_TRY(E.diag32.alloc(sizeof(float) * vs * (E.n_slices * 32)));
  TBK_CUDA(cudaMemsetAsync(E.diag64.p, 0, E.diag64.bytes, st));
  TBK_CUDA(cudaMemsetAsync(E.diag32.p, 0, E.diag32.bytes, st));
  ell_fill_kernel<<<(n + T - 1) / T, T, 0, st>>>(n, rp.as<int32_t>(), rc.as<int32_t>(), src.as<int64_t>(),
                                                  A->values.as<double>(), in_cplx, cplx, E.slice_off.as<int32_t>(),
                                                  E.col.as<int32_t>(), E.val64.as<double>(), E.val32.as<float>(),
                                                  E.diag64.as<double>(), E.diag32.as<float>());
  TBK_CHECK_LAUNCH();
  if (n % 32) {
    ell_tail_kernel<<<1, 32, 0, st>>>(n, E.n_slices, E.slice_off.as<int32_t>(), E.col.as<int32_t>(),
                                      E.val64.as<double>(), E.val32.as<float>(), cplx);
    TBK_CHECK_LAUNCH();
  }
  // maximum slice width (host copy of the widths)
  std::vector<int32_t> hw(E.n_slices);
  TBK_CUDA(cudaMemcpyAsync(hw.data(), w32.p, sizeof(int32_t) * E.n_slices, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  int32_t mw = 0;
  for (auto w : hw) mw = std::max(mw, w / 32);
  E.max_width = mw;
  A->ell_ready = true;
  return TBK_OK;
}

// FP64 values -> double-float (hi, lo) pairs: hi = rn(v), lo = rn(v - hi)
__global__ void to_dd_kernel(int64_t n, const double* __restrict__ v, float2* __restrict__ out) {
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const double x = v[q];
    const float h = __double2float_rn(x);
    out[q] = make_float2(h, __double2float_rn(x - (double)h));
  }
}

int ensure_ell_dd(tbk_sparse_s* A, cudaStream_t st) {
  TBK_TRY(ensure_ell(A, st));
  EllDev& E = A->ell;
  if (E.valdd.p) return TBK_OK;
  if (!E.val64.p || !E.diag64.p) return fail(TBK_ERR_INVALID, "double-float ELL needs the FP64 values");
  const int64_t nv = E.val64.bytes / sizeof(double), nd = E.diag64.bytes / sizeof(double);
  TBK_TRY(E.valdd.alloc(sizeof(float2) * nv));
  TBK_TRY(E.diagdd.alloc(sizeof(float2) * nd));
  to_dd_kernel<<<(unsigned)std::min<int64_t>((nv + 255) / 256, 65535), 256, 0, st>>>(nv, E.val64.as<double>(),
                                                                                   E.valdd.as<float2>());
  TBK_CHECK_LAUNCH();
  to_dd_kernel<<<(unsigned)std::min<int64_t>((nd + 255) / 256, 65535), 256, 0, st>>>(nd, E.diag64.as<double>(),
                                                                                   E.diagdd.as<float2>());
  TBK_CHECK_LAUNCH();
  return TBK_OK;
}

// ------------------------------------------------------------- row classes
// A row's class key: its number of off-diagonal entries and, in ELL order, each
// entry's column offset (column - row) and FP64 value bits.  Rows with equal
// keys are interchangeable for the recursion: the step kernel then computes
// their neighbours from a shared table.  Keys are hashed here; equality is
// confirmed entry by entry afterwards, so a hash collision only costs the
// class form, never a wrong product.
__device__ __forceinline__ uint64_t cls_mix(uint64_t x) {
  x ^= x >> 31;
  x *= 0x7fb5d329728ea185ull;
  x ^= x >> 27;
  x *= 0x81dadef4bc2dd44dull;
  x ^= x >> 33;
  return x;
}

__global__ void class_hash_kernel(int32_t n, const int32_t* __restrict__ soff, const int32_t* __restrict__ ecol,
                                  const double* __restrict__ v64, int cplx, uint64_t* __restrict__ hash) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t s = i >> 5, l = i & 31;
  const int64_t base = soff[s];
  const int32_t w = (soff[s + 1] - soff[s]) >> 5;
  uint64_t h = 0x9e3779b97f4a7c15ull;
  int32_t cnt = 0;
  for (int32_t k = 0; k < w; ++k) {
    const int64_t o = base + (int64_t)k * 32 + l;
    const int32_t c = ecol[o];
    if (c == i) continue;                                  // padding
    ++cnt;
    h = cls_mix(h ^ (uint64_t)(uint32_t)(c - i));
    h = cls_mix(h ^ (uint64_t)__double_as_longlong(cplx ? v64[2 * o] : v64[o]));
    if (cplx) h = cls_mix(h ^ (uint64_t)__double_as_longlong(v64[2 * o + 1]));
  }
  h = cls_mix(h ^ (uint64_t)cnt);
  hash[i] = h ? h : 1ull;                                  // 0 marks an empty table slot
}

// Open-addressing insert of every row's key (linear probing, at most cap
// probes); lanes of a warp with equal keys insert once.  rep[slot] = the
// smallest row of the key.
__global__ void class_insert_kernel(int32_t n, const uint64_t* __restrict__ hash,
                                    unsigned long long* __restrict__ keys, int32_t* __restrict__ rep, int32_t cap,
                                    int* __restrict__ overflow) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool act = i < n;
  const unsigned long long key = act ? (unsigned long long)hash[i] : 0ull;
  const unsigned m = __match_any_sync(0xffffffffu, key);
  if (!act || (threadIdx.x & 31) != __ffs(m) - 1) return;
  uint32_t slot = (uint32_t)(key ^ (key >> 32)) & (uint32_t)(cap - 1);
  for (int32_t probe = 0; probe < cap; ++probe) {
    const unsigned long long prev = atomicCAS(&keys[slot], 0ull, key);
    if (prev == 0ull || prev == key) {
      atomicMin(&rep[slot], i);
      return;
    }
    slot = (slot + 1) & (uint32_t)(cap - 1);
  }
  atomicOr(overflow, 1);
}

__global__ void class_assign_kernel(int32_t n, const uint64_t* __restrict__ hash,
                                    const unsigned long long* __restrict__ keys, const int32_t* __restrict__ slot_id,
                                    int32_t cap, uint8_t* __restrict__ cls, int* __restrict__ bad) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long key = hash[i];
  uint32_t slot = (uint32_t)(key ^ (key >> 32)) & (uint32_t)(cap - 1);
  for (int32_t probe = 0; probe < cap; ++probe) {
    if (keys[slot] == key) {
      cls[i] = (uint8_t)slot_id[slot];
      return;
    }
    slot = (slot + 1) & (uint32_t)(cap - 1);
  }
  atomicOr(bad, 1);
}

// Every row against its class's representative: same entry count, and in ELL
// order the same column offsets and bit-identical FP64 values.
__global__ void class_verify_kernel(int32_t n, const int32_t* __restrict__ soff, const int32_t* __restrict__ ecol,
                                    const double* __restrict__ v64, int cplx, const uint8_t* __restrict__ cls,
                                    const int32_t* __restrict__ rep_of, int* __restrict__ bad) {
  const int32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int32_t j = rep_of[cls[i]];
  const int32_t si = i >> 5, li = i & 31, sj = j >> 5, lj = j & 31;
  const int32_t wi = (soff[si + 1] - soff[si]) >> 5, wj = (soff[sj + 1] - soff[sj]) >> 5;
  int32_t ki = 0, kj = 0;
  const int vs = cplx ? 2 : 1;
  while (true) {
    while (ki < wi && ecol[soff[si] + (int64_t)ki * 32 + li] == i) ++ki;
    while (kj < wj && ecol[soff[sj] + (int64_t)kj * 32 + lj] == j) ++kj;
    if (ki >= wi || kj >= wj) break;
    const int64_t oi = soff[si] + (int64_t)ki * 32 + li, oj = soff[sj] + (int64_t)kj * 32 + lj;
    bool same = (ecol[oi] - i) == (ecol[oj] - j);
    for (int q = 0; q < vs; ++q)
      same = same && __double_as_longlong(v64[vs * oi + q]) == __double_as_longlong(v64[vs * oj + q]);
    if (!same) {
      atomicOr(bad, 1);
      return;
    }
    ++ki;
    ++kj;
  }
  if (ki < wi || kj < wj) atomicOr(bad, 1);                // different entry counts
}

// The class table from the representative rows: offsets, counts and the values
// in every precision (FP32 = the ELL's rounding, double-float = hi, lo as the
// ELL's double-float copy), unused tail entries zero.
__global__ void class_table_kernel(int32_t n_cls, int32_t W, const int32_t* __restrict__ rep_of,
                                   const int32_t* __restrict__ soff, const int32_t* __restrict__ ecol,
                                   const double* __restrict__ v64, int cplx, int32_t* __restrict__ cnt,
                                   int32_t* __restrict__ off, double* __restrict__ t64, float* __restrict__ t32,
                                   float* __restrict__ tdd) {
  const int32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n_cls) return;
  const int32_t j = rep_of[c], s = j >> 5, l = j & 31;
  const int32_t w = (soff[s + 1] - soff[s]) >> 5;
  const int vs = cplx ? 2 : 1;
  int32_t k = 0;
  for (int32_t e = 0; e < w; ++e) {
    const int64_t o = soff[s] + (int64_t)e * 32 + l;
    if (ecol[o] == j) continue;
    const int64_t t = (int64_t)c * W + k;
    off[t] = ecol[o] - j;
    for (int q = 0; q < vs; ++q) {
      const double x = v64[vs * o + q];
      const float h = __double2float_rn(x);
      t64[vs * t + q] = x;
      t32[vs * t + q] = h;
      tdd[2 * (vs * t + q)] = h;
      tdd[2 * (vs * t + q) + 1] = __double2float_rn(x - (double)h);
    }
    ++k;
  }
  cnt[c] = k;
  for (int32_t e = k; e < W; ++e) {
    const int64_t t = (int64_t)c * W + e;
    off[t] = 0;
    for (int q = 0; q < vs; ++q) {
      t64[vs * t + q] = 0.0;
      t32[vs * t + q] = 0.f;
      tdd[2 * (vs * t + q)] = 0.f;
      tdd[2 * (vs * t + q) + 1] = 0.f;
    }
  }
}

int ensure_classes(tbk_sparse_s* A, cudaStream_t st) {
  TBK_TRY(ensure_ell(A, st));
  EllDev& E = A->ell;
  if (E.cls_state != 0) return TBK_OK;
  E.cls_state = -1;
  if (const char* e = getenv("TBK_NO_CLASSES"))           // A/B override: always gather through the ELL
    if (atoi(e) != 0) return TBK_OK;
  const int32_t n = E.n_rows;
  const int32_t W = E.max_width;
  if (n < 1 || !E.val64.p || !E.col.p) return TBK_OK;
  if (W > kMaxClassEntries) return TBK_OK;
  constexpr int32_t cap = 1024;                            // table slots (power of two, > kMaxClasses)
  DevBuf hash, keys, rep, flags, slot_id, rep_of, cls;
  TBK_TRY(hash.alloc(sizeof(uint64_t) * n));
  TBK_TRY(keys.alloc(sizeof(unsigned long long) * cap));
  TBK_TRY(rep.alloc(sizeof(int32_t) * cap));
  TBK_TRY(flags.alloc(2 * sizeof(int)));
  TBK_CUDA(cudaMemsetAsync(keys.p, 0, keys.bytes, st));
  TBK_CUDA(cudaMemsetAsync(rep.p, 0x7f, rep.bytes, st));
  TBK_CUDA(cudaMemsetAsync(flags.p, 0, flags.bytes, st));
  const int T = 256;
  const unsigned g = (unsigned)((n + T - 1) / T);
  const int32_t* soff = E.slice_off.as<int32_t>();
  const int32_t* ecol = E.col.as<int32_t>();
  const double* v64 = E.val64.as<double>();
  class_hash_kernel<<<g, T, 0, st>>>(n, soff, ecol, v64, E.cplx, hash.as<uint64_t>());
  TBK_CHECK_LAUNCH();
  class_insert_kernel<<<g, T, 0, st>>>(n, hash.as<uint64_t>(), keys.as<unsigned long long>(), rep.as<int32_t>(), cap,
                                       flags.as<int>());
  TBK_CHECK_LAUNCH();
  std::vector<unsigned long long> hk(cap);
  std::vector<int32_t> hr(cap);
  int hf[2] = {0, 0};
  TBK_CUDA(cudaMemcpyAsync(hk.data(), keys.p, keys.bytes, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaMemcpyAsync(hr.data(), rep.p, rep.bytes, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaMemcpyAsync(hf, flags.p, sizeof(hf), cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  if (hf[0]) return TBK_OK;                                // more keys than slots
  // class ids in slot order (deterministic: the slots depend on the keys only)
  std::vector<int32_t> sid(cap, -1), rof;
  for (int32_t q = 0; q < cap; ++q)
    if (hk[q]) {
      sid[q] = (int32_t)rof.size();
      rof.push_back(hr[q]);
    }
  const int32_t C = (int32_t)rof.size();
  // entries per class rounded up to whole groups of 4 (zero tail entries: the
  // step kernels gather a class's entries four at a time without predicates)
  const int32_t Wt = (std::max(W, 1) + 3) / 4 * 4;
  if (C < 1 || C > kMaxClasses || (int64_t)C * Wt > kMaxClassEntries) return TBK_OK;
  TBK_TRY(slot_id.alloc(sizeof(int32_t) * cap));
  TBK_TRY(rep_of.alloc(sizeof(int32_t) * C));
  TBK_TRY(cls.alloc((size_t)E.n_slices * 32));
  TBK_CUDA(cudaMemcpyAsync(slot_id.p, sid.data(), sizeof(int32_t) * cap, cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemcpyAsync(rep_of.p, rof.data(), sizeof(int32_t) * C, cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemsetAsync(cls.p, 0, cls.bytes, st));
  class_assign_kernel<<<g, T, 0, st>>>(n, hash.as<uint64_t>(), keys.as<unsigned long long>(), slot_id.as<int32_t>(),
                                       cap, cls.as<uint8_t>(), flags.as<int>() + 1);
  TBK_CHECK_LAUNCH();
  class_verify_kernel<<<g, T, 0, st>>>(n, soff, ecol, v64, E.cplx, cls.as<uint8_t>(), rep_of.as<int32_t>(),
                                       flags.as<int>() + 1);
  TBK_CHECK_LAUNCH();
  const size_t vs = E.cplx ? 2 : 1;
  DevBuf cnt, off, t64, t32, tdd;
  TBK_TRY(cnt.alloc(sizeof(int32_t) * C));
  TBK_TRY(off.alloc(sizeof(int32_t) * C * Wt));
  TBK_TRY(t64.alloc(sizeof(double) * vs * C * Wt));
  TBK_TRY(t32.alloc(sizeof(float) * vs * C * Wt));
  TBK_TRY(tdd.alloc(2 * sizeof(float) * vs * C * Wt));
  class_table_kernel<<<(C + 63) / 64, 64, 0, st>>>(C, Wt, rep_of.as<int32_t>(), soff, ecol, v64, E.cplx,
                                                   cnt.as<int32_t>(), off.as<int32_t>(), t64.as<double>(),
                                                   t32.as<float>(), tdd.as<float>());
  TBK_CHECK_LAUNCH();
  TBK_CUDA(cudaMemcpyAsync(hf, flags.p, sizeof(hf), cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  if (hf[1]) return TBK_OK;                                // a row differs from its class (hash collision)
  E.n_cls = C;
  E.cls_w = Wt;
  E.cls = std::move(cls);
  E.cls_cnt = std::move(cnt);
  E.cls_off = std::move(off);
  E.cls_v64 = std::move(t64);
  E.cls_v32 = std::move(t32);
  E.cls_vdd = std::move(tdd);
  E.cls_state = 1;
  return TBK_OK;
}

}  // namespace tbk

using namespace tbk;

static int new_sparse(tbk_sparse_s** out, int32_t rows, int32_t cols, int64_t nnz, int cplx) {
  auto* A = new tbk_sparse_s();
  A->rows = rows;
  A->cols = cols;
  A->nnz = nnz;
  A->is_complex = cplx;
  int s;
  if ((s = A->col_ptr.alloc(sizeof(int32_t) * (cols + 1))) != TBK_OK ||
      (s = A->row_idx.alloc(sizeof(int32_t) * (nnz + 1))) != TBK_OK ||
      (s = A->values.alloc(sizeof(double) * (cplx ? 2 : 1) * (nnz + 1))) != TBK_OK) {
    delete A;
    return s;
  }
  *out = A;
  return TBK_OK;
}

extern "C" {

int tbk_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) { cudaGetLastError(); return 0; }
  return n;
}

static int build_matrix(tbk_sparse* out, tbk_lattice L, int32_t mode, const int32_t* extend, int32_t is_complex,
                        int32_t vel_axis, double vel_scale, void* stream) {
  if (!out || !L) return fail(TBK_ERR_INVALID, "tbk_build_hamiltonian: null argument");
  *out = nullptr;
  if (mode < 0 || mode > 2) return fail(TBK_ERR_INVALID, "unknown build mode %d", mode);
  cudaStream_t st = as_stream(stream);
  const Cell& C = L->cell;
  if (C.hops.empty()) { /* "Warning: no hopping is added!" — an all-zero matrix */ }
  BuildParams P;
  memset(&P, 0, sizeof(P));
  P.vel_axis = vel_axis;
  P.vel_scale = vel_scale;
  P.dim = C.dim;
  P.n_atoms = C.n_atoms;
  P.n_hops = (int32_t)C.hops.size();
  P.mode = mode;
  P.is_complex = is_complex ? 1 : 0;
  for (int i = 0; i < 3; ++i) { P.span[i] = L->span[i]; P.extend[i] = (mode == TBK_BUILD_PERIODIC_BARE && extend) ? (extend[i] != 0) : 0; }
  P.stride[C.dim - 1] = C.n_atoms;
  for (int i = C.dim - 2; i >= 0; --i) P.stride[i] = P.stride[i + 1] * L->span[i + 1];
  for (int i = 0; i < 9; ++i) P.bases[i] = C.bases[i];
  P.n_cols = (int32_t)L->total;
  P.gauge_kind = mode == TBK_BUILD_BARE ? GAUGE_NONE : L->gauge_kind;
  P.scalar_kind = mode == TBK_BUILD_BARE ? SCALAR_NONE : L->scalar_kind;
  for (int i = 0; i < 12; ++i) P.gauge_linear[i] = L->gauge_linear[i];
  P.disorder_W = L->disorder_W;
  P.disorder_seed = L->disorder_seed;
  // per-column candidate bound
  for (int a = 0; a < C.n_atoms; ++a) {
    int k = 0;
    for (auto& h : C.hops) k += (h.to == a) + (h.from == a);
    if (k > kMaxCand) return fail(TBK_ERR_UNSUPPORTED, "atom %d touches %d hopping terms (max %d)", a, k, kMaxCand);
  }
  // device copies of the cell and optional fields
  std::vector<DevHop> hh(C.hops.size());
  for (size_t k = 0; k < C.hops.size(); ++k) {
    hh[k].from = C.hops[k].from; hh[k].to = C.hops[k].to;
    for (int i = 0; i < 3; ++i) hh[k].v[i] = C.hops[k].v[i];
    hh[k].pad = 0; hh[k].tr = C.hops[k].tr; hh[k].ti = C.hops[k].ti;
  }
  DevBuf dh, dpos, dgauge, dscalar, dcomp, dinv, dwarn, derr, cnt;
  TBK_TRY(dh.alloc(sizeof(DevHop) * (hh.size() + 1)));
  TBK_TRY(dpos.alloc(sizeof(double) * C.pos.size()));
  if (!hh.empty()) TBK_CUDA(cudaMemcpyAsync(dh.p, hh.data(), sizeof(DevHop) * hh.size(), cudaMemcpyHostToDevice, st));
  TBK_CUDA(cudaMemcpyAsync(dpos.p, C.pos.data(), sizeof(double) * C.pos.size(), cudaMemcpyHostToDevice, st));
  P.hops = dh.as<DevHop>();
  P.pos = dpos.as<double>();
  if (P.gauge_kind == GAUGE_SITES) {
    TBK_TRY(dgauge.alloc(sizeof(double) * L->gauge_sites.size()));
    TBK_CUDA(cudaMemcpyAsync(dgauge.p, L->gauge_sites.data(), dgauge.bytes, cudaMemcpyHostToDevice, st));
    P.gauge_sites = dgauge.as<double>();
  }
  if (P.scalar_kind == SCALAR_SITES) {
    TBK_TRY(dscalar.alloc(sizeof(double) * L->scalar_sites.size()));
    TBK_CUDA(cudaMemcpyAsync(dscalar.p, L->scalar_sites.data(), dscalar.bytes, cudaMemcpyHostToDevice, st));
    P.scalar_sites = dscalar.as<double>();
  }
  P.n_kept = P.n_cols;
  if (mode == TBK_BUILD_SPARSE && !L->removed.empty()) {
    // index_comp_construct (TB/lattice.h:447-457) as a device compaction: the
    // site mask goes up once, kept flags are prefix-summed, and the bare ->
    // compressed map (-1 = removed) and its inverse are scattered from the scan
    int32_t kept = 0;
    TBK_TRY(compact_sites(L->removed.data(), L->total, &dcomp, &dinv, &kept, st));
    P.n_kept = kept;
    P.comp = dcomp.as<int32_t>();
    P.inv = dinv.as<int32_t>();
  }
  TBK_TRY(dwarn.alloc(sizeof(int32_t)));
  TBK_TRY(derr.alloc(sizeof(int32_t)));
  TBK_CUDA(cudaMemsetAsync(dwarn.p, 0, sizeof(int32_t), st));
  TBK_CUDA(cudaMemsetAsync(derr.p, 0, sizeof(int32_t), st));
  P.warn_flag = dwarn.as<int32_t>();
  const int32_t n = P.n_cols;
  TBK_TRY(cnt.alloc(sizeof(int32_t) * (n + 1)));
  TBK_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (n + 1), st));
  const int T = 128;
  build_count_kernel<<<(n + T - 1) / T, T, 0, st>>>(P, cnt.as<int32_t>(), derr.as<int32_t>());
  TBK_CHECK_LAUNCH();
  tbk_sparse_s* A = nullptr;
  DevBuf cp_tmp;
  TBK_TRY(cp_tmp.alloc(sizeof(int32_t) * (n + 1)));
  int32_t nnz = 0;
  TBK_TRY(exclusive_scan_i32(cnt.as<int32_t>(), cp_tmp.as<int32_t>(), n + 1, st, &nnz));
  int32_t herr = 0;
  TBK_CUDA(cudaMemcpyAsync(&herr, derr.p, sizeof(int32_t), cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  if (herr) return fail(TBK_ERR_UNSUPPORTED, "builder candidate overflow");
  TBK_TRY(new_sparse(&A, n, n, nnz, P.is_complex));
  A->col_ptr = std::move(cp_tmp);
  build_fill_kernel<<<(n + T - 1) / T, T, 0, st>>>(P, A->col_ptr.as<int32_t>(), A->row_idx.as<int32_t>(),
                                                    A->values.as<double>());
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { delete A; return fail(TBK_ERR_CUDA, "builder: %s", cudaGetErrorString(e)); }
  *out = A;
  return TBK_OK;
}

int tbk_build_hamiltonian(tbk_sparse* out, tbk_lattice L, int32_t mode, const int32_t* extend,
                          int32_t is_complex, void* stream) {
  return build_matrix(out, L, mode, extend, is_complex, -1, 0.0, stream);
}

int tbk_build_velocity_bond(tbk_sparse* out, tbk_lattice L, int32_t mode, const int32_t* extend, int32_t is_complex,
                            int32_t axis, double scale, void* stream) {
  if (!L) return fail(TBK_ERR_INVALID, "tbk_build_velocity_bond: null argument");
  if (axis < 0 || axis >= L->cell.dim) return fail(TBK_ERR_INVALID, "Error: axis out of range.");
  return build_matrix(out, L, mode, extend, is_complex, axis, scale, stream);
}

int tbk_build_position(tbk_sparse* out, tbk_lattice L, int32_t axis, void* stream) {
  if (!out || !L) return fail(TBK_ERR_INVALID, "tbk_build_position: null argument");
  *out = nullptr;
  const Cell& C = L->cell;
  if (axis < 0 || axis >= C.dim) axis = 0;   // "Error: axis out of range." -> axis 0
  // X = diag(x_i) over kept sites in index order, TB/lattice.h:323-332; host O(N)
  std::vector<double> x;
  x.reserve(L->total);
  int64_t n_cells = L->total / C.n_atoms;
  int32_t iv[3] = {0, 0, 0};
  for (int64_t c = 0; c < n_cells; ++c) {
    int64_t rem = c;
    for (int i = C.dim - 1; i >= 0; --i) { iv[i] = (int32_t)(rem % L->span[i]); rem /= L->span[i]; }
    for (int a = 0; a < C.n_atoms; ++a) {
      int64_t b = c * C.n_atoms + a;
      if (!L->removed.empty() && L->removed[b]) continue;
      double d = 0.0;
      for (int cc = 0; cc < C.dim; ++cc) d = d + C.bases[cc * 3 + axis] * (double)iv[cc];
      x.push_back(C.pos[a * 3 + axis] + d);
    }
  }
  const int32_t n = (int32_t)L->total, k = (int32_t)x.size();
  std::vector<int32_t> cp(n + 1), ri(k);
  for (int32_t j = 0; j <= n; ++j) cp[j] = std::min(j, k);
  for (int32_t j = 0; j < k; ++j) ri[j] = j;
  return tbk_sparse_from_csc(out, n, n, k, cp.data(), ri.data(), x.data(), 0, 0, stream);
}

int tbk_sparse_from_csc(tbk_sparse* out, int32_t rows, int32_t cols, int64_t nnz, const int32_t* col_ptr,
                        const int32_t* row_idx, const double* values, int32_t is_complex, int32_t device_ptrs,
                        void* stream) {
  if (!out || !col_ptr || (nnz > 0 && (!row_idx || !values)))
    return fail(TBK_ERR_INVALID, "tbk_sparse_from_csc: null argument");
  *out = nullptr;
  if (rows < 0 || cols < 0 || nnz < 0 || nnz > INT32_MAX) return fail(TBK_ERR_INVALID, "tbk_sparse_from_csc: bad sizes");
  cudaStream_t st = as_stream(stream);
  tbk_sparse_s* A = nullptr;
  TBK_TRY(new_sparse(&A, rows, cols, nnz, is_complex ? 1 : 0));
  cudaMemcpyKind k = device_ptrs ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
  size_t vb = sizeof(double) * (is_complex ? 2 : 1) * nnz;
  cudaError_t e = cudaMemcpyAsync(A->col_ptr.p, col_ptr, sizeof(int32_t) * (cols + 1), k, st);
  if (e == cudaSuccess && nnz) e = cudaMemcpyAsync(A->row_idx.p, row_idx, sizeof(int32_t) * nnz, k, st);
  if (e == cudaSuccess && nnz) e = cudaMemcpyAsync(A->values.p, values, vb, k, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { delete A; return fail(TBK_ERR_CUDA, "tbk_sparse_from_csc: %s", cudaGetErrorString(e)); }
  *out = A;
  return TBK_OK;
}

int tbk_sparse_row_classes(tbk_sparse A, int32_t* n_classes, void* stream) {
  if (!A || !n_classes) return fail(TBK_ERR_INVALID, "tbk_sparse_row_classes: null argument");
  TBK_TRY(ensure_classes(A, as_stream(stream)));
  *n_classes = A->ell.cls_state == 1 ? A->ell.n_cls : 0;
  return TBK_OK;
}

int tbk_sparse_info(tbk_sparse A, int32_t* rows, int32_t* cols, int64_t* nnz, int32_t* is_complex) {
  if (!A) return fail(TBK_ERR_INVALID, "tbk_sparse_info: null matrix");
  if (rows) *rows = A->rows;
  if (cols) *cols = A->cols;
  if (nnz) *nnz = A->nnz;
  if (is_complex) *is_complex = A->is_complex;
  return TBK_OK;
}

int tbk_sparse_download(tbk_sparse A, int32_t* col_ptr, int32_t* row_idx, double* values, void* stream) {
  if (!A) return fail(TBK_ERR_INVALID, "tbk_sparse_download: null matrix");
  cudaStream_t st = as_stream(stream);
  if (col_ptr) TBK_CUDA(cudaMemcpyAsync(col_ptr, A->col_ptr.p, sizeof(int32_t) * (A->cols + 1), cudaMemcpyDeviceToHost, st));
  if (row_idx && A->nnz) TBK_CUDA(cudaMemcpyAsync(row_idx, A->row_idx.p, sizeof(int32_t) * A->nnz, cudaMemcpyDeviceToHost, st));
  if (values && A->nnz)
    TBK_CUDA(cudaMemcpyAsync(values, A->values.p, sizeof(double) * (A->is_complex ? 2 : 1) * A->nnz, cudaMemcpyDeviceToHost, st));
  TBK_CUDA(cudaStreamSynchronize(st));
  return TBK_OK;
}

void tbk_sparse_destroy(tbk_sparse A) {
  if (A) cudaDeviceSynchronize();
  delete A;
}

int tbk_sparse_rescale(tbk_sparse* out, tbk_sparse H, double a, double b, void* stream) {
  if (!out || !H) return fail(TBK_ERR_INVALID, "tbk_sparse_rescale: null argument");
  *out = nullptr;
  if (H->rows != H->cols) return fail(TBK_ERR_INVALID, "rescale needs a square matrix");
  if (!(a != 0.0)) return fail(TBK_ERR_INVALID, "rescale: a must be nonzero (got %g)", a);
  cudaStream_t st = as_stream(stream);
  const int32_t n = H->rows;
  const int T = 256;
  DevBuf cnt, cp;
  TBK_TRY(cnt.alloc(sizeof(int32_t) * (n + 1)));
  TBK_TRY(cp.alloc(sizeof(int32_t) * (n + 1)));
  TBK_CUDA(cudaMemsetAsync(cnt.p, 0, sizeof(int32_t) * (n + 1), st));
  if (n) {
    rescale_count_kernel<<<(n + T - 1) / T, T, 0, st>>>(n, H->col_ptr.as<int32_t>(), H->row_idx.as<int32_t>(), cnt.as<int32_t>());
    TBK_CHECK_LAUNCH();
  }
  int32_t nnz = 0;
  TBK_TRY(exclusive_scan_i32(cnt.as<int32_t>(), cp.as<int32_t>(), n + 1, st, &nnz));
  tbk_sparse_s* A = nullptr;
  TBK_TRY(new_sparse(&A, n, n, nnz, H->is_complex));
  A->col_ptr = std::move(cp);
  if (n) {
    rescale_fill_kernel<<<(n + T - 1) / T, T, 0, st>>>(n, H->col_ptr.as<int32_t>(), H->row_idx.as<int32_t>(),
                                                       H->values.as<double>(), H->is_complex, a, b,
                                                       A->col_ptr.as<int32_t>(), A->row_idx.as<int32_t>(),
                                                       A->values.as<double>());
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { delete A; return fail(TBK_ERR_CUDA, "rescale: %s", cudaGetErrorString(e)); }
  *out = A;
  return TBK_OK;
}

int tbk_sparse_commutator(tbk_sparse* out, tbk_sparse H, tbk_sparse X, void* stream) {
  if (!out || !H || !X) return fail(TBK_ERR_INVALID, "tbk_sparse_commutator: null argument");
  *out = nullptr;
  if (H->rows != H->cols || X->rows != H->rows || X->cols != H->cols)
    return fail(TBK_ERR_INVALID, "commutator: size mismatch");
  cudaStream_t st = as_stream(stream);
  const int32_t n = H->rows;
  const int T = 256;
  DevBuf x;
  TBK_TRY(x.alloc(sizeof(double) * (n + 1)));
  tbk_sparse_s* A = nullptr;
  TBK_TRY(new_sparse(&A, n, n, H->nnz, H->is_complex));
  cudaError_t e = cudaMemcpyAsync(A->col_ptr.p, H->col_ptr.p, sizeof(int32_t) * (n + 1), cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && H->nnz) e = cudaMemcpyAsync(A->row_idx.p, H->row_idx.p, sizeof(int32_t) * H->nnz, cudaMemcpyDeviceToDevice, st);
  if (e == cudaSuccess && n) {
    diag_extract_kernel<<<(n + T - 1) / T, T, 0, st>>>(n, X->col_ptr.as<int32_t>(), X->row_idx.as<int32_t>(),
                                                       X->values.as<double>(), X->is_complex, x.as<double>());
    commutator_kernel<<<(n + T - 1) / T, T, 0, st>>>(n, H->col_ptr.as<int32_t>(), H->row_idx.as<int32_t>(),
                                                     H->values.as<double>(), H->is_complex, x.as<double>(),
                                                     A->values.as<double>());
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) { delete A; return fail(TBK_ERR_CUDA, "commutator: %s", cudaGetErrorString(e)); }
  *out = A;
  return TBK_OK;
}

}  // extern "C"
