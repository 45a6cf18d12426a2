// tbk_internal.h — shared internals of libtbk (device sparse objects, errors).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/tbk.h"

namespace tbk {

// ---- error handling: every C entry point returns a status and records a message
void set_error(int code, const std::string& msg);
int fail(int code, const char* fmt, ...);
#define TBK_CUDA(call)                                                              \
  do {                                                                              \
    cudaError_t e_ = (call);                                                        \
    if (e_ != cudaSuccess)                                                          \
      return ::tbk::fail(TBK_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #call,   \
                         cudaGetErrorString(e_));                                   \
  } while (0)
#define TBK_CHECK_LAUNCH() TBK_CUDA(cudaGetLastError())
#define TBK_TRY(expr)                                                               \
  do {                                                                              \
    int s_ = (expr);                                                                \
    if (s_ != TBK_OK) return s_;                                                    \
  } while (0)

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// ---- stream-ordered allocation context.  While a thread has one installed,
// DevBuf takes its memory from the context's pool on the context's stream and
// gives it back with cudaFreeAsync, so that freeing never waits for the device.
struct AsyncAllocCtx {
  cudaMemPool_t pool = nullptr;
  cudaStream_t stream = nullptr;
};
extern thread_local const AsyncAllocCtx* tl_async_alloc;

// ---- device buffer (RAII, cudaMalloc or the thread's stream-ordered pool)
struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  const AsyncAllocCtx* ctx = nullptr;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  DevBuf(DevBuf&& o) noexcept : p(o.p), bytes(o.bytes), ctx(o.ctx) { o.p = nullptr; o.bytes = 0; o.ctx = nullptr; }
  DevBuf& operator=(DevBuf&& o) noexcept {
    if (this != &o) {
      release();
      p = o.p; bytes = o.bytes; ctx = o.ctx;
      o.p = nullptr; o.bytes = 0; o.ctx = nullptr;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void release() {
    if (p) {
      if (ctx) cudaFreeAsync(p, ctx->stream);
      else cudaFree(p);
    }
    p = nullptr; bytes = 0; ctx = nullptr;
  }
  int alloc(size_t n) {
    release();
    if (n == 0) n = 16;
    cudaError_t e;
    if (tl_async_alloc) {
      e = cudaMallocFromPoolAsync(&p, n, tl_async_alloc->pool, tl_async_alloc->stream);
      if (e == cudaSuccess) ctx = tl_async_alloc;
    } else {
      e = cudaMalloc(&p, n);
    }
    if (e != cudaSuccess) { p = nullptr; return fail(TBK_ERR_NOMEM, "device allocation of %zu bytes: %s", n, cudaGetErrorString(e)); }
    bytes = n;
    return TBK_OK;
  }
  template <class T> T* as() const { return reinterpret_cast<T*>(p); }
};

// Sliced-ELL view of a square matrix for the recursion kernels: rows are cut in
// slices of 32; slice s stores width_s entries per row, column-major inside the
// slice (entry k of row 32*s + l at off[s] + 32*k + l).  The diagonal is kept
// apart so that every row owns its v_n element.  Padding entries point at the
// row itself with value 0.
struct EllDev {
  int32_t n_rows = 0, n_slices = 0;
  int64_t n_entries = 0;
  int32_t max_width = 0;
  int32_t cplx = 0;   // value type of the ELL: complex, or real when every imaginary part is zero
  DevBuf slice_off;   // int32 [n_slices + 1]
  DevBuf col;         // int32 [n_entries]
  DevBuf val64;       // double / double2 [n_entries]
  DevBuf diag64;      // double / double2 [n_rows]
  DevBuf val32;       // float / float2 [n_entries]  (mixed precision)
  DevBuf diag32;      // float / float2 [n_rows]
  DevBuf valdd;       // double-float (hi, lo) pairs, real or complex [n_entries] (on demand)
  DevBuf diagdd;      // [n_rows]
  // Row classes (ensure_classes): when every row's off-diagonal entries form
  // one of at most kMaxClasses lists of (column - row, value) — the case of a
  // lattice Hamiltonian without vacancies whose hoppings do not vary from cell
  // to cell — the recursion computes each neighbour as row + offset from the
  // row's class instead of loading its column index and value.  Exact: every
  // row is compared entry by entry with its class's representative row.
  int32_t cls_state = 0;   // 0 not examined, 1 classes ready, -1 not applicable
  int32_t n_cls = 0;       // number of classes
  int32_t cls_w = 0;       // table row length: the ELL width rounded up to a multiple of 4 (zero tail)
  DevBuf cls;              // uint8 [n_slices * 32]: class of each row (0 for the tail)
  DevBuf cls_cnt;          // int32 [n_cls]: entries of each class
  DevBuf cls_off;          // int32 [n_cls * cls_w]: column - row, ELL order
  DevBuf cls_v64;          // double / double2 [n_cls * cls_w]
  DevBuf cls_v32;          // float / float2
  DevBuf cls_vdd;          // double-float pairs (real: float2, complex: float4)
};
constexpr int32_t kMaxClasses = 255;
constexpr int32_t kMaxClassEntries = 1024;   // n_cls * cls_w (shared-memory table of the step kernel)

}  // namespace tbk

// Device-resident sparse matrix: Eigen-compatible CSC (the reference-facing
// form) plus the sliced-ELL of its rows used by the recursion kernels.
struct tbk_sparse_s {
  int32_t rows = 0, cols = 0;
  int64_t nnz = 0;
  int32_t is_complex = 0;
  tbk::DevBuf col_ptr;   // int32 [cols+1]
  tbk::DevBuf row_idx;   // int32 [nnz]
  tbk::DevBuf values;    // double or double2 [nnz]
  bool ell_ready = false;
  tbk::EllDev ell;
};

namespace tbk {
// builder.cu
int ensure_ell(tbk_sparse_s* A, cudaStream_t st);
int ensure_ell_dd(tbk_sparse_s* A, cudaStream_t st);   // double-float copy of the FP64 values
int ensure_classes(tbk_sparse_s* A, cudaStream_t st);  // row classes of the ELL (cls_state 1 or -1)
int exclusive_scan_i32(const int32_t* in, int32_t* out, int64_t n, cudaStream_t st, int32_t* total_host);
int exclusive_scan_i64(const int64_t* in, int64_t* out, int64_t n, cudaStream_t st, int64_t* total_host);
int sm_count();
// complex64 K-tiled stores written by a recursion step (Kubo blocks).  Element
// k of block m sits at ((k / 16) * kM + m) * 16 + k % 16.  The step's columns
// form `halves` groups (1 or 2) of R / halves columns; group h writes block
// km[h] (none when negative) of store[h], k = row * (R / halves) + column in
// the group, with either the step output or V x for its operator V (values
// vval[h] / vdiag[h], same ELL structure as H; null: H's own values).
struct KStore {
  float2* store[2] = {nullptr, nullptr};
  const void* vval[2] = {nullptr, nullptr};
  const void* vdiag[2] = {nullptr, nullptr};
  int32_t km[2] = {-1, -1};
  int32_t usev[2] = {0, 0};
  int32_t kM = 0;
  int32_t halves = 1;
  const void* addv = nullptr;      // Clenshaw steps: output += (addc[0] + i addc[1]) addv
  double addc[2] = {0.0, 0.0};
};

// kpm.cu — one fused recursion step with the one-pass kernel in a precision
// TBK_PREC_* (complex64, complex128 or double-float vectors): y = H x (first)
// or y = 2 H x - pv; moment partials into part[2 * grid].  Block loaders:
// Eigen-layout kets / seeded random phases.
int step_config(tbk_sparse_s* A, int Rc, int prec, int* grid, int* n_tiles, cudaStream_t st);
// kstore: optional complex64 K-tiled store that receives the step's output as
// block km of kM (store_y false: only there)
// vop: with kstore, store vop x instead of the output; vop must share A's ELL
// structure (same_ell_structure) and precision arrays
// dots: form the moment partial sums (false: the step only feeds other work)
int step_any(tbk_sparse_s* A, int Rc, int prec, const void* x, void* y, const void* pv, bool first, double* part,
             int grid, int n_tiles, cudaStream_t st, float2* kstore = nullptr, int32_t kM = 0, int32_t km = 0,
             bool store_y = true, tbk_sparse_s* vop = nullptr, bool dots = true);
// ELL value / diagonal arrays of a precision (FP32, FP64 or double-float pairs)
const void* ell_vals(const EllDev& E, int prec);
const void* ell_diag(const EllDev& E, int prec);
// one recursion step (not the first block's braket form) writing the K-tiled
// stores described by ks (output or operator products per column group)
int step_ks(tbk_sparse_s* A, int Rc, int prec, const void* x, void* y, const void* pv, bool first, double* part,
            int grid, int n_tiles, cudaStream_t st, const KStore& ks, int mode = 2);
// true when B's sliced ELL has A's slices, widths and columns (values may differ)
int same_ell_structure(tbk_sparse_s* A, tbk_sparse_s* B, bool* same, cudaStream_t st);
int load_block_any(int prec, int32_t n, int32_t R, int32_t r0, int32_t Rp, const double2* src, void* dst,
                   cudaStream_t st);
int random_block_any(int prec, int32_t n, int32_t R, int32_t r0, int32_t Rp, uint64_t seed, void* dst,
                     cudaStream_t st);
}  // namespace tbk
