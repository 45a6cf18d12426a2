// cusparse_kpm.cu — the reference's GPU moments algorithm, restated as a
// timing baseline (not part of libtbk; nothing in the product calls it).
//
// What it restates: cuda::Cheb_first_kind_seq_braket of the reference,
// tight_binding/numerics_cuda.cu:190-255 (real matrix) and :266-323 (complex
// matrix).  Per call it uploads the CSC matrix and the bras / kets, creates a
// cuSPARSE and a cuBLAS handle, sizes one SpMM work buffer, and then per moment
//   real M:    two FP64 SpMMs (Re and Im column blocks) Tn_2 <- 2 M Tn_1 - Tn_2
//              and two cublasDdot traces (host pointer mode: each one waits)
//   complex M: one complex128 SpMM and one cublasZdotc (real part),
// then frees everything.  The reference prints each moment to stdout; that is
// left out here.  Moments: mu_0 = <bras|kets>, mu_1 = <bras|M kets>, then
// mu_i from the in-place recursion, i < n (n >= 2).
#include <cublas_v2.h>
#include <cuda_runtime.h>
#include <cusparse.h>

#include <chrono>
#include <cstdint>
#include <utility>
#include <vector>

namespace {

struct Timer {
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double ms() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  }
};

#define REF_TRY(x)                                  \
  do {                                              \
    if ((x) != 0) { status = __LINE__; goto done; } \
  } while (0)

}  // namespace

extern "C" {

// bras / kets: N x R column-major complex128 (interleaved); times_ms (may be
// NULL): [0] whole call, [1] moment loop only.  Returns 0 or the source line of
// the first failing call.
int ref_cusparse_braket_real(int32_t n_rows, int64_t nnz, const int32_t* cp, const int32_t* ri, const double* v,
                             int32_t n, const double* bras, const double* kets, int32_t R, double* mu_out,
                             double* times_ms) {
  Timer all;
  if (n < 2) return -1;
  int status = 0;
  const int64_t NR = (int64_t)n_rows * R;
  // the reference evaluates bras.real() / .imag() / kets.real() / .imag() on the host
  std::vector<double> h_br(NR), h_bi(NR), h_kr(NR), h_ki(NR);
  for (int64_t q = 0; q < NR; ++q) {
    h_br[q] = bras[2 * q];
    h_bi[q] = bras[2 * q + 1];
    h_kr[q] = kets[2 * q];
    h_ki[q] = kets[2 * q + 1];
  }
  int32_t *d_cp = nullptr, *d_ri = nullptr;
  double *d_v = nullptr, *br = nullptr, *bi = nullptr, *t2r = nullptr, *t2i = nullptr, *t1r = nullptr, *t1i = nullptr;
  void* buf = nullptr;
  cusparseHandle_t sp = nullptr;
  cublasHandle_t bl = nullptr;
  cusparseSpMatDescr_t A = nullptr;
  cusparseDnMatDescr_t dbr = nullptr, dbi = nullptr, d2r = nullptr, d2i = nullptr, d1r = nullptr, d1i = nullptr;
  const size_t vb = sizeof(double) * NR;
  double alpha0 = 1.0, beta0 = 0.0, alpha = 2.0, beta = -1.0, a = 0.0, b = 0.0;
  size_t bs1 = 0, bs2 = 0;
  Timer loop;
  REF_TRY(cudaMalloc(&d_cp, sizeof(int32_t) * (n_rows + 1)));
  REF_TRY(cudaMalloc(&d_ri, sizeof(int32_t) * (nnz ? nnz : 1)));
  REF_TRY(cudaMalloc(&d_v, sizeof(double) * (nnz ? nnz : 1)));
  REF_TRY(cudaMemcpy(d_cp, cp, sizeof(int32_t) * (n_rows + 1), cudaMemcpyHostToDevice));
  REF_TRY(cudaMemcpy(d_ri, ri, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice));
  REF_TRY(cudaMemcpy(d_v, v, sizeof(double) * nnz, cudaMemcpyHostToDevice));
  for (double** p : {&br, &bi, &t2r, &t2i, &t1r, &t1i}) REF_TRY(cudaMalloc(p, vb));
  REF_TRY(cudaMemcpy(br, h_br.data(), vb, cudaMemcpyHostToDevice));
  REF_TRY(cudaMemcpy(bi, h_bi.data(), vb, cudaMemcpyHostToDevice));
  REF_TRY(cudaMemcpy(t2r, h_kr.data(), vb, cudaMemcpyHostToDevice));
  REF_TRY(cudaMemcpy(t2i, h_ki.data(), vb, cudaMemcpyHostToDevice));
  REF_TRY(cusparseCreateCsc(&A, n_rows, n_rows, nnz, d_cp, d_ri, d_v, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I,
                            CUSPARSE_INDEX_BASE_ZERO, CUDA_R_64F));
  REF_TRY(cusparseCreateDnMat(&dbr, n_rows, R, n_rows, br, CUDA_R_64F, CUSPARSE_ORDER_COL));
  REF_TRY(cusparseCreateDnMat(&dbi, n_rows, R, n_rows, bi, CUDA_R_64F, CUSPARSE_ORDER_COL));
  REF_TRY(cusparseCreateDnMat(&d2r, n_rows, R, n_rows, t2r, CUDA_R_64F, CUSPARSE_ORDER_COL));
  REF_TRY(cusparseCreateDnMat(&d2i, n_rows, R, n_rows, t2i, CUDA_R_64F, CUSPARSE_ORDER_COL));
  REF_TRY(cusparseCreateDnMat(&d1r, n_rows, R, n_rows, t1r, CUDA_R_64F, CUSPARSE_ORDER_COL));
  REF_TRY(cusparseCreateDnMat(&d1i, n_rows, R, n_rows, t1i, CUDA_R_64F, CUSPARSE_ORDER_COL));
  REF_TRY(cusparseCreate(&sp));
  REF_TRY(cublasCreate(&bl));
  REF_TRY(cusparseSpMM_bufferSize(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha0, A,
                                  d2r, &beta0, dbr, CUDA_R_64F, CUSPARSE_SPMM_ALG_DEFAULT, &bs1));
  REF_TRY(cusparseSpMM_bufferSize(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, A,
                                  d2r, &beta, dbr, CUDA_R_64F, CUSPARSE_SPMM_ALG_DEFAULT, &bs2));
  REF_TRY(cudaMalloc(&buf, bs1 > bs2 ? (bs1 ? bs1 : 1) : (bs2 ? bs2 : 1)));
  loop = Timer();
  // T_1 = M T_0 (both parts), mu_0 and mu_1
  REF_TRY(cusparseSpMM(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha0, A, d2r,
                       &beta0, d1r, CUDA_R_64F, CUSPARSE_SPMM_ALG_DEFAULT, buf));
  REF_TRY(cusparseSpMM(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha0, A, d2i,
                       &beta0, d1i, CUDA_R_64F, CUSPARSE_SPMM_ALG_DEFAULT, buf));
  REF_TRY(cublasDdot(bl, (int)NR, br, 1, t2r, 1, &a));
  REF_TRY(cublasDdot(bl, (int)NR, bi, 1, t2i, 1, &b));
  mu_out[0] = a + b;
  REF_TRY(cublasDdot(bl, (int)NR, br, 1, t1r, 1, &a));
  REF_TRY(cublasDdot(bl, (int)NR, bi, 1, t1i, 1, &b));
  mu_out[1] = a + b;
  for (int32_t i = 2; i < n; ++i) {
    // T_2 <- 2 M T_1 - T_2 in place, then the roles swap
    REF_TRY(cusparseSpMM(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, A, d1r,
                         &beta, d2r, CUDA_R_64F, CUSPARSE_SPMM_ALG_DEFAULT, buf));
    REF_TRY(cusparseSpMM(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &alpha, A, d1i,
                         &beta, d2i, CUDA_R_64F, CUSPARSE_SPMM_ALG_DEFAULT, buf));
    REF_TRY(cublasDdot(bl, (int)NR, br, 1, t2r, 1, &a));
    REF_TRY(cublasDdot(bl, (int)NR, bi, 1, t2i, 1, &b));
    mu_out[i] = a + b;
    std::swap(d1r, d2r);
    std::swap(d1i, d2i);
    std::swap(t1r, t2r);
    std::swap(t1i, t2i);
  }
  if (times_ms) times_ms[1] = loop.ms();
done:
  if (buf) cudaFree(buf);
  if (sp) cusparseDestroy(sp);
  if (bl) cublasDestroy(bl);
  for (cusparseDnMatDescr_t d : {dbr, dbi, d2r, d2i, d1r, d1i})
    if (d) cusparseDestroyDnMat(d);
  if (A) cusparseDestroySpMat(A);
  for (void* p : {(void*)d_cp, (void*)d_ri, (void*)d_v, (void*)br, (void*)bi, (void*)t2r, (void*)t2i, (void*)t1r,
                  (void*)t1i})
    if (p) cudaFree(p);
  if (times_ms) times_ms[0] = all.ms();
  return status;
}

int ref_cusparse_braket_complex(int32_t n_rows, int64_t nnz, const int32_t* cp, const int32_t* ri, const double* v,
                                int32_t n, const double* bras, const double* kets, int32_t R, double* mu_out,
                                double* times_ms) {
  Timer all;
  if (n < 2) return -1;
  int status = 0;
  const int64_t NR = (int64_t)n_rows * R;
  int32_t *d_cp = nullptr, *d_ri = nullptr;
  cuDoubleComplex *d_v = nullptr, *db = nullptr, *t2 = nullptr, *t1 = nullptr;
  void* buf = nullptr;
  cusparseHandle_t sp = nullptr;
  cublasHandle_t bl = nullptr;
  cusparseSpMatDescr_t A = nullptr;
  cusparseDnMatDescr_t dB = nullptr, d2 = nullptr, d1 = nullptr;
  const size_t vb = sizeof(cuDoubleComplex) * NR;
  cuDoubleComplex one{1.0, 0.0}, zero{0.0, 0.0}, two{2.0, 0.0}, mone{-1.0, 0.0}, tr{0.0, 0.0};
  size_t bs1 = 0, bs2 = 0;
  Timer loop;
  REF_TRY(cudaMalloc(&d_cp, sizeof(int32_t) * (n_rows + 1)));
  REF_TRY(cudaMalloc(&d_ri, sizeof(int32_t) * (nnz ? nnz : 1)));
  REF_TRY(cudaMalloc(&d_v, sizeof(cuDoubleComplex) * (nnz ? nnz : 1)));
  REF_TRY(cudaMemcpy(d_cp, cp, sizeof(int32_t) * (n_rows + 1), cudaMemcpyHostToDevice));
  REF_TRY(cudaMemcpy(d_ri, ri, sizeof(int32_t) * nnz, cudaMemcpyHostToDevice));
  REF_TRY(cudaMemcpy(d_v, v, sizeof(cuDoubleComplex) * nnz, cudaMemcpyHostToDevice));
  for (cuDoubleComplex** p : {&db, &t2, &t1}) REF_TRY(cudaMalloc(p, vb));
  REF_TRY(cudaMemcpy(db, bras, vb, cudaMemcpyHostToDevice));
  REF_TRY(cudaMemcpy(t2, kets, vb, cudaMemcpyHostToDevice));
  REF_TRY(cusparseCreateCsc(&A, n_rows, n_rows, nnz, d_cp, d_ri, d_v, CUSPARSE_INDEX_32I, CUSPARSE_INDEX_32I,
                            CUSPARSE_INDEX_BASE_ZERO, CUDA_C_64F));
  REF_TRY(cusparseCreateDnMat(&dB, n_rows, R, n_rows, db, CUDA_C_64F, CUSPARSE_ORDER_COL));
  REF_TRY(cusparseCreateDnMat(&d2, n_rows, R, n_rows, t2, CUDA_C_64F, CUSPARSE_ORDER_COL));
  REF_TRY(cusparseCreateDnMat(&d1, n_rows, R, n_rows, t1, CUDA_C_64F, CUSPARSE_ORDER_COL));
  REF_TRY(cusparseCreate(&sp));
  REF_TRY(cublasCreate(&bl));
  REF_TRY(cusparseSpMM_bufferSize(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, A, d2,
                                  &zero, dB, CUDA_C_64F, CUSPARSE_SPMM_ALG_DEFAULT, &bs1));
  REF_TRY(cusparseSpMM_bufferSize(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &two, A, d2,
                                  &mone, dB, CUDA_C_64F, CUSPARSE_SPMM_ALG_DEFAULT, &bs2));
  REF_TRY(cudaMalloc(&buf, bs1 > bs2 ? (bs1 ? bs1 : 1) : (bs2 ? bs2 : 1)));
  loop = Timer();
  REF_TRY(cusparseSpMM(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &one, A, d2, &zero, d1,
                       CUDA_C_64F, CUSPARSE_SPMM_ALG_DEFAULT, buf));
  REF_TRY(cublasZdotc(bl, (int)NR, db, 1, t2, 1, &tr));
  mu_out[0] = tr.x;
  REF_TRY(cublasZdotc(bl, (int)NR, db, 1, t1, 1, &tr));
  mu_out[1] = tr.x;
  for (int32_t i = 2; i < n; ++i) {
    REF_TRY(cusparseSpMM(sp, CUSPARSE_OPERATION_NON_TRANSPOSE, CUSPARSE_OPERATION_NON_TRANSPOSE, &two, A, d1, &mone,
                         d2, CUDA_C_64F, CUSPARSE_SPMM_ALG_DEFAULT, buf));
    REF_TRY(cublasZdotc(bl, (int)NR, db, 1, t2, 1, &tr));
    mu_out[i] = tr.x;
    std::swap(d1, d2);
    std::swap(t1, t2);
  }
  if (times_ms) times_ms[1] = loop.ms();
done:
  if (buf) cudaFree(buf);
  if (sp) cusparseDestroy(sp);
  if (bl) cublasDestroy(bl);
  for (cusparseDnMatDescr_t d : {dB, d2, d1})
    if (d) cusparseDestroyDnMat(d);
  if (A) cusparseDestroySpMat(A);
  for (void* p : {(void*)d_cp, (void*)d_ri, (void*)d_v, (void*)db, (void*)t2, (void*)t1})
    if (p) cudaFree(p);
  if (times_ms) times_ms[0] = all.ms();
  return status;
}

}  // extern "C"
