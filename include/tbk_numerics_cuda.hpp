/*
 * tbk_numerics_cuda.hpp — the bodies of the reference's two GPU moment
 * overloads, cuda::Cheb_first_kind_seq_braket (declared in
 * tight_binding/numerics_cuda.cuh:8-14, defined in
 * tight_binding/numerics_cuda.cu:190-323), forwarded to libtbk's C ABI.
 *
 * Use: in the reference, replace the body of numerics_cuda.cu with
 *     #include "numerics_cuda.cuh"
 *     #include "tbk_numerics_cuda.hpp"
 * and link libtbk.so.  The overloads are defined here with external linkage,
 * so include this header in exactly one translation unit.
 * GreenFunctionImag (tight_binding/lattice.h:608-612) keeps calling the same
 * overloads under USE_CUDA.  Only these Eigen members are used:
 * SparseMatrix::rows / nonZeros / outerIndexPtr / innerIndexPtr / valuePtr
 * (compressed CSC, int32 indices: the reference's requirement too) and
 * MatrixXcd::data / cols (column-major complex<double>).
 *
 * Behaviour kept from the reference: n < 2 prints "n must be greater than or
 * equal to 2" to std::cerr and returns an empty vector.  Changed: a failing
 * call prints libtbk's message and returns an empty vector instead of
 * silently returning garbage.  TBK_SHIM_FLAGS (default TBK_PREC_FP64) picks
 * the precision; bras and kets that are the same matrix use the doubling
 * path (half the recursion steps).
 */
#ifndef TBK_NUMERICS_CUDA_HPP
#define TBK_NUMERICS_CUDA_HPP

#include <complex>
#include <cstdint>
#include <iostream>
#include <vector>

#include "tbk.h"

#ifndef TBK_SHIM_FLAGS
#define TBK_SHIM_FLAGS TBK_PREC_FP64
#endif

namespace cuda {
namespace tbk_shim {
template <typename SparseM>
std::vector<double> braket(const SparseM& M, int n, const Eigen::MatrixXcd& bras_T, const Eigen::MatrixXcd& kets,
                           bool cplx) {
  if (n < 2) {
    std::cerr << "n must be greater than or equal to 2" << std::endl;
    return {};
  }
  std::vector<double> mu(n);
  const bool same = bras_T.data() == kets.data();
  const int32_t flags = TBK_SHIM_FLAGS | (same ? TBK_FLAG_DOUBLING : 0);
  const double* b = reinterpret_cast<const double*>(bras_T.data());
  const double* k = reinterpret_cast<const double*>(kets.data());
  const double* v = reinterpret_cast<const double*>(M.valuePtr());
  const int s = cplx ? tbk_cheb_braket_complex((int32_t)M.rows(), (int64_t)M.nonZeros(), M.outerIndexPtr(),
                                               M.innerIndexPtr(), v, n, b, k, (int32_t)kets.cols(), flags, mu.data())
                     : tbk_cheb_braket_real((int32_t)M.rows(), (int64_t)M.nonZeros(), M.outerIndexPtr(),
                                            M.innerIndexPtr(), v, n, b, k, (int32_t)kets.cols(), flags, mu.data());
  if (s != TBK_OK) {
    std::cerr << tbk_last_error() << std::endl;
    return {};
  }
  return mu;
}
}  // namespace tbk_shim

std::vector<double> Cheb_first_kind_seq_braket(const Eigen::SparseMatrix<double>& M, int n,
                                               const Eigen::MatrixXcd& bras_T, const Eigen::MatrixXcd& kets) {
  return tbk_shim::braket(M, n, bras_T, kets, false);
}
std::vector<double> Cheb_first_kind_seq_braket(const Eigen::SparseMatrix<std::complex<double>>& M, int n,
                                               const Eigen::MatrixXcd& bras_T, const Eigen::MatrixXcd& kets) {
  return tbk_shim::braket(M, n, bras_T, kets, true);
}
}  // namespace cuda

#endif /* TBK_NUMERICS_CUDA_HPP */
