// The drop-in shim (include/tbk_numerics_cuda.hpp) compiled the way the
// reference would compile it: the two cuda::Cheb_first_kind_seq_braket
// overloads declared as in the reference's numerics_cuda.cuh, their bodies from
// the shim, Eigen replaced by the stand-in under tests/cpp/eigen_standin.
// Checks (exit code 0 when all pass):
//   1. real ring, identity kets: mu_n = sum_k T_n(2 cos(2 pi k / N) / a), 1e-10
//   2. complex ring with a flux phase: sum_k T_n(2 cos(2 pi k / N + phi) / a)
//   3. bras a copy of kets (plain braket path) equals bras == kets (doubling)
//   4. n < 2 returns an empty vector
#include <cmath>
#include <complex>
#include <cstdio>
#include <type_traits>
#include <vector>

#include <Eigen/Dense>
#include <Eigen/Sparse>

namespace cuda {
std::vector<double> Cheb_first_kind_seq_braket(const Eigen::SparseMatrix<double>& M, int n,
                                               const Eigen::MatrixXcd& bras_T, const Eigen::MatrixXcd& kets);
std::vector<double> Cheb_first_kind_seq_braket(const Eigen::SparseMatrix<std::complex<double>>& M, int n,
                                               const Eigen::MatrixXcd& bras_T, const Eigen::MatrixXcd& kets);
}  // namespace cuda

#include "tbk_numerics_cuda.hpp"

using cd = std::complex<double>;
static int failures = 0;
static void expect(bool ok, const char* what, double v) {
  std::printf("%s %s (%.3g)\n", ok ? "PASS" : "FAIL", what, v);
  if (!ok) ++failures;
}

// periodic ring with hopping t e^{i phi} from site j to j + 1; column j holds
// rows j - 1 and j + 1 (sorted); H~ = H / a
template <typename S>
static Eigen::SparseMatrix<S> ring(int N, double a, double phi) {
  std::vector<int> outer(N + 1), inner;
  std::vector<S> vals;
  for (int j = 0; j < N; ++j) {
    outer[j] = (int)inner.size();
    const int lo = (j + N - 1) % N, hi = (j + 1) % N;
    S up, dn;
    if constexpr (std::is_same<S, double>::value) {
      up = 1.0 / a;
      dn = 1.0 / a;
    } else {
      up = std::polar(1.0 / a, phi);     // H[j+1][j]
      dn = std::polar(1.0 / a, -phi);    // H[j-1][j]
    }
    if (lo < hi) {
      inner.push_back(lo); vals.push_back(dn);
      inner.push_back(hi); vals.push_back(up);
    } else {
      inner.push_back(hi); vals.push_back(up);
      inner.push_back(lo); vals.push_back(dn);
    }
  }
  outer[N] = (int)inner.size();
  return Eigen::SparseMatrix<S>(N, N, outer, inner, vals);
}

static double exact(int N, double a, double phi, int n) {
  double s = 0.0;
  for (int k = 0; k < N; ++k) s += std::cos(n * std::acos(2.0 * std::cos(2.0 * M_PI * k / N + phi) / a));
  return s;
}

int main() {
  if (tbk_device_count() < 1) {
    std::printf("FAIL no CUDA device\n");
    return 2;
  }
  const int N = 64, M = 96;
  const double a = 2.5, phi = 0.3;
  Eigen::MatrixXcd I(N, N);
  for (int i = 0; i < N; ++i) I(i, i) = 1.0;
  {
    auto H = ring<double>(N, a, 0.0);
    auto mu = cuda::Cheb_first_kind_seq_braket(H, M, I, I);
    double err = (int)mu.size() == M ? 0.0 : 1.0;
    for (int n = 0; n < (int)mu.size(); ++n) err = std::max(err, std::abs(mu[n] - exact(N, a, 0.0, n)) / N);
    expect(err <= 1e-10, "real ring: exact traces", err);
    Eigen::MatrixXcd B = I;                              // same values, another pointer: plain braket path
    auto mb = cuda::Cheb_first_kind_seq_braket(H, M, B, I);
    double e3 = mb.size() == mu.size() ? 0.0 : 1.0;
    for (size_t n = 0; n < mb.size() && n < mu.size(); ++n) e3 = std::max(e3, std::abs(mb[n] - mu[n]) / N);
    expect(e3 <= 1e-12, "braket path equals doubling path", e3);
    expect(cuda::Cheb_first_kind_seq_braket(H, 1, I, I).empty(), "n < 2 returns an empty vector", 0.0);
  }
  {
    auto H = ring<cd>(N, a, phi);
    auto mu = cuda::Cheb_first_kind_seq_braket(H, M, I, I);
    double err = (int)mu.size() == M ? 0.0 : 1.0;
    for (int n = 0; n < (int)mu.size(); ++n) err = std::max(err, std::abs(mu[n] - exact(N, a, phi, n)) / N);
    expect(err <= 1e-10, "complex ring with flux: exact traces", err);
  }
  tbk_cheb_braket_release();
  if (failures == 0) std::printf("ALL PASSED\n");
  return failures ? 1 : 0;
}
