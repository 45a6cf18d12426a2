// tbk.hpp — C++17 mirror of the kernel-polynomial API of chenzehan/tight_binding
// over libtbk's C ABI (tbk.h).  Same names, argument meaning and error
// behaviour as the reference where it has them:
//   UnitCell<Dim>                      TB/unit_cell.h:65-156
//   PartialLattice<Dim>                TB/lattice.h:22-103
//   GreenFunction / GreenFunctionImag  TB/lattice.h:545-647
//   matrix_spectral_range_sparse       TB/numerical.h:24-46 (device Lanczos)
//   cheb_expand / time_evolve          TB/numerical.h:346-361
//   Cheb_first_kind_seq_view           TB/numerical.h:346-361
//   cuda::Cheb_first_kind_seq_braket   TB/numerics_cuda.cuh:10-13
//   bases_of_uniform_ampl_with_random_phases  TB/numerical.h:120-122 (seeded)
//   density_of_states_seq              TB/functions.h:15-32
//   DosServer                          (no counterpart: many solves advanced together)
// Sparse matrices live on the device (SparseMatrix owns a tbk_sparse); dense
// blocks use the Eigen::MatrixXcd layout (column-major complex128).  Failures
// throw std::runtime_error carrying tbk_last_error(); the reference's
// "n must be greater than or equal to 2" case is a throw as well.
#pragma once
#include <array>
#include <complex>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <tuple>
#include <type_traits>
#include <utility>
#include <vector>

#include "tbk.h"

namespace tbk {

using Complex = std::complex<double>;
using Vector3d = std::array<double, 3>;
template <int Dim>
using LatticeVector = std::array<int32_t, Dim>;

inline void check(int status) {
  if (status != TBK_OK)
    throw std::runtime_error("tbk error " + std::to_string(status) + ": " + tbk_last_error());
}

// Column-major rows x cols complex128 block: the layout of Eigen::MatrixXcd.
struct MatrixXcd {
  int32_t rows = 0, cols = 0;
  std::vector<Complex> data;
  MatrixXcd() = default;
  MatrixXcd(int32_t r, int32_t c) : rows(r), cols(c), data((size_t)r * (size_t)c) {}
  Complex& operator()(int32_t i, int32_t j) { return data[(size_t)j * rows + i]; }
  const Complex& operator()(int32_t i, int32_t j) const { return data[(size_t)j * rows + i]; }
  const double* raw() const { return reinterpret_cast<const double*>(data.data()); }
  double* raw() { return reinterpret_cast<double*>(data.data()); }
  static MatrixXcd Identity(int32_t n) {
    MatrixXcd m(n, n);
    for (int32_t i = 0; i < n; ++i) m(i, i) = 1.0;
    return m;
  }
};

// |r>_i = exp(2 pi i u)/sqrt(n), u = the seeded counter-based uniform (the
// reference draws from std::rand; every column has unit norm either way).
inline MatrixXcd bases_of_uniform_ampl_with_random_phases(int32_t n, int32_t m, uint64_t seed = 0) {
  MatrixXcd k(n, m);
  check(tbk_random_phase_kets(n, m, seed, k.raw()));
  return k;
}

template <int Dim>
class UnitCell {
 public:
  UnitCell(const std::vector<Vector3d>& lattice_vectors, const std::vector<std::pair<std::string, Vector3d>>& atoms) {
    if ((int)lattice_vectors.size() != Dim) throw std::invalid_argument("UnitCell: one lattice vector per dimension");
    std::vector<double> lv, pos;
    std::vector<const char*> names;
    for (const auto& v : lattice_vectors) lv.insert(lv.end(), v.begin(), v.end());
    for (const auto& a : atoms) {
      names.push_back(a.first.c_str());
      pos.insert(pos.end(), a.second.begin(), a.second.end());
    }
    check(tbk_cell_create(&h_, Dim, lv.data(), (int32_t)atoms.size(), names.data(), pos.data()));
  }
  UnitCell(const UnitCell& o) { check(tbk_cell_copy(&h_, o.h_)); }
  UnitCell& operator=(const UnitCell& o) {
    if (this != &o) {
      tbk_cell c = nullptr;
      check(tbk_cell_copy(&c, o.h_));
      tbk_cell_destroy(h_);
      h_ = c;
    }
    return *this;
  }
  ~UnitCell() { tbk_cell_destroy(h_); }

  // explicit hopping from -> to across lattice_vector (TB/unit_cell.h:188-205)
  UnitCell& add_hopping(const std::string& from, const std::string& to, LatticeVector<Dim> lattice_vector,
                        Complex t) {
    int32_t v[3] = {0, 0, 0};
    for (int i = 0; i < Dim; ++i) v[i] = lattice_vector[i];
    check(tbk_cell_add_hopping(h_, from.c_str(), to.c_str(), v, t.real(), t.imag()));
    return *this;
  }
  // every hopping of the n-th nearest-neighbour shell of `from` (TB/unit_cell.h:207-256)
  UnitCell& add_hopping(const std::string& from, int32_t NN, Complex t) {
    check(tbk_cell_add_hopping_nn(h_, from.c_str(), NN, t.real(), t.imag()));
    return *this;
  }
  int get_atom_number() const {
    int32_t d, a, h;
    check(tbk_cell_info(h_, &d, &a, &h));
    return a;
  }
  int get_atom_index(const std::string& name) const {
    int32_t i;
    check(tbk_cell_atom_index(h_, name.c_str(), &i));
    return i;
  }
  tbk_cell handle() const { return h_; }

 private:
  tbk_cell h_ = nullptr;
};

// Device-resident sparse matrix (Eigen-compatible CSC; the role of
// Eigen::SparseMatrix<Scalar> on this path).  Move-only.
class SparseMatrix {
 public:
  explicit SparseMatrix(tbk_sparse h = nullptr) : h_(h) {}
  SparseMatrix(SparseMatrix&& o) noexcept : h_(o.h_) { o.h_ = nullptr; }
  SparseMatrix& operator=(SparseMatrix&& o) noexcept {
    if (this != &o) { tbk_sparse_destroy(h_); h_ = o.h_; o.h_ = nullptr; }
    return *this;
  }
  SparseMatrix(const SparseMatrix&) = delete;
  SparseMatrix& operator=(const SparseMatrix&) = delete;
  ~SparseMatrix() { tbk_sparse_destroy(h_); }

  // from host CSC arrays (values: nnz doubles, or 2*nnz interleaved complex)
  static SparseMatrix from_csc(int32_t rows, int32_t cols, int64_t nnz, const int32_t* col_ptr,
                               const int32_t* row_idx, const double* values, bool is_complex) {
    tbk_sparse h = nullptr;
    check(tbk_sparse_from_csc(&h, rows, cols, nnz, col_ptr, row_idx, values, is_complex ? 1 : 0, 0, nullptr));
    return SparseMatrix(h);
  }
  int32_t rows() const { int32_t r, c, x; int64_t z; check(tbk_sparse_info(h_, &r, &c, &z, &x)); return r; }
  int32_t cols() const { int32_t r, c, x; int64_t z; check(tbk_sparse_info(h_, &r, &c, &z, &x)); return c; }
  int64_t nonZeros() const { int32_t r, c, x; int64_t z; check(tbk_sparse_info(h_, &r, &c, &z, &x)); return z; }
  bool is_complex() const { int32_t r, c, x; int64_t z; check(tbk_sparse_info(h_, &r, &c, &z, &x)); return x != 0; }
  // host copies of the three CSC arrays
  void download(std::vector<int32_t>& col_ptr, std::vector<int32_t>& row_idx, std::vector<double>& values) const {
    col_ptr.resize((size_t)cols() + 1);
    row_idx.resize((size_t)nonZeros());
    values.resize((size_t)nonZeros() * (is_complex() ? 2 : 1));
    check(tbk_sparse_download(h_, col_ptr.data(), row_idx.data(), values.data(), nullptr));
  }
  tbk_sparse handle() const { return h_; }

 private:
  tbk_sparse h_ = nullptr;
};

template <int Dim>
class PartialLattice {
 public:
  PartialLattice(const UnitCell<Dim>& cell, LatticeVector<Dim> span_size) {
    int32_t sp[3] = {1, 1, 1};
    for (int i = 0; i < Dim; ++i) sp[i] = span_size[i];
    check(tbk_lattice_create(&h_, cell.handle(), sp));
  }
  PartialLattice(const PartialLattice&) = delete;
  PartialLattice& operator=(const PartialLattice&) = delete;
  ~PartialLattice() { tbk_lattice_destroy(h_); }

  int get_total_number() const {
    int64_t n;
    check(tbk_lattice_total_number(h_, &n));
    return (int)n;
  }
  // on-site U[-W/2, W/2] from a seeded counter-based generator (the reference
  // fills set_scalar_field from a stateful RNG, TB/snippets.h:765-767)
  void set_scalar_disorder(double W, uint64_t seed) { check(tbk_lattice_set_scalar_disorder(h_, W, seed)); }
  void set_scalar_values(const std::vector<double>& V) { check(tbk_lattice_set_scalar_sites(h_, V.data())); }
  // vacancies, TB/lattice.h:389-418 (remove_atoms_random drawn from `seed`)
  void remove_atoms(const std::string& atom_name, const std::vector<LatticeVector<Dim>>& i) {
    std::vector<int32_t> c;
    c.reserve(i.size() * Dim);
    for (const auto& v : i)
      for (int d = 0; d < Dim; ++d) c.push_back(v[d]);
    check(tbk_lattice_remove_atoms(h_, atom_name.c_str(), c.data(), (int64_t)i.size()));
  }
  void remove_atoms_random(const std::string& atom_name, int n, uint64_t seed = 0) {
    check(tbk_lattice_remove_atoms_random(h_, atom_name.c_str(), n, seed));
  }
  // A(r) = G r + c (TB/lattice.h:495-505)
  void set_gauge_linear(const std::array<double, 9>& G_rowmajor, const Vector3d& c) {
    check(tbk_lattice_set_gauge_linear(h_, G_rowmajor.data(), c.data()));
  }

  template <class Scalar>
  SparseMatrix get_Hamiltonian_periodic_extend_bare_sparse(LatticeVector<Dim> extend) {
    int32_t e[3] = {0, 0, 0};
    for (int i = 0; i < Dim; ++i) e[i] = extend[i];
    return build(TBK_BUILD_PERIODIC_BARE, e, is_cplx<Scalar>());
  }
  template <class Scalar>
  SparseMatrix get_Hamiltonian_bare_sparse() { return build(TBK_BUILD_BARE, nullptr, is_cplx<Scalar>()); }
  template <class Scalar>
  SparseMatrix get_Hamiltonian_sparse() { return build(TBK_BUILD_SPARSE, nullptr, is_cplx<Scalar>()); }

  SparseMatrix op_position(int axis) {
    tbk_sparse h = nullptr;
    check(tbk_build_position(&h, h_, axis, nullptr));
    return SparseMatrix(h);
  }
  // X H - H X with the bare real Hamiltonian (TB/lattice.h:338-345)
  SparseMatrix op_velocity(int axis) {
    SparseMatrix H = get_Hamiltonian_bare_sparse<double>();
    SparseMatrix X = op_position(axis);
    tbk_sparse h = nullptr;
    check(tbk_sparse_commutator(&h, H.handle(), X.handle(), nullptr));
    return SparseMatrix(h);
  }
  // bond-displacement velocity (periodic axes as in `periodic`): each hopping
  // times scale * (r_i - r_j) along its own bond; scale = 1/a gives [X, H~]
  // wherever a bond does not wrap
  template <class Scalar>
  SparseMatrix op_velocity_bond(int axis, LatticeVector<Dim> periodic, double scale = 1.0) {
    int32_t ext[3] = {0, 0, 0};
    for (int i = 0; i < Dim; ++i) ext[i] = periodic[i];
    tbk_sparse h = nullptr;
    check(tbk_build_velocity_bond(&h, h_, TBK_BUILD_PERIODIC_BARE, ext, is_cplx<Scalar>(), axis, scale, nullptr));
    return SparseMatrix(h);
  }
  tbk_lattice handle() const { return h_; }

 private:
  template <class Scalar>
  static constexpr int is_cplx() { return std::is_same<Scalar, Complex>::value ? 1 : 0; }
  SparseMatrix build(int mode, const int32_t* extend, int cplx) {
    tbk_sparse h = nullptr;
    check(tbk_build_hamiltonian(&h, h_, mode, extend, cplx, nullptr));
    return SparseMatrix(h);
  }
  tbk_lattice h_ = nullptr;
};

namespace cuda {
// mu_k = Re tr(bras_T^dagger T_k(M) kets), k < n (TB/numerics_cuda.cu:190-323).
// precision: TBK_PREC_FP64 (the reference's complex128 recursion), TBK_PREC_DD
// or TBK_PREC_MIXED; bras == kets (same object) takes the doubling path.
inline std::vector<double> Cheb_first_kind_seq_braket(const SparseMatrix& M, int n, const MatrixXcd& bras_T,
                                                      const MatrixXcd& kets, int precision = TBK_PREC_FP64) {
  if (n < 2) throw std::invalid_argument("n must be greater than or equal to 2");
  if (bras_T.rows != M.rows() || kets.rows != M.rows() || bras_T.cols != kets.cols)
    throw std::invalid_argument("Cheb_first_kind_seq_braket: block shapes do not match the matrix");
  const bool same = &bras_T == &kets;
  tbk_kpm plan = nullptr;
  check(tbk_kpm_create(&plan, M.handle(), kets.cols, precision | (same ? TBK_FLAG_DOUBLING : 0)));
  std::vector<double> mu((size_t)n);
  const int s = tbk_kpm_run(plan, n, bras_T.raw(), kets.raw(), mu.data(), nullptr);
  tbk_kpm_destroy(plan);
  check(s);
  return mu;
}
}  // namespace cuda

// numerical::linalg::matrix_spectral_range_sparse (TB/numerical.h:24-46):
// extreme eigenvalues {E_min, E_max} of a Hermitian matrix, here by device
// Lanczos (no 5,000-row cap; Ritz values lie inside the spectrum)
inline std::pair<double, double> matrix_spectral_range_sparse(const SparseMatrix& A, int iters = 200,
                                                              uint64_t seed = 0) {
  double e0 = 0.0, e1 = 0.0;
  check(tbk_spectral_range(A.handle(), iters, seed, &e0, &e1, nullptr, nullptr, nullptr));
  return {e0, e1};
}

// GreenFunction<Scalar> (TB/lattice.h:553-576): b = (E_max + E_min)/2,
// scaled_HE = (HE - b I)/a on the device, with
//   GreenFunction(N, HE, E_min, E_max)          a = (E_max - E_min)/2
//   GreenFunction(N, HE, ref_HE, epsilon=0.01)  range of ref_HE, a = (E_max - E_min)/(2 - epsilon)
//   GreenFunction(N, HE)                        = GreenFunction(N, HE, HE)
struct GreenFunction {
  int N;
  double a, b, E_min, E_max;
  SparseMatrix scaled_HE;

  GreenFunction(int N_, const SparseMatrix& HE, double E_min_, double E_max_)
      : N(N_), a((E_max_ - E_min_) / 2), b((E_max_ + E_min_) / 2), E_min(E_min_), E_max(E_max_) {
    rescale(HE);
  }
  GreenFunction(int N_, const SparseMatrix& HE, const SparseMatrix& ref_HE, double epsilon = 0.01) : N(N_) {
    std::tie(E_min, E_max) = matrix_spectral_range_sparse(ref_HE);
    a = (E_max - E_min) / (2 - epsilon);
    b = (E_max + E_min) / 2;
    rescale(HE);
  }
  GreenFunction(int N_, const SparseMatrix& HE) : GreenFunction(N_, HE, HE) {}
  void rescale(const SparseMatrix& HE) {
    tbk_sparse h = nullptr;
    check(tbk_sparse_rescale(&h, HE.handle(), a, b, nullptr));
    scaled_HE = SparseMatrix(h);
  }
  double scale(double x, double id = 1.0) const { return (x - b * id) / a; }
  Complex scale(Complex x, Complex id) const { return (x - b * id) / a; }

  // e -> sum_n g_n Im(alpha_n(e)) mu_n with the Lorentz(N, 4) kernel the
  // reference hard-codes (TB/lattice.h:600-647)
  struct GreenFunctionImag {
    int N = 0;
    std::vector<double> moments, g;
    double operator()(Complex z) const {
      const double zz[2] = {z.real(), z.imag()};
      double out = 0.0;
      check(tbk_green_imag_eval(N, g.data(), moments.data(), 1, zz, &out, nullptr));
      return out;
    }
    double operator()(double e) const { return (*this)(Complex(e, 0.0)); }
    // DCT-III route (TB/lattice.h:625-640): {x_k, f(x_k)} on N*n Chebyshev nodes
    std::pair<std::vector<double>, std::vector<double>> fft(int n = 1) const {
      const int up = n > 1 ? n : 1;
      std::vector<double> E((size_t)N * up), v((size_t)N * up);
      check(tbk_green_imag_fft(N, g.data(), moments.data(), up, E.data(), v.data(), nullptr));
      return {E, v};
    }
  };
  GreenFunctionImag imag(const MatrixXcd& bras, const MatrixXcd& kets, int precision = TBK_PREC_FP64) const {
    GreenFunctionImag f;
    f.N = N;
    f.moments = cuda::Cheb_first_kind_seq_braket(scaled_HE, N, bras, kets, precision);
    f.g.resize((size_t)N);
    check(tbk_kernel_seq(TBK_KERNEL_LORENTZ, N, 4.0, 0.0, f.g.data()));
    return f;
  }
};

// sum_k coef[k] T_k(Ht) kets on the device: the Cheb_first_kind_seq_view walk
// plus host sum of TB/numerical.h:346-361 / TB/snippets.h:194-217 in one call
inline MatrixXcd cheb_expand(const SparseMatrix& Ht, const std::vector<Complex>& coef, const MatrixXcd& kets,
                             int precision = TBK_PREC_FP64) {
  MatrixXcd out(kets.rows, kets.cols);
  check(tbk_cheb_expand(Ht.handle(), (int32_t)coef.size(), reinterpret_cast<const double*>(coef.data()), kets.cols,
                        kets.raw(), out.raw(), precision, nullptr));
  return out;
}
// numerical::Chebyshev::expn_coef_alpha_seq (TB/numerical.h:304-316):
// 1/(z - x) = sum_k alpha_k(z) T_k(x)
inline std::vector<Complex> expn_coef_alpha_seq(Complex z, int n) {
  std::vector<Complex> a((size_t)n);
  check(tbk_expn_coef_alpha_seq(z.real(), z.imag(), n, reinterpret_cast<double*>(a.data())));
  return a;
}

// numerical::Chebyshev::Cheb_first_kind_seq_view (TB/numerical.h:346-361):
// next() -> {i, T_i(x) v}; the recursion state stays on the device
class Cheb_first_kind_seq_view {
 public:
  Cheb_first_kind_seq_view(const SparseMatrix& x, const MatrixXcd& v, int precision = TBK_PREC_FP64)
      : rows_(v.rows), cols_(v.cols) {
    check(tbk_cheb_view_create(&h_, x.handle(), v.cols, v.raw(), precision));
  }
  Cheb_first_kind_seq_view(const Cheb_first_kind_seq_view&) = delete;
  Cheb_first_kind_seq_view& operator=(const Cheb_first_kind_seq_view&) = delete;
  ~Cheb_first_kind_seq_view() { tbk_cheb_view_destroy(h_); }
  std::pair<int, MatrixXcd> next() {
    MatrixXcd out(rows_, cols_);
    int32_t i = 0;
    check(tbk_cheb_view_next(h_, &i, out.raw(), nullptr));
    return {i, out};
  }

 private:
  tbk_cheb_view h_ = nullptr;
  int32_t rows_, cols_;
};

// exp(-i HE t) kets for the Hamiltonian of G (HE = a scaled_HE + b)
inline MatrixXcd time_evolve(const GreenFunction& G, double t, const MatrixXcd& kets, double tol = 1e-15,
                             int precision = TBK_PREC_FP64) {
  int32_t k = 0;
  check(tbk_cheb_evolution_terms(G.a, t, tol, &k));
  std::vector<Complex> c((size_t)k);
  check(tbk_cheb_coef_evolution(G.a, G.b, t, k, reinterpret_cast<double*>(c.data())));
  return cheb_expand(G.scaled_HE, c, kets, precision);
}

// TB/functions.h:15-32: periodic bare H, G(N, H, E_min - 1e-8, E_max + 1e-8),
// R random-phase kets, DoS = -f(e) / (R pi) at every e of E_list (scaled units).
template <class Scalar, int Dim>
std::vector<double> density_of_states_seq(PartialLattice<Dim>& X, int N, const std::vector<double>& E_list,
                                          double E_min, double E_max, int R = 4, uint64_t seed = 0,
                                          int precision = TBK_PREC_FP64) {
  LatticeVector<Dim> ext;
  ext.fill(1);
  SparseMatrix H = X.template get_Hamiltonian_periodic_extend_bare_sparse<Scalar>(ext);
  GreenFunction G(N, H, E_min - 1e-8, E_max + 1e-8);
  MatrixXcd kets = bases_of_uniform_ampl_with_random_phases(X.get_total_number(), R, seed);
  auto f = G.imag(kets, kets, precision);
  std::vector<double> dos;
  dos.reserve(E_list.size());
  for (double e : E_list) dos.push_back(-1.0 / R / 3.14159265358979323846 * f(e));
  return dos;
}

// Many DoS solves advanced together (tbk_server_*): submit lattices, poll moments.
class DosServer {
 public:
  explicit DosServer(double budget_gb = 120.0, int steps_per_round = 16, bool autotune = true,
                     int max_resident = 4096, int result_arena_mb = 64, double step_gb = 2.0) {
    tbk_server_config cfg{budget_gb, steps_per_round, autotune ? 1 : 0, max_resident, result_arena_mb, step_gb};
    check(tbk_server_create(&h_, &cfg));
  }
  DosServer(const DosServer&) = delete;
  DosServer& operator=(const DosServer&) = delete;
  ~DosServer() { tbk_server_destroy(h_); }

  // periodic bare Hamiltonian of X (every axis periodic), bounds [e_min, e_max]
  template <int Dim>
  int64_t submit(const PartialLattice<Dim>& X, int n_mom, int R, uint64_t seed, double e_min, double e_max,
                 int precision = TBK_PREC_MIXED) {
    tbk_request q{};
    q.lattice = X.handle();
    q.build_mode = TBK_BUILD_PERIODIC_BARE;
    for (int i = 0; i < 3; ++i) q.extend[i] = i < Dim ? 1 : 0;
    q.is_complex = 0;
    q.n_mom = n_mom;
    q.R = R;
    q.precision = precision;
    q.seed = seed;
    q.e_min = e_min;
    q.e_max = e_max;
    int64_t t = 0;
    check(tbk_server_submit(h_, &q, &t));
    n_mom_[t] = n_mom;
    return t;
  }
  // conductivity request (TBK_REQ_KUBO_BASTIN / _GREENWOOD): H of X with the
  // given periodic axes (complex), v_a = [x_a, H~]; poll returns the
  // 2 M^2 doubles of g_m g_n mu_nm (row-major complex)
  template <int Dim>
  int64_t submit_kubo(const PartialLattice<Dim>& X, int kind, int M, int R, uint64_t seed, double e_min,
                      double e_max, std::array<int, 2> axes, LatticeVector<Dim> periodic, int kernel = TBK_KERNEL_LORENTZ,
                      double kernel_p0 = 6.0, int precision = TBK_PREC_DD) {
    tbk_request q{};
    q.lattice = X.handle();
    q.build_mode = TBK_BUILD_PERIODIC_BARE;
    for (int i = 0; i < 3; ++i) q.extend[i] = i < Dim ? periodic[i] : 0;
    q.is_complex = 1;
    q.n_mom = M;
    q.R = R;
    q.precision = precision;
    q.seed = seed;
    q.e_min = e_min;
    q.e_max = e_max;
    q.kind = kind;
    q.axis[0] = axes[0];
    q.axis[1] = axes[1];
    q.kernel = kernel;
    q.kernel_p0 = kernel_p0;
    int64_t t = 0;
    check(tbk_server_submit(h_, &q, &t));
    n_mom_[t] = 2 * M * M;
    return t;
  }
  // true and the moments when done within wait_ms; throws if the request failed
  bool poll(int64_t ticket, int wait_ms, std::vector<double>& mu, double times_ms[4] = nullptr) {
    mu.resize((size_t)n_mom_.at(ticket));
    const int s = tbk_server_poll(h_, ticket, wait_ms, mu.data(), times_ms);
    if (s == TBK_PENDING) return false;
    n_mom_.erase(ticket);
    check(s);
    return true;
  }
  tbk_server handle() const { return h_; }

 private:
  tbk_server h_ = nullptr;
  std::map<int64_t, int> n_mom_;
};

}  // namespace tbk
