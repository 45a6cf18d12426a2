// C++ use of the kernel-polynomial path through include/tbk.hpp, written the
// way the reference's own drivers use its API (TB/functions.h, TB/snippets.h).
// Prints one line per check and exits non-zero on the first failure.
//   1. ring of 96 sites, t = 1, periodic: moments with identity kets against
//      the exact traces sum_k T_n(2 cos(2 pi k / N) / a)  (FP64, DD: 1e-10;
//      mixed: 2e-5 of mu_0)
//   2. n < 2 is rejected with the reference's message
//   3. density_of_states_seq on a disordered square lattice: non-negative on
//      the grid, integrates to ~1 (trapezoid), matches the DCT-III route
//   4. bras != kets (plain braket) equals bras == kets (doubling) on the same
//      kets to 1e-12
//   5. DosServer: a double-float request equals the FP64 solve to 1e-10, and
//      the same request twice gives the same bits
//   6. GreenFunction(N, H): the Lanczos range of a ring is [-2, 2] (1e-8) and
//      a = 4 / (2 - 0.01)
//   7. time_evolve on the ring: plane wave k picks up exp(-i 2 cos(k) t) (1e-11)
//   8. remove_atoms_random on a honeycomb: the open-BC Hamiltonian keeps
//      total - n columns with entries, the rest empty (compressed index)
//   9. moment file round trip through tbk_moments_save / tbk_moments_load
//  10. Cheb_first_kind_seq_view on a ring plane wave: T_i(H~) v = T_i(lambda) v
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "tbk.hpp"

using namespace tbk;

static int failures = 0;
static void expect(bool ok, const char* what, double value) {
  std::printf("%s %s (%.3g)\n", ok ? "PASS" : "FAIL", what, value);
  if (!ok) ++failures;
}

int main() {
  if (tbk_device_count() < 1) {
    std::printf("FAIL no CUDA device\n");
    return 2;
  }
  const double pi = 3.14159265358979323846;
  // ---- 1. ring: exact traces
  {
    const int L = 96, M = 64;
    UnitCell<1> chain({{1, 0, 0}}, {{"A", {0, 0, 0}}});
    chain.add_hopping("A", 1, Complex(1.0, 0.0));
    PartialLattice<1> X(chain, {L});
    SparseMatrix H = X.get_Hamiltonian_periodic_extend_bare_sparse<double>({1});
    const double a = 2.05;
    GreenFunction G(M, H, -a, a);
    std::vector<double> exact(M, 0.0);
    for (int k = 0; k < L; ++k) {
      const double th = std::acos(2.0 * std::cos(2 * pi * k / L) / a);
      for (int n = 0; n < M; ++n) exact[n] += std::cos(n * th);
    }
    MatrixXcd eye = MatrixXcd::Identity(L);
    for (int prec : {TBK_PREC_FP64, TBK_PREC_DD, TBK_PREC_MIXED}) {
      auto mu = cuda::Cheb_first_kind_seq_braket(G.scaled_HE, M, eye, eye, prec);
      double err = 0.0;
      for (int n = 0; n < M; ++n) err = std::fmax(err, std::fabs(mu[n] - exact[n]) / L);
      const double tol = prec == TBK_PREC_MIXED ? 2e-5 : 1e-10;
      const std::string what = std::string("ring exact traces, precision ") + std::to_string(prec);
      expect(err <= tol, what.c_str(), err);
    }
  }
  // ---- 2. the reference's n >= 2 rule
  {
    UnitCell<1> chain({{1, 0, 0}}, {{"A", {0, 0, 0}}});
    chain.add_hopping("A", 1, Complex(1.0, 0.0));
    PartialLattice<1> X(chain, {8});
    SparseMatrix H = X.get_Hamiltonian_periodic_extend_bare_sparse<double>({1});
    MatrixXcd k = bases_of_uniform_ampl_with_random_phases(8, 2, 1);
    bool threw = false;
    try {
      cuda::Cheb_first_kind_seq_braket(H, 1, k, k);
    } catch (const std::invalid_argument& e) {
      threw = std::string(e.what()).find("n must be greater than or equal to 2") != std::string::npos;
    }
    expect(threw, "n < 2 rejected with the reference's message", 0.0);
  }
  // ---- 3. DoS of a disordered square lattice
  {
    UnitCell<2> square({{1, 0, 0}, {0, 1, 0}}, {{"A", {0, 0, 0}}});
    square.add_hopping("A", 1, Complex(1.0, 0.0));
    PartialLattice<2> X(square, {48, 48});
    X.set_scalar_disorder(1.0, 5);
    const int N = 256;
    std::vector<double> e_list;
    for (int i = 0; i < 801; ++i) e_list.push_back(-0.998 + 1.996 * i / 800.0);
    auto dos = density_of_states_seq<double>(X, N, e_list, -4.6, 4.6, 8, 3);
    double mn = 1e30, integral = 0.0;
    for (size_t i = 0; i < dos.size(); ++i) {
      mn = std::fmin(mn, dos[i]);
      if (i) integral += 0.5 * (dos[i] + dos[i - 1]) * (e_list[i] - e_list[i - 1]);
    }
    expect(mn > -1e-3, "DoS non-negative on the grid", mn);
    expect(std::fabs(integral - 1.0) < 2e-2, "DoS integrates to 1 (scaled units)", integral);
    // the same moments through the DCT-III route at its nodes: it returns
    // sum (2 - d_n0) g_n mu_n T_n(x) / sqrt(1 - x^2) = -f(x), since
    // Im alpha_n(x) = -(2 - d_n0) T_n(x) / sqrt(1 - x^2)
    SparseMatrix H = X.get_Hamiltonian_periodic_extend_bare_sparse<double>({1, 1});
    GreenFunction G(N, H, -4.6 - 1e-8, 4.6 + 1e-8);
    MatrixXcd kets = bases_of_uniform_ampl_with_random_phases(X.get_total_number(), 8, 3);
    auto f = G.imag(kets, kets);
    auto ev = f.fft(1);
    double diff = 0.0, scale = 0.0;
    for (int i = 0; i < N; i += 17) {
      diff = std::fmax(diff, std::fabs(ev.second[i] + f(ev.first[i])));
      scale = std::fmax(scale, std::fabs(ev.second[i]));
    }
    expect(diff <= 1e-9 * scale, "DCT-III route equals direct evaluation", diff / scale);
  }
  // ---- 4. plain braket vs doubling
  {
    UnitCell<2> hc({{1.5, -0.8660254037844386, 0}, {1.5, 0.8660254037844386, 0}}, {{"A", {0, 0, 0}}, {"B", {1, 0, 0}}});
    hc.add_hopping("A", 1, Complex(-2.7, 0.0));
    PartialLattice<2> X(hc, {24, 24});
    X.set_scalar_disorder(0.8, 2);
    SparseMatrix H = X.get_Hamiltonian_periodic_extend_bare_sparse<double>({1, 1});
    GreenFunction G(100, H, -8.7, 8.7);
    MatrixXcd k1 = bases_of_uniform_ampl_with_random_phases(X.get_total_number(), 6, 9);
    MatrixXcd k2 = k1;                                   // distinct object: plain braket path
    auto mu_d = cuda::Cheb_first_kind_seq_braket(G.scaled_HE, 100, k1, k1);
    auto mu_p = cuda::Cheb_first_kind_seq_braket(G.scaled_HE, 100, k2, k1);
    double err = 0.0;
    for (int n = 0; n < 100; ++n) err = std::fmax(err, std::fabs(mu_d[n] - mu_p[n]) / mu_p[0]);
    expect(err < 1e-12, "doubling equals the plain braket (FP64)", err);
  }
  // ---- 5. the serving API: a request through the server equals the same
  //         request alone (moments of the same seeded kets)
  {
    UnitCell<2> square({{1, 0, 0}, {0, 1, 0}}, {{"A", {0, 0, 0}}});
    square.add_hopping("A", 1, Complex(1.0, 0.0));
    PartialLattice<2> X(square, {40, 40});
    X.set_scalar_disorder(0.6, 4);
    DosServer srv(4.0, 8, false);
    const int64_t a = srv.submit(X, 96, 8, 11, -4.4, 4.4, TBK_PREC_DD);
    const int64_t b = srv.submit(X, 96, 8, 11, -4.4, 4.4, TBK_PREC_DD);
    std::vector<double> ma, mb;
    int tries = 0;
    while (!srv.poll(a, 100, ma) && ++tries < 600) {}
    tries = 0;
    while (!srv.poll(b, 100, mb) && ++tries < 600) {}
    SparseMatrix H = X.get_Hamiltonian_periodic_extend_bare_sparse<double>({1, 1});
    GreenFunction G(96, H, -4.4, 4.4);
    MatrixXcd kets = bases_of_uniform_ampl_with_random_phases(X.get_total_number(), 8, 11);
    auto ref = cuda::Cheb_first_kind_seq_braket(G.scaled_HE, 96, kets, kets, TBK_PREC_FP64);
    double err = 0.0, same = 0.0;
    for (int n = 0; n < 96 && ma.size() == 96 && mb.size() == 96; ++n) {
      err = std::fmax(err, std::fabs(ma[n] - ref[n]) / ref[0]);
      same = std::fmax(same, std::fabs(ma[n] - mb[n]));
    }
    expect(ma.size() == 96 && err <= 1e-10, "server (double-float) equals the FP64 solve", err);
    expect(same == 0.0, "the same request twice gives the same bits", same);
  }
  // ---- 6. bound-free GreenFunction: Lanczos spectral range
  {
    UnitCell<1> chain({{1, 0, 0}}, {{"A", {0, 0, 0}}});
    chain.add_hopping("A", 1, Complex(1.0, 0.0));
    PartialLattice<1> X(chain, {96});
    SparseMatrix H = X.get_Hamiltonian_periodic_extend_bare_sparse<double>({1});
    GreenFunction G(64, H);
    const double err = std::fmax(std::fabs(G.E_min + 2.0), std::fabs(G.E_max - 2.0));
    expect(err <= 1e-8, "GreenFunction(N, H) range of the ring", err);
    expect(std::fabs(G.a - 4.0 / 1.99) <= 1e-8, "GreenFunction(N, H) contraction epsilon 0.01", G.a);
  }
  // ---- 7. time evolution of a plane wave on the ring
  {
    const int L = 96;
    UnitCell<1> chain({{1, 0, 0}}, {{"A", {0, 0, 0}}});
    chain.add_hopping("A", 1, Complex(1.0, 0.0));
    PartialLattice<1> X(chain, {L});
    SparseMatrix H = X.get_Hamiltonian_periodic_extend_bare_sparse<double>({1});
    GreenFunction G(16, H, -2.1, 2.1);
    const int q = 7;
    const double kq = 2 * pi * q / L, t = 4.5;
    MatrixXcd psi(L, 1);
    for (int i = 0; i < L; ++i) psi(i, 0) = std::polar(1.0 / std::sqrt((double)L), kq * i);
    MatrixXcd out = time_evolve(G, t, psi);
    const Complex ph = std::polar(1.0, -2.0 * std::cos(kq) * t);
    double err = 0.0;
    for (int i = 0; i < L; ++i) err = std::fmax(err, std::abs(out(i, 0) - ph * psi(i, 0)));
    expect(err <= 1e-11, "time_evolve plane wave phase", err);
  }
  // ---- 8. vacancies
  {
    UnitCell<2> hc({{1.5, 0.8660254037844386, 0}, {1.5, -0.8660254037844386, 0}}, {{"A", {0, 0, 0}}, {"B", {1, 0, 0}}});
    hc.add_hopping("A", 1, Complex(-2.7, 0.0));
    PartialLattice<2> X(hc, {32, 24});
    X.remove_atoms_random("B", 100, 7);
    X.remove_atoms("A", {{0, 0}, {5, 6}});
    SparseMatrix H = X.get_Hamiltonian_sparse<double>();
    std::vector<int32_t> cp, ri;
    std::vector<double> v;
    H.download(cp, ri, v);
    const int kept = 2 * 32 * 24 - 102;
    // columns past the kept count are empty; the kept block holds the bonds
    int nonempty = 0;
    for (int j = 0; j < kept; ++j) nonempty += cp[j + 1] > cp[j];
    const bool ok = cp.size() == (size_t)(2 * 32 * 24 + 1) && cp[kept] == cp.back() && nonempty > kept - 20 &&
                    cp.back() % 2 == 0;
    expect(ok, "remove_atoms(_random): compressed open-BC Hamiltonian", (double)nonempty);
  }
  // ---- 9. moment files
  {
    std::vector<double> mu(300);
    for (size_t k = 0; k < mu.size(); ++k) mu[k] = std::cos(0.1 * (double)k) / (1.0 + (double)k);
    tbk_moments_header h{};
    h.kind = TBK_MOMENTS_DOS;
    h.rows = (int32_t)mu.size();
    h.cols = 1;
    h.R = 8;
    h.seed = 42;
    h.e_min = -4.05;
    h.e_max = 4.05;
    std::snprintf(h.label, sizeof(h.label), "square 64x64");
    const char* path = "tbk_cpp_moments.tbm";
    check(tbk_moments_save(path, &h, mu.data()));
    tbk_moments_header g{};
    std::vector<double> back(mu.size());
    check(tbk_moments_load(path, &g, back.data(), (int64_t)back.size()));
    std::remove(path);
    const bool ok = back == mu && g.R == 8 && g.seed == 42 && std::string(g.label) == "square 64x64";
    expect(ok, "moment file round trip", 0.0);
  }
  // ---- 10. Cheb_first_kind_seq_view
  {
    const int L = 64;
    UnitCell<1> chain({{1, 0, 0}}, {{"A", {0, 0, 0}}});
    chain.add_hopping("A", 1, Complex(1.0, 0.0));
    PartialLattice<1> X(chain, {L});
    SparseMatrix H = X.get_Hamiltonian_periodic_extend_bare_sparse<double>({1});
    GreenFunction G(16, H, -2.1, 2.1);
    const double kq = 2 * pi * 5 / L, lam = 2.0 * std::cos(kq) / 2.1;
    MatrixXcd psi(L, 1);
    for (int i = 0; i < L; ++i) psi(i, 0) = std::polar(1.0 / std::sqrt((double)L), kq * i);
    Cheb_first_kind_seq_view view(G.scaled_HE, psi);
    double err = 0.0;
    bool order = true;
    for (int k = 0; k < 6; ++k) {
      auto [i, blk] = view.next();
      order = order && i == k;
      const double t = std::cos(k * std::acos(lam));
      for (int r = 0; r < L; ++r) err = std::fmax(err, std::abs(blk(r, 0) - t * psi(r, 0)));
    }
    expect(order && err <= 1e-13, "Cheb_first_kind_seq_view on a plane wave", err);
  }
  std::printf("%s\n", failures ? "FAILED" : "ALL PASSED");
  return failures ? 1 : 0;
}
