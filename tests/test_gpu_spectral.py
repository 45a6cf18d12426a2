"""Device Lanczos spectral range (tbk_spectral_range) against dense
eigenvalues of the same CSC matrix (numpy eigvalsh), and the bound-free
GreenFunction constructors built on it (TB/lattice.h:560-576,
TB/numerical.h:24-46)."""
import numpy as np
import pytest

from helpers import landau_gauge

pytestmark = pytest.mark.gpu


def _dense(H):
    cp, ri, v = H.to_csc()
    n = len(cp) - 1
    D = np.zeros((n, n), dtype=np.complex128)
    for j in range(n):
        D[ri[cp[j]:cp[j + 1]], j] = v[cp[j]:cp[j + 1]]
    return D


def _cases(tb):
    sq = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (14, 11))
    sq.set_scalar_disorder(2.0, 3)
    hc = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, -2.7), (9, 8))
    G, c = landau_gauge(0.05)
    hc.set_gauge_linear(G, c)
    hc.set_scalar_disorder(0.5, 7)
    chain = tb.PartialLattice(tb.Chain().add_hopping("A", 1, 1.0), (4,))
    return [("square_disorder_real", sq.get_Hamiltonian_sparse(float)),
            ("honeycomb_gauge_complex", hc.get_Hamiltonian_sparse(complex)),
            ("chain4_breakdown", chain.get_Hamiltonian_sparse(float))]


def test_spectral_range_matches_dense(gpu):
    tb = gpu
    for name, H in _cases(tb):
        w = np.linalg.eigvalsh(_dense(H))
        e0, e1, r0, r1 = tb.spectral_range(H, iters=300, seed=11)
        scale = max(1.0, abs(w[0]), abs(w[-1]))
        assert abs(e0 - w[0]) <= 1e-8 * scale, (name, e0, w[0])
        assert abs(e1 - w[-1]) <= 1e-8 * scale, (name, e1, w[-1])
        assert r0 >= 0 and r1 >= 0


def test_ritz_values_inside_spectrum_and_residual_bound(gpu):
    tb = gpu
    _, H = _cases(tb)[1]
    w = np.linalg.eigvalsh(_dense(H))
    for iters in (4, 10, 30):
        e0, e1, r0, r1 = tb.spectral_range(H, iters=iters, seed=2)
        assert w[0] - 1e-10 <= e0 and e1 <= w[-1] + 1e-10
        # an eigenvalue lies within the residual norm of each Ritz value
        assert np.min(np.abs(w - e0)) <= r0 * (1 + 1e-9) + 1e-10
        assert np.min(np.abs(w - e1)) <= r1 * (1 + 1e-9) + 1e-10


def test_green_function_bound_free_constructors(gpu):
    tb = gpu
    _, H = _cases(tb)[0]
    w = np.linalg.eigvalsh(_dense(H))
    G = tb.GreenFunction(32, H)
    assert abs(G.E_min - w[0]) <= 1e-8 and abs(G.E_max - w[-1]) <= 1e-8
    assert abs(G.a - (w[-1] - w[0]) / (2 - 0.01)) <= 1e-8
    assert abs(G.b - (w[-1] + w[0]) / 2) <= 1e-8
    G2 = tb.GreenFunction(32, H, H, 0.1)          # (N, HE, ref_HE, epsilon)
    assert abs(G2.a - (w[-1] - w[0]) / 1.9) <= 1e-8
    # the rescaled spectrum sits inside [-1 + eps/2, 1 - eps/2] (to Lanczos accuracy)
    ws = np.linalg.eigvalsh(_dense(G.scaled_HE))
    assert ws[0] >= -1 + 0.005 - 1e-8 and ws[-1] <= 1 - 0.005 + 1e-8


def test_spectral_range_large_lattice_moments_bounded(gpu):
    """2M-site honeycomb with disorder: Lanczos range brackets the Gershgorin
    interval from inside, and the DoS moments with G(N, H) stay bounded."""
    tb = gpu
    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, -2.7), (1024, 1024))
    X.set_scalar_disorder(1.0, 9)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    e0, e1, r0, r1 = tb.spectral_range(H, iters=200, seed=1)
    gersh = 3 * 2.7 + 0.5
    assert -gersh <= e0 < -7.5 and 7.5 < e1 <= gersh
    G = tb.GreenFunction(256, H)
    mu = tb.KpmSolver(G.scaled_HE, 4, precision="fp64", doubling=True).run_random(256, seed=3)
    assert np.all(np.isfinite(mu)) and np.max(np.abs(mu)) <= abs(mu[0]) * (1 + 1e-9)


def test_spectral_range_against_sparse_eigensolver(gpu):
    """40,000-site disordered square lattice (past the reference's 5,000-row
    Spectra cap): Lanczos extremes against ARPACK (scipy eigsh) on the same
    CSC, and Ritz values inside the spectrum."""
    tb = gpu
    sla = pytest.importorskip("scipy.sparse.linalg")
    sp = pytest.importorskip("scipy.sparse")
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (200, 200))
    X.set_scalar_disorder(1.5, 8)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    cp, ri, v = H.to_csc()
    n = len(cp) - 1
    A = sp.csc_matrix((v.real if np.iscomplexobj(v) else v, ri, cp), shape=(n, n))
    lo = sla.eigsh(A, k=1, which="SA", tol=1e-12, return_eigenvectors=False)[0]
    hi = sla.eigsh(A, k=1, which="LA", tol=1e-12, return_eigenvectors=False)[0]
    e0, e1, r0, r1 = tb.spectral_range(H, iters=600, seed=4)
    assert lo - 1e-9 <= e0 <= lo + 1e-5 and hi - 1e-5 <= e1 <= hi + 1e-9, (e0, lo, e1, hi)
