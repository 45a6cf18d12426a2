"""Chebyshev expansions applied to vectors (tbk_cheb_expand) against the
oracle's Cheb_first_kind_seq_view walk (TB/numerical.h:346-361), the
time-evolution operator against dense exp(-i H t), and the single-energy
delta projection of conductivity_test_sawtooth (TB/snippets.h:173-223)."""
import numpy as np
import pytest
import scipy.sparse as sp

import oracle as orc
from helpers import landau_gauge

pytestmark = pytest.mark.gpu
TOL = {"fp64": 1e-12, "dd": 1e-12, "mixed": 2e-5}


def _honeycomb(tb, span=(10, 9)):
    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, -2.7), span)
    G, c = landau_gauge(0.04)
    X.set_gauge_linear(G, c)
    X.set_scalar_disorder(0.8, 2)
    H = X.get_Hamiltonian_sparse(complex)
    return tb.GreenFunction(32, H, -8.6, 8.6)


def _scipy(M):
    cp, ri, v = M.to_csc()
    n = len(cp) - 1
    return sp.csc_matrix((v, ri, cp), shape=(n, n))


@pytest.mark.parametrize("precision", ["fp64", "dd", "mixed"])
@pytest.mark.parametrize("R", [1, 3, 20])
def test_cheb_expand_matches_oracle(gpu, precision, R):
    tb = gpu
    G = _honeycomb(tb)
    Ht = G.scaled_HE
    n = Ht.shape[0]
    rng = np.random.default_rng(R)
    coef = rng.standard_normal(41) + 1j * rng.standard_normal(41)
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, R, 5)
    got = tb.cheb_expand(Ht, coef, kets, precision)
    cp, ri, v = Ht.to_csc()
    ref = orc.cheb_expand(n, cp, ri, v, coef, kets)
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    assert err <= TOL[precision], err


def test_cheb_expand_edge_term_counts(gpu):
    tb = gpu
    G = _honeycomb(tb, (5, 4))
    Ht = G.scaled_HE
    n = Ht.shape[0]
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, 2, 1)
    assert np.array_equal(tb.cheb_expand(Ht, [1.0], kets, "fp64"), kets)  # T_0 only
    # double-float vectors carry 48 significant bits
    assert np.max(np.abs(tb.cheb_expand(Ht, [1.0], kets) - kets)) <= 1e-15
    Hs = _scipy(Ht)
    assert np.allclose(tb.sparse_apply(Ht, kets), Hs @ kets, rtol=0, atol=1e-14)
    assert np.allclose(tb.cheb_expand(Ht, [0.0, 0.0, 1.0], kets), 2 * (Hs @ (Hs @ kets)) - kets, rtol=0, atol=1e-13)


def test_time_evolution_matches_dense(gpu):
    tb = gpu
    G = _honeycomb(tb, (7, 6))
    HE = _scipy(G.scaled_HE).toarray() * G.a + G.b * np.eye(G.scaled_HE.shape[0])
    w, U = np.linalg.eigh(HE)
    kets = tb.bases_of_uniform_ampl_with_random_phases(HE.shape[0], 3, 9)
    for t in (0.0, 0.7, 6.0):
        ref = U @ (np.exp(-1j * w * t)[:, None] * (U.conj().T @ kets))
        got = tb.time_evolve(G, t, kets)
        assert np.max(np.abs(got - ref)) <= 1e-11, t


def test_time_evolution_large_properties(gpu):
    """262,144-site square lattice with disorder: norm kept, and
    exp(-iH t1) exp(-iH t2) = exp(-iH (t1 + t2)) (size-independent checks)."""
    tb = gpu
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (512, 512))
    X.set_scalar_disorder(1.0, 4)
    G = tb.GreenFunction(16, X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float), -4.6, 4.6)
    kets = tb.bases_of_uniform_ampl_with_random_phases(512 * 512, 2, 3)
    a = tb.time_evolve(G, 3.0, tb.time_evolve(G, 2.0, kets))
    b = tb.time_evolve(G, 5.0, kets)
    assert np.max(np.abs(np.linalg.norm(b, axis=0) - 1.0)) <= 1e-12
    assert np.max(np.abs(a - b)) <= 1e-12


def test_conductivity_test_sawtooth_matches_oracle(gpu):
    tb = gpu
    X = tb.PartialLattice(tb.sawtooth_chain_p(0.25, 0.3535), (150,))
    N, E, R, seed = 64, -0.5, 4, 7
    got = tb.conductivity_test_sawtooth(X, N, E, R=R, seed=seed)
    # oracle restatement on the same (bit-exact) rescaled H and velocity
    t = -E / 2
    G = tb.GreenFunction(N, X.get_Hamiltonian_sparse(float), 4 * t - 2 - 1e-6, 4 * t + 1e-6)
    e = G.scale(E, 1.0)
    V = _scipy(tb.commutator(G.scaled_HE, X.op_position(0)))
    cp, ri, v = G.scaled_HE.to_csc()
    n = len(cp) - 1
    coef = orc.delta_coefficients(e, N)
    assert np.allclose(tb.delta_coefficients(e, N), coef, rtol=1e-14, atol=1e-14)
    kets = orc.random_phase_kets(n, R, seed)
    kR = orc.cheb_expand(n, cp, ri, v, coef, kets)
    kL = V @ orc.cheb_expand(n, cp, ri, v, coef, V @ kets)
    ref = np.sum(kL.real * kR.real + kL.imag * kR.imag) / R
    assert abs(got - ref) <= 1e-10 * max(1.0, abs(ref)), (got, ref)


@pytest.mark.parametrize("precision", ["fp64", "dd", "mixed"])
def test_cheb_first_kind_seq_view(gpu, precision):
    """Cheb_first_kind_seq_view (TB/numerical.h:346-361): next() yields
    (i, T_i(H~) v) in order, against the oracle's blocks; more vectors than one
    chunk; Cheb_first_kind_seq_on_bases collects the same blocks."""
    tb = gpu
    G = _honeycomb(tb, (7, 6))
    Ht = G.scaled_HE
    n = Ht.shape[0]
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, 40, 3)
    cp, ri, v = Ht.to_csc()
    ref = orc.cheb_blocks(n, cp, ri, v, 9, kets)                 # (K, R, n)
    view = tb.Cheb_first_kind_seq_view(Ht, kets, precision)
    tol = {"fp64": 1e-13, "dd": 1e-13, "mixed": 1e-5}[precision]
    for k in range(9):
        i, blk = view.next()
        assert i == k
        assert np.max(np.abs(blk - ref[k].T)) <= tol * max(1.0, np.max(np.abs(ref[k])))
    blocks = tb.Cheb_first_kind_seq_on_bases(Ht, 4, kets[:, 0], precision)
    for k in range(4):
        assert np.max(np.abs(blocks[k] - ref[k][0])) <= tol * max(1.0, np.max(np.abs(ref[k])))
