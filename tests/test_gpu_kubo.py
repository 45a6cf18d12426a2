"""Kubo path on the GPU vs the FP64 oracle on the same seeded vectors.

Stored Chebyshev blocks are complex64 on the GPU; stated bound for mu_nm:
max |mu_gpu - mu_oracle| <= MU_TOL * max |mu_oracle|.  The Gamma contractions and
the integration run in FP64 (1e-12 / exact on identical mu)."""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu
MU_TOL = 2e-5


def _system(tb, L=(12, 10), flux=1 / 64, cplx=True):
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), L)
    G = np.zeros((3, 3))
    G[1, 0] = 2 * np.pi * flux            # Landau gauge A = (0, B x, 0)
    X.set_gauge_linear(G, np.zeros(3))
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([0, 1], complex if cplx else float)
    return X, H


def _oracle_ops(tb, X, Ht):
    cp, ri, v = Ht.to_csc()
    n = len(cp) - 1
    xs = X.op_position(0).to_csc()[2]
    ys = X.op_position(1).to_csc()[2]
    vx = orc.commutator_values(n, cp, ri, v, xs)
    vy = orc.commutator_values(n, cp, ri, v, ys)
    return n, cp, ri, v, (cp, ri, vx), (cp, ri, vy)


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("tensor", [False, True])
@pytest.mark.parametrize("which", ["bastin", "greenwood"])
def test_mu_nm_vs_oracle(gpu, which, tensor):
    tb = gpu
    X, H = _system(tb)
    G = tb.GreenFunction(32, H, -4.1, 4.1)
    Ht = G.scaled_HE
    v_x = tb.commutator(Ht, X.op_position(0))
    v_y = tb.commutator(Ht, X.op_position(1))
    n, cp, ri, v, ovx, ovy = _oracle_ops(tb, X, Ht)
    kets = orc.random_phase_kets(n, 3, 2)
    g = orc.kernel_seq(orc.K_LORENTZ, 32, 6.0)
    if which == "bastin":
        mu = tb.kubo_mu(Ht, None, None, v_x, v_y, M=32, kets=kets, kernel=tb.Lorentz(6.0), tensor=tensor)
        ref = orc.kubo_mu(n, cp, ri, v, 32, kets, AR=ovx, BR=ovy, g=g)
    else:
        mu = tb.kubo_mu(Ht, v_x, v_x, None, None, M=32, kets=kets, kernel=tb.Lorentz(6.0), tensor=tensor)
        ref = orc.kubo_mu(n, cp, ri, v, 32, kets, AL=ovx, BL=ovx, g=g)
    assert _rel(mu, ref) <= MU_TOL, _rel(mu, ref)


def test_mu_chunking_and_seeded_kets(gpu):
    tb = gpu
    X, H = _system(tb, (8, 8))
    G = tb.GreenFunction(16, H, -4.1, 4.1)
    Ht = G.scaled_HE
    v_x = tb.commutator(Ht, X.op_position(0))
    n = Ht.shape[0]
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, 70, 4)
    one = tb.kubo_mu(Ht, None, None, v_x, v_x, M=16, kets=kets)
    # a tiny block budget forces chunks of fewer vectors
    tiny = 2.5 * 16 * 64 * 8 * 8 / 1e9
    chunked = tb.kubo_mu(Ht, None, None, v_x, v_x, M=16, kets=kets, budget_gb=tiny)
    assert _rel(chunked, one) <= 1e-5
    # random kets generated on the device == host-generated kets of the same seed
    dev = tb.kubo_mu(Ht, None, None, v_x, v_x, M=16, R=70, seed=4)
    assert _rel(dev, one) <= 1e-5


def test_gamma_contractions_fp64(gpu):
    tb = gpu
    rng = np.random.default_rng(0)
    M = 48
    mu = rng.normal(size=(M, M)) + 1j * rng.normal(size=(M, M))
    eps = tb.chebyshev_nodes(64)
    z = tb.bastin_zeta(mu, eps, 2.5)
    zr = orc.bastin_zeta(mu, eps, 2.5)
    assert _rel(z, zr) <= 1e-11
    s = tb.greenwood_sigma(mu, eps, 3.0)
    sr = orc.greenwood_sigma(mu, eps, 3.0)
    assert _rel(s, sr) <= 1e-11
    E, re, im = tb.bastin_integrate(eps, z)
    Eo, reo, imo = orc.bastin_integrate(eps, z)
    assert np.array_equal(E, Eo) and np.allclose(re, reo, rtol=1e-14, atol=0) and np.allclose(im, imo, rtol=1e-14, atol=0)


@pytest.mark.parametrize("tensor", [False, True])
def test_bastin_sigma_xy_end_to_end(gpu, tensor):
    """conductivity_Kubo_Bastin (TB/snippets.h:306-456) vs the oracle pipeline;
    stated bound: sigma_xy within 1e-5 of max |sigma| of the FP64 oracle."""
    tb = gpu
    X, H = _system(tb, (16, 16), flux=1 / 16)
    N, R = 64, 4
    out = tb.conductivity_Kubo_Bastin(H, X.op_position(0), X.op_position(1), N, -4.0, 4.0, R=R, seed=2,
                                      tensor=tensor)
    Ht = out["G"].scaled_HE
    n, cp, ri, v, ovx, ovy = _oracle_ops(tb, X, Ht)
    kets = orc.random_phase_kets(n, R, 2)
    g = orc.kernel_seq(orc.K_LORENTZ, N, 6.0)
    mu = orc.kubo_mu(n, cp, ri, v, N, kets, AR=ovx, BR=ovy, g=g)
    eps = tb.chebyshev_nodes(N)
    zeta = orc.bastin_zeta(mu, eps, 1.0)
    E, sr, si = orc.bastin_integrate(eps, zeta)
    assert np.array_equal(out["E"], E)
    assert _rel(out["sigma_re"], sr) <= 1e-5, _rel(out["sigma_re"], sr)


def test_greenwood_spectrum_and_v_moments(gpu):
    tb = gpu
    X, H = _system(tb, (10, 10), cplx=True)
    eps, sigma, mu = tb.conductivity_spectrum(H, X.op_position(0), X.op_position(1), 32, R=8, seed=1)
    assert sigma.shape == (32,) and np.all(np.isfinite(sigma))
    Xc = tb.PartialLattice(tb.Chain().add_hopping("A", 1, 1.0), (40,))
    V = tb.generate_V_moments(Xc, 12, R=6, seed=0)
    assert V.shape == (12, 12) and np.all(np.tril(V, -1) == 0)
    # oracle: bare H, G(12, H, -1.000001, 1.000001), v_x = op_velocity(0)
    H0 = Xc.get_Hamiltonian_bare_sparse(float)
    G = tb.GreenFunction(12, H0, -1.000001, 1.000001)
    cp, ri, v = G.scaled_HE.to_csc()
    vel = Xc.op_velocity(0).to_csc()
    kets = orc.random_phase_kets(40, 6, 0)
    ref = np.triu(np.real(orc.kubo_mu(40, cp, ri, v, 12, kets, AL=vel, BL=vel)) / 6)
    assert _rel(V, ref) <= MU_TOL


@pytest.mark.parametrize("which", ["bastin", "greenwood"])
def test_mu_nm_dd_recursion(gpu, which):
    """double-float recursion for the stored blocks: the complex128 bound."""
    tb = gpu
    X, H = _system(tb)
    G = tb.GreenFunction(32, H, -4.1, 4.1)
    Ht = G.scaled_HE
    v_x = tb.commutator(Ht, X.op_position(0))
    v_y = tb.commutator(Ht, X.op_position(1))
    n, cp, ri, v, ovx, ovy = _oracle_ops(tb, X, Ht)
    kets = orc.random_phase_kets(n, 3, 2)
    g = orc.kernel_seq(orc.K_LORENTZ, 32, 6.0)
    if which == "bastin":
        mu = tb.kubo_mu(Ht, None, None, v_x, v_y, M=32, kets=kets, kernel=tb.Lorentz(6.0), tensor=True, recursion="dd")
        mu64 = tb.kubo_mu(Ht, None, None, v_x, v_y, M=32, kets=kets, kernel=tb.Lorentz(6.0), tensor=True, recursion="fp64")
        ref = orc.kubo_mu(n, cp, ri, v, 32, kets, AR=ovx, BR=ovy, g=g)
    else:
        mu = tb.kubo_mu(Ht, v_x, v_x, None, None, M=32, kets=kets, kernel=tb.Lorentz(6.0), tensor=True, recursion="dd")
        mu64 = tb.kubo_mu(Ht, v_x, v_x, None, None, M=32, kets=kets, kernel=tb.Lorentz(6.0), tensor=True, recursion="fp64")
        ref = orc.kubo_mu(n, cp, ri, v, 32, kets, AL=ovx, BL=ovx, g=g)
    assert _rel(mu, ref) <= MU_TOL, _rel(mu, ref)
    # the blocks are rounded to complex64 either way: dd and FP64 recursions agree to that rounding
    assert _rel(mu, mu64) <= 1e-6, _rel(mu, mu64)


@pytest.mark.parametrize("which", ["bastin", "greenwood"])
def test_mu_nm_mixed_recursion(gpu, which):
    """complex64 recursion (FP32 H~) for the stored blocks: same bound as the
    complex128 recursion on M = 32."""
    tb = gpu
    X, H = _system(tb)
    G = tb.GreenFunction(32, H, -4.1, 4.1)
    Ht = G.scaled_HE
    v_x = tb.commutator(Ht, X.op_position(0))
    v_y = tb.commutator(Ht, X.op_position(1))
    n, cp, ri, v, ovx, ovy = _oracle_ops(tb, X, Ht)
    kets = orc.random_phase_kets(n, 3, 2)
    g = orc.kernel_seq(orc.K_LORENTZ, 32, 6.0)
    if which == "bastin":
        mu = tb.kubo_mu(Ht, None, None, v_x, v_y, M=32, kets=kets, kernel=tb.Lorentz(6.0), tensor=True,
                        recursion="mixed")
        ref = orc.kubo_mu(n, cp, ri, v, 32, kets, AR=ovx, BR=ovy, g=g)
    else:
        mu = tb.kubo_mu(Ht, v_x, v_x, None, None, M=32, kets=kets, kernel=tb.Lorentz(6.0), tensor=True,
                        recursion="mixed")
        ref = orc.kubo_mu(n, cp, ri, v, 32, kets, AL=ovx, BL=ovx, g=g)
    assert _rel(mu, ref) <= MU_TOL, _rel(mu, ref)


def test_bastin_sigma_xy_mixed_recursion(gpu):
    """sigma_xy with the complex64 recursion: stated bound 1e-5 of max |sigma| of
    the FP64 oracle pipeline (as the complex128 recursion), M = 64."""
    tb = gpu
    X, H = _system(tb, (16, 16), flux=1 / 16)
    N, R = 64, 4
    out = tb.conductivity_Kubo_Bastin(H, X.op_position(0), X.op_position(1), N, -4.0, 4.0, R=R, seed=2,
                                      tensor=True, recursion="mixed")
    Ht = out["G"].scaled_HE
    n, cp, ri, v, ovx, ovy = _oracle_ops(tb, X, Ht)
    kets = orc.random_phase_kets(n, R, 2)
    g = orc.kernel_seq(orc.K_LORENTZ, N, 6.0)
    mu = orc.kubo_mu(n, cp, ri, v, N, kets, AR=ovx, BR=ovy, g=g)
    eps = tb.chebyshev_nodes(N)
    E, sr, si = orc.bastin_integrate(eps, orc.bastin_zeta(mu, eps, 1.0))
    assert _rel(out["sigma_re"], sr) <= 1e-5, _rel(out["sigma_re"], sr)


@pytest.mark.parametrize("recursion", ["dd", "fp64", "mixed"])
@pytest.mark.parametrize("which", ["bastin", "greenwood"])
def test_fused_operator_products_same_bits(gpu, which, recursion):
    """The output operator (a commutator, H~'s sparsity) applied inside the
    recursion step, and both sides run as one recursion of twice the width,
    store the same complex64 bits as separate passes."""
    tb = gpu
    X, H = _system(tb, L=(20, 16))
    G = tb.GreenFunction(48, H, -4.1, 4.1)
    Ht = G.scaled_HE
    v_x = tb.commutator(Ht, X.op_position(0))
    v_y = tb.commutator(Ht, X.op_position(1))
    kw = dict(M=48, R=4, seed=3, kernel=tb.Lorentz(6.0), tensor=True, recursion=recursion)
    if which == "bastin":
        a = tb.kubo_mu(Ht, None, None, v_x, v_y, fuse_ops=True, **kw)
        b = tb.kubo_mu(Ht, None, None, v_x, v_y, **kw)
        c = tb.kubo_mu(Ht, None, None, v_x, v_y, fuse_ops=True, both_sides=True, **kw)
    else:
        a = tb.kubo_mu(Ht, v_x, v_x, None, None, fuse_ops=True, **kw)
        b = tb.kubo_mu(Ht, v_x, v_x, None, None, **kw)
        c = tb.kubo_mu(Ht, v_x, v_x, None, None, fuse_ops=True, both_sides=True, **kw)
    assert np.array_equal(a, b)      # fused products vs separate passes
    assert np.array_equal(a, c)      # vs both sides as one recursion


def test_greenwood_mu_fcc_wide_rows(gpu):
    """FCC (12 neighbours: pipelined gathers) Kubo-Greenwood mu_nm against the
    oracle, and the fused / two-sided variants against the plain one."""
    tb = gpu
    X = tb.PartialLattice(tb.FCC().add_hopping("A", 1, 1.0), (8, 7, 6))
    X.set_scalar_disorder(2.0, 4)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1, 1], complex)
    G = tb.GreenFunction(40, H, -13.0, 13.0)
    Ht = G.scaled_HE
    v_x = tb.commutator(Ht, X.op_position(0))
    cp, ri, v = Ht.to_csc()
    n = len(cp) - 1
    xs = X.op_position(0).to_csc()[2]
    ovx = (cp, ri, orc.commutator_values(n, cp, ri, v, xs))
    kets = orc.random_phase_kets(n, 4, 6)
    g = orc.kernel_seq(orc.K_LORENTZ, 40, 6.0)
    kw = dict(M=40, kets=kets, kernel=tb.Lorentz(6.0), tensor=True)
    mu = tb.kubo_mu(Ht, v_x, v_x, None, None, **kw)
    ref = orc.kubo_mu(n, cp, ri, v, 40, kets, AL=ovx, BL=ovx, g=g)
    assert _rel(mu, ref) <= MU_TOL, _rel(mu, ref)
    assert np.array_equal(mu, tb.kubo_mu(Ht, v_x, v_x, None, None, fuse_ops=True, **kw))
    assert np.array_equal(mu, tb.kubo_mu(Ht, v_x, v_x, None, None, fuse_ops=True, both_sides=True, **kw))


def test_repeated_calls_reuse_pool_and_release(gpu):
    """Stores of at most 16 GB come from a pool kept between calls: repeated
    calls give the same bits, and so does a call after tbk_kubo_release."""
    tb = gpu
    X, H = _system(tb, L=(20, 18))
    Ht = tb.GreenFunction(48, H, -4.1, 4.1).scaled_HE
    v_x = tb.commutator(Ht, X.op_position(0))
    v_y = tb.commutator(Ht, X.op_position(1))
    kw = dict(M=48, R=5, seed=3, kernel=tb.Lorentz(6.0), tensor=True)
    a = tb.kubo_mu(Ht, None, None, v_x, v_y, **kw)
    b = tb.kubo_mu(Ht, None, None, v_x, v_y, **kw)
    assert np.array_equal(a, b)
    tb.kubo_release()
    tb.kubo_release()                                   # twice: nothing left to return
    assert np.array_equal(tb.kubo_mu(Ht, None, None, v_x, v_y, **kw), a)
