"""Kubo conductivities at configuration scale against the FP64 reference form.

The FP64 reference form (kubo_mu(..., recursion="fp64", fp64_blocks=True)):
complex128 recursion, complex128 stored Chebyshev blocks and an FP64 CUDA-core
GEMM for mu_nm — FP64 from end to end.  It is pinned here to the CPU oracle
at 1e-10 on a small lattice, then used as the reference for the product path
(complex64 or double-float recursion, complex64 stored blocks, tcgen05
split-TF32 GEMM); the complex64 storage bounds both recursions alike:

  sigma_xy, square 256 x 256 open-x / periodic-y, Landau flux 1/64, M = 512,
  R = 16 (seed 2), 512 Fermi energies:
      max |sigma_xy - sigma_xy(FP64)| / max |sigma_xy(FP64)|       <= 1e-5
      (measured 1.9e-6 with either recursion)
  sigma_xx, FCC 64^3 periodic, disorder U[-1, 1] (seed 4), M = 1024, R = 8,
  1,024 energies (the Greenwood configuration at 1/8 of its sites, which the
  FP64 GEMM finishes in seconds):
      max over |eps| <= 0.9 of |d sigma_xx| / max |sigma_xx(FP64)|  <= 1e-5
      (measured 3.7e-7 double-float, 3.8e-7 complex64)
      max over all 1,024 energies                                   <= 5e-3
      (measured 2.1e-3 / 2.0e-3, at the two outermost Chebyshev nodes, where the
      Greenwood sum divides by 1 - eps^2 = 2.4e-6 and the band-edge sigma_xx
      is a cancellation of large terms)
"""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu
XX_TOL_WINDOW = 1e-5
XX_TOL_ALL = 5e-3


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("which", ["bastin", "greenwood"])
def test_fp64_form_vs_oracle(gpu, which):
    tb = gpu
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (12, 10))
    G0 = np.zeros((3, 3))
    G0[1, 0] = 2 * np.pi / 64
    X.set_gauge_linear(G0, np.zeros(3))
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([0, 1], complex)
    G = tb.GreenFunction(40, H, -4.1, 4.1)
    Ht = G.scaled_HE
    v_x = tb.commutator(Ht, X.op_position(0))
    v_y = tb.commutator(Ht, X.op_position(1))
    cp, ri, v = Ht.to_csc()
    n = len(cp) - 1
    ovx = (cp, ri, orc.commutator_values(n, cp, ri, v, X.op_position(0).to_csc()[2]))
    ovy = (cp, ri, orc.commutator_values(n, cp, ri, v, X.op_position(1).to_csc()[2]))
    kets = orc.random_phase_kets(n, 5, 2)
    g = orc.kernel_seq(orc.K_LORENTZ, 40, 6.0)
    kw = dict(M=40, kets=kets, kernel=tb.Lorentz(6.0), recursion="fp64", fp64_blocks=True)
    if which == "bastin":
        ops = (None, None, v_x, v_y)
        ref = orc.kubo_mu(n, cp, ri, v, 40, kets, AR=ovx, BR=ovy, g=g)
    else:
        ops = (v_x, v_x, None, None)
        ref = orc.kubo_mu(n, cp, ri, v, 40, kets, AL=ovx, BL=ovx, g=g)
    mu = tb.kubo_mu(Ht, *ops, **kw)
    assert _rel(mu, ref) <= 1e-10, _rel(mu, ref)
    # one vector per chunk (a block budget of 1.5 complex128 block pairs of 128 padded rows): same result
    one = 1.5 * 2 * 40 * 128 * 16 / 1e9
    assert _rel(tb.kubo_mu(Ht, *ops, budget_gb=one, **kw), ref) <= 1e-10


@pytest.mark.parametrize("recursion", ["mixed", "dd"])
def test_bastin_sigma_xy_config3_full(gpu, recursion):
    tb = gpu
    L, M, R = 256, 512, 16
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (L, L))
    G0 = np.zeros((3, 3))
    G0[1, 0] = 2 * np.pi / 64
    X.set_gauge_linear(G0, np.zeros(3))
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([0, 1], complex)
    args = (H, X.op_position(0), X.op_position(1), M, -4.0, 4.0)
    prod = tb.conductivity_Kubo_Bastin(*args, R=R, seed=2, tensor=True, recursion=recursion)
    ref = tb.conductivity_Kubo_Bastin(*args, R=R, seed=2, recursion="fp64", fp64_blocks=True)
    assert np.array_equal(prod["E"], ref["E"]) and len(ref["E"]) > 0
    err = _rel(prod["sigma_re"], ref["sigma_re"])
    print("sigma_xy config 3 (%s): max |d sigma| / max |sigma| = %.3e; mu: %.3e"
          % (recursion, err, _rel(prod["mu"], ref["mu"])))
    assert err <= 1e-5


@pytest.mark.parametrize("recursion", ["mixed", "dd"])
def test_greenwood_sigma_xx_fcc64(gpu, recursion):
    tb = gpu
    L, M, R = 64, 1024, 8
    X = tb.PartialLattice(tb.FCC().add_hopping("A", 1, 1.0), (L, L, L))
    X.set_scalar_disorder(2.0, 4)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1, 1], complex)
    args = (H, X.op_position(0), X.op_position(1), M)
    eps, s_prod, mu_p = tb.conductivity_spectrum(*args, R=R, seed=4, E_min=-13.0, E_max=13.0, tensor=True,
                                                 recursion=recursion)
    eps2, s_ref, mu_r = tb.conductivity_spectrum(*args, R=R, seed=4, E_min=-13.0, E_max=13.0, recursion="fp64",
                                                 fp64_blocks=True)
    assert np.array_equal(eps, eps2)
    d = np.abs(s_prod - s_ref) / np.max(np.abs(s_ref))
    win = np.abs(eps) <= 0.9
    print("sigma_xx FCC 64^3 (%s): window %.3e, all %.3e, mu %.3e" % (recursion, d[win].max(), d.max(),
                                                                        _rel(mu_p, mu_r)))
    assert d[win].max() <= XX_TOL_WINDOW
    assert d.max() <= XX_TOL_ALL
