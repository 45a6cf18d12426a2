"""Row classes (computed neighbours) against the ELL form of the same matrix.

A translation-invariant matrix gets the class form: each row's neighbours are
row + offset from a small per-class table.  The class form must give the same
bits as the ELL form (same entries, same order, same arithmetic) in every
precision and recursion mode, apply where rows repeat (periodic and open
lattices, constant complex hoppings, a small Landau-gauge lattice whose phases
repeat per column) and fall back to the ELL where they do not (an unstructured
matrix, a gauge with more than 255 distinct rows).  TBK_NO_CLASSES=1, read when a matrix
is first examined, forces the ELL form for the comparison.
"""
import os

import numpy as np
import pytest

import oracle as orc
from helpers import landau_gauge

pytestmark = pytest.mark.gpu


def _rescaled(tb, X, extend, cplx, a):
    if extend is None:
        H = X.get_Hamiltonian_sparse(complex if cplx else float)
    else:
        H = X.get_Hamiltonian_periodic_extend_bare_sparse(extend, complex if cplx else float)
    return tb.GreenFunction(8, H, -a, a).scaled_HE


def _both_forms(tb, build):
    """build() twice: once examined with the class form allowed, once with the
    ELL form forced; returns (matrix with classes, matrix without)."""
    A = build()
    nA = A.row_classes()
    os.environ["TBK_NO_CLASSES"] = "1"
    try:
        B = build()
        assert B.row_classes() == 0
    finally:
        del os.environ["TBK_NO_CLASSES"]
    return A, B, nA


def _honeycomb(tb, L=64):
    def build():
        X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, -2.7), (L, L))
        X.set_scalar_disorder(1.0, 1)
        return _rescaled(tb, X, [1, 1], False, 8.7)
    return build


@pytest.mark.parametrize("prec", ["mixed", "fp64", "dd"])
@pytest.mark.parametrize("doubling", [True, False])
def test_classes_bit_identical_honeycomb(gpu, prec, doubling):
    tb = gpu
    A, B, n_cls = _both_forms(tb, _honeycomb(tb))
    assert 1 <= n_cls <= 18          # two atoms x (interior, two wrapped edges) per axis
    R = 32 if prec == "mixed" else 16
    mu_a = tb.KpmSolver(A, R, precision=prec, doubling=doubling).run_random(96, 3)
    mu_b = tb.KpmSolver(B, R, precision=prec, doubling=doubling).run_random(96, 3)
    assert np.array_equal(mu_a, mu_b)


@pytest.mark.parametrize("R", [1, 3, 8, 40])
def test_classes_fcc_complex_braket_and_oracle(gpu, R):
    """FCC, 12 neighbours, constant complex hopping (complex class table),
    braket mode with different bras; also against the CPU oracle."""
    tb = gpu

    def build():
        X = tb.PartialLattice(tb.FCC().add_hopping("A", 1, complex(0.8, 0.6)), (12, 12, 12))
        X.set_scalar_disorder(2.0, 4)
        return _rescaled(tb, X, [1, 1, 1], True, 13.0)

    A, B, n_cls = _both_forms(tb, build)
    assert 1 <= n_cls <= 27
    n = A.shape[0]
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, R, 5)
    bras = tb.bases_of_uniform_ampl_with_random_phases(n, R, 6)
    for prec in ("fp64", "dd", "mixed"):
        mu_a = tb.KpmSolver(A, R, precision=prec, doubling=False).run(64, bras, kets)
        mu_b = tb.KpmSolver(B, R, precision=prec, doubling=False).run(64, bras, kets)
        assert np.array_equal(mu_a, mu_b), prec
    cp, ri, v = A.to_csc()
    ref = orc.cheb_moments(n, cp, ri, v, 64, bras, kets)
    mu = tb.KpmSolver(A, R, precision="fp64", doubling=False).run(64, bras, kets)
    assert np.max(np.abs(mu - ref)) <= 1e-10 * max(abs(ref[0]), 1.0)
    # the drop-in from host CSC arrays detects the classes of the same matrix
    mu_d = tb.Cheb_first_kind_seq_braket((n, cp, ri, v), 64, bras, kets, precision="fp64")
    assert np.array_equal(mu_d, mu)


def test_classes_open_boundary_and_landau(gpu):
    tb = gpu

    def open_square():
        X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (20, 24))
        return _rescaled(tb, X, None, False, 4.5)

    A, B, n_cls = _both_forms(tb, open_square)
    assert 1 <= n_cls <= 9
    mu_a = tb.KpmSolver(A, 8, precision="mixed", doubling=True).run_random(128, 1)
    mu_b = tb.KpmSolver(B, 8, precision="mixed", doubling=True).run_random(128, 1)
    assert np.array_equal(mu_a, mu_b)

    def landau():
        X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (16, 16))
        X.set_gauge_linear(*landau_gauge(2 * np.pi / 16))
        return _rescaled(tb, X, [0, 1], True, 4.5)

    A, B, n_cls = _both_forms(tb, landau)
    assert 1 <= n_cls <= 255          # the phases repeat along y: one class per column at most (x 3 edges)
    for prec in ("fp64", "dd", "mixed"):
        mu_a = tb.KpmSolver(A, 8, precision=prec, doubling=True).run_random(64, 2)
        mu_b = tb.KpmSolver(B, 8, precision=prec, doubling=True).run_random(64, 2)
        assert np.array_equal(mu_a, mu_b), prec


def test_classes_not_applicable(gpu):
    tb = gpu
    import scipy.sparse as sp

    rng = np.random.default_rng(4)
    A = sp.random(3000, 3000, density=0.003, random_state=5)
    A = A + A.T + sp.diags(rng.standard_normal(3000))
    M = tb.SparseMatrix.from_scipy(A)
    assert M.row_classes() == 0                                                  # every row its own
    mu = tb.KpmSolver(M, 4, precision="fp64", doubling=False).run_random(16, 1)
    assert np.all(np.isfinite(mu))
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (300, 4))
    X.set_gauge_linear(*landau_gauge(2 * np.pi / 1024))
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([0, 1], complex)
    assert tb.GreenFunction(8, H, -4.5, 4.5).scaled_HE.row_classes() == 0      # 300 distinct phase columns


def test_classes_expansion_and_kubo_blocks(gpu):
    """The other users of the step kernel: Clenshaw expansions and the Kubo
    block recursion (K-tiled stores) give the same bits in both forms."""
    tb = gpu

    def build():
        X = tb.PartialLattice(tb.FCC().add_hopping("A", 1, 1.0), (10, 10, 10))
        X.set_scalar_disorder(2.0, 4)
        return _rescaled(tb, X, [1, 1, 1], True, 13.0)

    A, B, n_cls = _both_forms(tb, build)
    assert n_cls >= 1
    n = A.shape[0]
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, 5, 7)
    coef = np.random.default_rng(1).standard_normal(40)
    for prec in ("dd", "mixed"):
        assert np.array_equal(tb.cheb_expand(A, coef, kets, prec), tb.cheb_expand(B, coef, kets, prec)), prec
    mu_a = tb.kubo_mu(A, M=32, R=4, seed=3, tensor=False, recursion="dd")
    mu_b = tb.kubo_mu(B, M=32, R=4, seed=3, tensor=False, recursion="dd")
    assert np.array_equal(mu_a, mu_b)
