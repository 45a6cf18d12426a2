"""Chebyshev moments on the GPU vs the FP64 oracle on the same seeded inputs.

Tolerances (stated, relative to mu_0 = Re tr(bras^dagger kets)):
  FP64 drop-in (complex128 recursion)           <= 1e-10
  FP64 with moment doubling                     <= 1e-10
  mixed precision (complex64 recursion, FP64
  moment sums), M <= 256                        <= MIXED_TOL
  double-float recursion (FP32 hi + lo pairs)   <= DD_TOL
"""
import numpy as np
import pytest

import oracle as orc
from helpers import landau_gauge, spec_from, with_onsite_zeros

pytestmark = pytest.mark.gpu
MIXED_TOL = 2e-5
DD_TOL = 1e-10


def _system(tb, kind="square", L=(16, 16), cplx=False, disorder=None, gauge=None):
    if kind == "square":
        cell = tb.Square().add_hopping("A", 1, 1.0)
    elif kind == "honeycomb":
        cell = tb.Honeycomb().add_hopping("A", 1, -2.7)
    else:
        cell = tb.FCC().add_hopping("A", 1, 1.0)
    X = tb.PartialLattice(cell, L)
    if disorder:
        X.set_scalar_disorder(*disorder)
    if gauge is not None:
        X.set_gauge_linear(*gauge)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1] * len(L), complex if cplx else float)
    return X, H


def _rescaled_csc(tb, H, a, b=0.0):
    G = tb.GreenFunction(8, H, b - a, b + a)
    cp, ri, v = G.scaled_HE.to_csc()
    return G, cp, ri, v


def _err(mu, ref):
    return float(np.max(np.abs(mu - ref)) / abs(ref[0]))


@pytest.mark.parametrize("cplx", [False, True])
def test_dropin_fp64_c1_config(gpu, cplx):
    tb = gpu
    # square 64x64 periodic, t = 1, bounds +-4.05, M = 256, R = 8, seed 0
    X, H = _system(tb, "square", (64, 64), cplx)
    G, cp, ri, v = _rescaled_csc(tb, H, 4.05)
    n = len(cp) - 1
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, 8, 0)
    mu = tb.Cheb_first_kind_seq_braket((n, cp, ri, v), 256, kets, kets, precision="fp64")
    ref = orc.cheb_moments(n, cp, ri, v, 256, kets, kets)
    assert _err(mu, ref) <= 1e-10
    assert abs(mu[0] - 8.0) < 1e-12


def test_dropin_fp64_bras_ne_kets_complex_gauge(gpu):
    tb = gpu
    X, H = _system(tb, "honeycomb", (10, 9), True, disorder=(1.0, 1), gauge=landau_gauge(2 * np.pi / 23))
    G, cp, ri, v = _rescaled_csc(tb, H, 9.0, 0.05)
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, 5, 3)
    bras = orc.random_phase_kets(n, 5, 4)
    mu = tb.Cheb_first_kind_seq_braket((n, cp, ri, v), 64, bras, kets, precision="fp64")
    ref = orc.cheb_moments(n, cp, ri, v, 64, bras, kets)
    assert np.max(np.abs(mu - ref)) <= 1e-10 * np.max(np.abs(ref))


@pytest.mark.parametrize("R", [1, 3, 8, 33, 40])
def test_fp64_r_chunking_and_padding(gpu, R):
    tb = gpu
    X, H = _system(tb, "square", (12, 10), False, disorder=(0.5, 2))
    G, cp, ri, v = _rescaled_csc(tb, H, 4.5)
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, R, 9)
    mu = tb.Cheb_first_kind_seq_braket((n, cp, ri, v), 33, kets, kets, precision="fp64")
    ref = orc.cheb_moments(n, cp, ri, v, 33, kets, kets)
    assert _err(mu, ref) <= 1e-10


@pytest.mark.parametrize("n_mom", [2, 3, 17, 64])
def test_fp64_doubling_matches_oracle(gpu, n_mom):
    tb = gpu
    X, H = _system(tb, "honeycomb", (8, 8), False, disorder=(1.0, 1))
    G, cp, ri, v = _rescaled_csc(tb, H, 8.5)
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, 4, 1)
    mu = tb.Cheb_first_kind_seq_braket((n, cp, ri, v), n_mom, kets, kets, precision="fp64", doubling=True)
    ref = orc.cheb_moments(n, cp, ri, v, n_mom, kets, kets)
    assert _err(mu, ref) <= 1e-10


@pytest.mark.parametrize("name,model,span,t", [("square_L16_t1", "Square", (16, 16), 1.0),
                                               ("honeycomb_L12_t-2.7", "Honeycomb", (12, 12), -2.7),
                                               ("fcc_L6_t1", "FCC", (6, 6, 6), 1.0)])
def test_fp64_exact_trace_golden(gpu, name, model, span, t):
    tb = gpu
    from pathlib import Path
    gold = np.load(Path(__file__).resolve().parent / "golden" / "exact_moments.npz")
    mu_exact, a = gold[name], float(gold[name + "__a"][0])
    X = tb.PartialLattice(getattr(tb, model)().add_hopping("A", 1, t), span)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1] * len(span), float)
    G = tb.GreenFunction(len(mu_exact), H, -a, a)
    n = H.shape[0]
    eye = np.asfortranarray(np.eye(n, dtype=np.complex128))
    solver = tb.KpmSolver(G.scaled_HE, n, precision="fp64", doubling=False)
    mu = solver.run(len(mu_exact), eye, eye)
    assert np.max(np.abs(mu - mu_exact)) / mu_exact[0] <= 1e-10


@pytest.mark.parametrize("cplx,R", [(False, 8), (True, 8), (False, 32), (False, 1), (False, 64)])
def test_mixed_precision_bound(gpu, cplx, R):
    tb = gpu
    X, H = _system(tb, "square", (64, 64), cplx, disorder=(0.5, 7))
    G, cp, ri, v = _rescaled_csc(tb, H, 4.5)
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, R, 0)
    ref = orc.cheb_moments(n, cp, ri, v, 256, kets, kets)
    for doubling in (False, True):
        mu = tb.Cheb_first_kind_seq_braket((n, cp, ri, v), 256, kets, kets, precision="mixed", doubling=doubling)
        assert _err(mu, ref) <= MIXED_TOL, (doubling, _err(mu, ref))


def test_resident_plan_is_deterministic_and_random_kets(gpu):
    tb = gpu
    X, H = _system(tb, "honeycomb", (32, 32), False, disorder=(1.0, 1))
    G, cp, ri, v = _rescaled_csc(tb, H, 8.5)
    n = len(cp) - 1
    s = tb.KpmSolver(G.scaled_HE, 16, precision="mixed", doubling=True)
    a = s.run_random(128, 5)
    b = s.run_random(128, 5)
    assert np.array_equal(a, b)
    kets = orc.random_phase_kets(n, 16, 5)        # same seeded kets, generated on the host
    ref = orc.cheb_moments(n, cp, ri, v, 128, kets, kets)
    assert _err(a, ref) <= MIXED_TOL
    f = tb.KpmSolver(G.scaled_HE, 16, precision="fp64", doubling=True)
    assert _err(f.run_random(128, 5), ref) <= 1e-10
    ms, launches, bytes_ = s.last_timing()
    assert launches == 65 and ms > 0 and bytes_ > 0
    from tight_binding_gb300 import capi
    m = tb.KpmSolver(G.scaled_HE, 16, precision="mixed", doubling=True, flags=capi.FLAG_PERSISTENT)
    assert _err(m.run_random(128, 5), ref) <= MIXED_TOL
    ms, launches, bytes_ = m.last_timing()
    assert launches == 1 and ms > 0 and bytes_ > 0        # 2,048 sites: one-launch recursion


def test_errors(gpu):
    tb = gpu
    X, H = _system(tb, "square", (4, 4), False)
    G, cp, ri, v = _rescaled_csc(tb, H, 4.5)
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, 2, 0)
    with pytest.raises(tb.TbkError):
        tb.Cheb_first_kind_seq_braket((n, cp, ri, v), 1, kets, kets)
    with pytest.raises(ValueError):
        tb.Cheb_first_kind_seq_braket((n, cp, ri, v), 8, orc.random_phase_kets(n, 2, 1), kets, doubling=True)
    with pytest.raises(tb.TbkError):
        tb.Cheb_first_kind_seq_braket((0, np.zeros(1, np.int32), np.zeros(0, np.int32), np.zeros(0)), 8,
                                      np.zeros((0, 1), complex), np.zeros((0, 1), complex))


def test_large_mixed_properties(gpu):
    """Benchmark-size system (honeycomb 1024^2, R = 32): size-independent checks."""
    tb = gpu
    X, H = _system(tb, "honeycomb", (1024, 1024), False, disorder=(1.0, 1))
    G = tb.GreenFunction(64, H, -8.6, 8.6)
    s = tb.KpmSolver(G.scaled_HE, 32, precision="mixed", doubling=True)
    f = tb.KpmSolver(G.scaled_HE, 32, precision="fp64", doubling=False)
    mu = s.run_random(64, 1)
    ref = f.run_random(64, 1)
    assert abs(ref[0] - 32.0) < 1e-9                      # normalised kets: mu_0 = R
    assert np.all(np.abs(mu) <= 32.0 * (1 + 1e-6))         # |T_n| <= 1 on the rescaled spectrum
    assert _err(mu, ref) <= MIXED_TOL


@pytest.mark.parametrize("cplx,R", [(False, 8), (True, 8), (False, 32), (False, 1), (True, 40)])
def test_dd_precision_bound(gpu, cplx, R):
    """double-float recursion: FP64-class moments (same systems as the mixed bound)."""
    tb = gpu
    X, H = _system(tb, "square", (64, 64), cplx, disorder=(0.5, 7))
    G, cp, ri, v = _rescaled_csc(tb, H, 4.5)
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, R, 0)
    ref = orc.cheb_moments(n, cp, ri, v, 256, kets, kets)
    for doubling in (False, True):
        mu = tb.Cheb_first_kind_seq_braket((n, cp, ri, v), 256, kets, kets, precision="dd", doubling=doubling)
        assert _err(mu, ref) <= DD_TOL, (doubling, _err(mu, ref))


def test_dd_exact_trace_golden(gpu):
    tb = gpu
    from pathlib import Path
    gold = np.load(Path(__file__).resolve().parent / "golden" / "exact_moments.npz")
    mu_exact, a = gold["honeycomb_L12_t-2.7"], float(gold["honeycomb_L12_t-2.7__a"][0])
    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, -2.7), (12, 12))
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    G = tb.GreenFunction(len(mu_exact), H, -a, a)
    n = H.shape[0]
    eye = np.asfortranarray(np.eye(n, dtype=np.complex128))
    mu = tb.KpmSolver(G.scaled_HE, n, precision="dd", doubling=False).run(len(mu_exact), eye, eye)
    assert np.max(np.abs(mu - mu_exact)) / mu_exact[0] <= DD_TOL


def test_two_step_passes_match_single_steps(gpu):
    """TBK_FLAG_TWO_STEP (two recursion steps per pass, temporal blocking): the
    vectors are the same bits as one step per pass (same per-row arithmetic);
    the moments differ only by the order of the FP32 per-thread sums."""
    tb = gpu
    X, H = _system(tb, "honeycomb", (256, 256), False, disorder=(1.0, 1))
    G, cp, ri, v = _rescaled_csc(tb, H, 8.7)
    Ht = G.scaled_HE
    two = tb.capi.FLAG_TWO_STEP
    for M in (128, 130, 3):
        fused = tb.KpmSolver(Ht, 32, precision="mixed", doubling=True, flags=two).run_random(M, 5)
        single = tb.KpmSolver(Ht, 32, precision="mixed", doubling=True).run_random(M, 5)
        assert _err(fused, single) <= 1e-6, (M, _err(fused, single))
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, 32, 5)
    ref = orc.cheb_moments(n, cp, ri, v, 130, kets, kets)
    mu = tb.KpmSolver(Ht, 32, precision="mixed", doubling=True, flags=two).run_random(130, 5)
    assert _err(mu, ref) <= MIXED_TOL, _err(mu, ref)


@pytest.mark.parametrize("precision,doubling", [("fp64", True), ("fp64", False), ("mixed", True), ("dd", True)])
def test_graph_replay_matches_direct_launches(gpu, precision, doubling):
    """Small single-chunk plans capture their recursion on the second identical
    run and replay it after: every run gives the bits of a plan that never
    captures, also when the moment count changes between runs."""
    tb = gpu
    from tight_binding_gb300 import capi

    _, H = _system(tb, "square", (64, 64), disorder=(1.0, 3))
    G, cp, ri, v = _rescaled_csc(tb, H, 4.6)
    kets = tb.bases_of_uniform_ampl_with_random_phases(64 * 64, 8, 0)
    bras = kets if doubling else tb.bases_of_uniform_ampl_with_random_phases(64 * 64, 8, 1)
    g = tb.KpmSolver(G.scaled_HE, 8, precision=precision, doubling=doubling)
    d = tb.KpmSolver(G.scaled_HE, 8, precision=precision, doubling=doubling, flags=capi.FLAG_NO_GRAPH)
    for M in (256, 256, 256, 256, 100, 100, 100, 256):
        a = g.run(M, bras, kets)
        b = d.run(M, bras, kets)
        assert np.array_equal(a, b), M
    ref = orc.cheb_moments(64 * 64, cp, ri, v, 256, bras, kets)
    tol = {"fp64": 1e-10, "dd": DD_TOL, "mixed": MIXED_TOL}[precision]
    assert np.max(np.abs(a - ref)) / abs(ref[0]) <= tol


@pytest.mark.parametrize("precision,doubling,cplx,R", [("fp64", True, False, 8), ("fp64", False, True, 3),
                                                       ("mixed", True, True, 8), ("mixed", False, False, 5),
                                                       ("dd", True, False, 4), ("dd", False, True, 2)])
def test_one_launch_recursion_matches_oracle(gpu, precision, doubling, cplx, R):
    """TBK_FLAG_PERSISTENT: the whole recursion in one launch (one CTA per
    complex64 vector where H~ has row classes, else one thread-block cluster
    per random vector): moments against the oracle and against the
    one-launch-per-step path."""
    tb = gpu
    from tight_binding_gb300 import capi

    gauge = landau_gauge(0.05) if cplx else None
    _, H = _system(tb, "honeycomb", (40, 36), cplx=cplx, disorder=(1.0, 5), gauge=gauge)
    G, cp, ri, v = _rescaled_csc(tb, H, 8.8)
    n = H.shape[0]
    kets = tb.bases_of_uniform_ampl_with_random_phases(n, R, 2)
    bras = kets if doubling else tb.bases_of_uniform_ampl_with_random_phases(n, R, 3)
    one = tb.KpmSolver(G.scaled_HE, R, precision=precision, doubling=doubling, flags=capi.FLAG_PERSISTENT)
    multi = tb.KpmSolver(G.scaled_HE, R, precision=precision, doubling=doubling)
    M = 300
    a = one.run(M, bras, kets)
    assert one.last_timing()[1] == 1                     # one recursion launch
    b = multi.run(M, bras, kets)
    ref = orc.cheb_moments(n, cp, ri, v, M, bras, kets)
    tol = {"fp64": 1e-10, "dd": DD_TOL, "mixed": MIXED_TOL}[precision]
    assert np.max(np.abs(a - ref)) / abs(ref[0]) <= tol
    assert np.max(np.abs(a - b)) / abs(ref[0]) <= (1e-13 if precision != "mixed" else 1e-6)


@pytest.mark.parametrize("precision,doubling", [("fp64", False), ("fp64", True), ("mixed", True), ("dd", False),
                                                ("dd", True)])
@pytest.mark.parametrize("case", ["fcc_disorder", "square_nn2_gauge"])
def test_wide_rows_pipelined_gathers(gpu, precision, doubling, case):
    """Rows wider than one group of 4 gathers (FCC: 12 neighbours; square with
    first and second neighbours: 8) take the pipelined column loads."""
    tb = gpu
    if case == "fcc_disorder":
        _, H = _system(tb, "fcc", (10, 9, 8), disorder=(2.0, 4))
        a = 13.2
    else:
        cell = tb.Square().add_hopping("A", 1, 1.0).add_hopping("A", 2, 0.3)
        X = tb.PartialLattice(cell, (20, 18))
        X.set_gauge_linear(*landau_gauge(0.07))
        H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], complex)
        a = 5.4
    G, cp, ri, v = _rescaled_csc(tb, H, a)
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, 6, 2)
    bras = kets if doubling else orc.random_phase_kets(n, 6, 3)
    mu = tb.Cheb_first_kind_seq_braket((n, cp, ri, v), 80, bras, kets, precision=precision, doubling=doubling)
    ref = orc.cheb_moments(n, cp, ri, v, 80, bras, kets)
    tol = {"fp64": 1e-10, "dd": DD_TOL, "mixed": MIXED_TOL}[precision]
    assert _err(mu, ref) <= tol
