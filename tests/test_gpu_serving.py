"""Serving loop on the GPU: every request against the FP64 oracle on the same
seeded kets, the same bits alone and in a mix, and admission under a budget.

Tolerances (relative to mu_0, as for the single-solve moments):
  FP64 requests   <= 1e-10
  mixed requests  <= MIXED_TOL (M <= 256)"""
import numpy as np
import pytest

import oracle as orc
from serving_cases import bounds, cell, lattice

pytestmark = pytest.mark.gpu
MIXED_TOL = 2e-5


def _oracle(tb, X, n_mom, R, seed, emin, emax):
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1] * X.dim, float)
    G = tb.GreenFunction(8, H, emin, emax)
    cp, ri, v = G.scaled_HE.to_csc()
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, R, seed)
    return orc.cheb_moments(n, cp, ri, v, n_mom, kets, kets)


def _err(mu, ref):
    return float(np.max(np.abs(mu - ref)) / abs(ref[0]))


CASES = [  # kind, L, W, M, R, precision
    ("square", 24, 1.0, 128, 4, "mixed"),
    ("honeycomb", 16, 0.5, 64, 8, "fp64"),
    ("kagome", 12, 2.0, 96, 5, "mixed"),
    ("lieb", 12, 0.0, 80, 64, "fp64"),
    ("fcc", 8, 1.5, 201, 16, "mixed"),
    ("square", 10, 0.3, 2, 3, "fp64"),
    ("honeycomb", 20, 1.2, 256, 64, "mixed"),
    ("kagome", 14, 0.7, 120, 8, "dd"),
    ("fcc", 6, 1.0, 64, 33, "dd"),
    ("square", 40, 0.8, 96, 80, "mixed"),        # two complex64 lanes (64 + 16 vectors), two width groups
]


def test_requests_vs_oracle(gpu):
    tb = gpu
    with tb.DosServer(autotune=True, steps_per_round=8) as srv:
        tickets = []
        for i, (kind, L, W, M, R, prec) in enumerate(CASES):
            X = lattice(tb, kind, L, W, seed=100 + i)
            emin, emax = bounds(kind, W)
            tickets.append(srv.submit(X, M, R, seed=i, e_min=emin, e_max=emax, precision=prec))
        for i, (kind, L, W, M, R, prec) in enumerate(CASES):
            mu, times = srv.result(tickets[i], timeout_s=120)
            X = lattice(tb, kind, L, W, seed=100 + i)
            ref = _oracle(tb, X, M, R, i, *bounds(kind, W))
            tol = MIXED_TOL if prec == "mixed" else 1e-10
            assert _err(mu, ref) <= tol, (kind, prec, _err(mu, ref))
            assert abs(mu[0] - R) < 1e-4 * R
            assert times[3] >= times[2] >= 0
        st = srv.stats()
        assert st["done"] == len(CASES) and st["failed"] == 0
        assert st["reserved_bytes"] == 0
        tun = srv.tuning()
        assert len(tun) == 26                         # 13 (precision, width) groups, ELL and class form each
        assert sum(t["form"] == "classes" for t in tun) == 13


def _mix(tb, cells):
    out = []
    kinds = ["square", "honeycomb", "kagome", "lieb", "fcc"]
    rng = np.random.default_rng(5)
    for i in range(12):
        kind = kinds[i % 5]
        L = int(rng.integers(8, 14)) if kind == "fcc" else int(rng.integers(16, 72))
        W = float(rng.uniform(0, 2))
        out.append(dict(kind=kind, L=L, W=W, M=int(rng.choice([64, 128, 256])), R=int(rng.choice([4, 8, 16, 32, 64])),
                        prec="fp64" if i % 3 == 0 else "mixed", seed=200 + i))
    return out


def _submit(tb, srv, c, cells):
    X = lattice(tb, c["kind"], c["L"], c["W"], seed=c["seed"], cells=cells)
    emin, emax = bounds(c["kind"], c["W"])
    return srv.submit(X, c["M"], c["R"], seed=c["seed"], e_min=emin, e_max=emax, precision=c["prec"])


@pytest.mark.parametrize("prec", ["mixed", "fp64", "dd"])
def test_alone_equals_in_mix(gpu, prec):
    """A request's moments are the same bits alone, in a mix of other lattices,
    widths and precisions, and with another round length and launch shape."""
    tb = gpu
    cells = {k: cell(tb, k) for k in ("square", "honeycomb", "kagome", "lieb", "fcc")}
    probe = dict(kind="honeycomb", L=48, W=1.3, M=200, R=16, prec=prec, seed=77)
    with tb.DosServer(autotune=True, steps_per_round=16) as srv:
        alone, _ = srv.result(_submit(tb, srv, probe, cells))
        mix = _mix(tb, cells)
        tickets = [_submit(tb, srv, c, cells) for c in mix[:6]]
        t_probe = _submit(tb, srv, probe, cells)
        tickets += [_submit(tb, srv, c, cells) for c in mix[6:]]
        in_mix, _ = srv.result(t_probe)
        for t in tickets:
            srv.result(t)
        assert srv.stats()["peak_resident"] > 1
    assert np.array_equal(alone, in_mix)
    with tb.DosServer(autotune=False, steps_per_round=4) as srv2:
        other, _ = srv2.result(_submit(tb, srv2, probe, cells))
    assert np.array_equal(alone, other)


def test_class_form_equals_ell(gpu, monkeypatch):
    """Requests whose H~ has row classes run in the class form by default; a
    server created with TBK_SERVE_CLASSES=0 keeps them in the ELL form.  Both
    give the same bits, alone and in a mix."""
    tb = gpu
    cells = {k: cell(tb, k) for k in ("square", "honeycomb", "kagome", "lieb", "fcc")}
    probe = dict(kind="honeycomb", L=48, W=1.3, M=200, R=16, prec="mixed", seed=77)
    monkeypatch.setenv("TBK_SERVE_CLASSES", "0")
    with tb.DosServer(autotune=False) as srv:
        ell, _ = srv.result(_submit(tb, srv, probe, cells))
    monkeypatch.delenv("TBK_SERVE_CLASSES")
    with tb.DosServer(autotune=True, steps_per_round=16) as srv:
        alone, _ = srv.result(_submit(tb, srv, probe, cells))
        mix = _mix(tb, cells)
        tickets = [_submit(tb, srv, c, cells) for c in mix[:6]]
        t_probe = _submit(tb, srv, probe, cells)
        tickets += [_submit(tb, srv, c, cells) for c in mix[6:]]
        in_mix, _ = srv.result(t_probe)
        for t in tickets:
            srv.result(t)
        assert sum(t["form"] == "classes" for t in srv.tuning()) == 13
    assert np.array_equal(alone, in_mix)
    assert np.array_equal(alone, ell)


def test_budget_admission(gpu):
    tb = gpu
    X = lattice(tb, "square", 96, 1.0, seed=1)
    emin, emax = bounds("square", 1.0)
    peak, res = tb.request_footprint(X, 128, 32, "mixed", emin, emax)
    # room for one build peak plus half of one request's vector blocks: a
    # resident request (which holds all of its blocks) and a second build never fit
    budget = peak + 96 * 96 * 32 * 8
    with tb.DosServer(budget_gb=budget / 1e9, autotune=False) as srv:
        ts = [srv.submit(X, 128, 32, seed=s, e_min=emin, e_max=emax) for s in range(5)]
        mus = [srv.result(t)[0] for t in ts]
        st = srv.stats()
        assert st["done"] == 5
        assert st["peak_reserved_bytes"] <= budget
        assert st["peak_resident"] == 1          # one build peak fits, two do not
        assert st["build_overshoot_bytes"] <= 0  # the pool never held more than was charged
        big = lattice(tb, "square", 400)
        with pytest.raises(tb.TbkError) as e:
            srv.submit(big, 128, 64, seed=0, e_min=emin, e_max=emax)
        assert e.value.code == tb.capi.TBK_ERR_BUDGET
    # different seeds, different moments; the same seed alone reproduces
    assert not np.array_equal(mus[0], mus[1])
    ref = _oracle(tb, X, 128, 32, 3, emin, emax)
    assert _err(mus[3], ref) <= MIXED_TOL


def test_many_small_requests_packed(gpu):
    tb = gpu
    cells = {"square": cell(tb, "square")}
    with tb.DosServer(autotune=False, steps_per_round=16) as srv:
        ts = [_submit(tb, srv, dict(kind="square", L=8 + (i % 24), W=0.5, M=64, R=4, prec="mixed", seed=i), cells)
              for i in range(96)]
        res = [srv.result(t)[0] for t in ts]
        st = srv.stats()
    assert st["done"] == 96
    # 33 steps each: 3 rounds alone; packed, fewer rounds than one after another
    assert st["rounds"] < 3 * 96
    assert st["peak_resident"] > 1
    for i in (0, 37, 95):
        X = lattice(tb, "square", 8 + (i % 24), 0.5, seed=i)
        ref = _oracle(tb, X, 64, 4, i, *bounds("square", 0.5))
        assert _err(res[i], ref) <= MIXED_TOL


def test_poll_unknown_ticket(gpu):
    tb = gpu
    with tb.DosServer(autotune=False) as srv:
        with pytest.raises(KeyError):
            srv.poll(12345)
        import ctypes as C
        assert tb.capi.lib().tbk_server_poll(srv._h, 12345, 0, None, None) == tb.capi.TBK_ERR_INVALID


def test_failed_build_fails_only_its_request(gpu):
    """Fault injection on the host side: a lattice the builder rejects (an atom
    touching more than its hopping-term limit) fails its own request with the
    builder's status and message; the requests around it complete and the
    admission charge is returned."""
    tb = gpu
    from tight_binding_gb300.serving import model_bounds
    bad_cell = tb.FCC()
    for nn in range(1, 7):                      # 43 canonical hoppings, 86 terms touch atom A
        bad_cell.add_hopping("A", nn, 1.0)
    bad = tb.PartialLattice(bad_cell, (6, 6, 6))
    good = lattice(tb, "square", 24, 0.5, seed=1)
    lo, hi = model_bounds("square", 0.5)
    with tb.DosServer(autotune=False) as srv:
        t1 = srv.submit(good, 64, 4, seed=1, e_min=lo, e_max=hi)
        t2 = srv.submit(bad, 64, 4, seed=2, e_min=-60, e_max=60)
        t3 = srv.submit(good, 64, 4, seed=3, e_min=lo, e_max=hi)
        r1 = srv.result(t1)[0]
        with pytest.raises(tb.TbkError) as e:
            srv.result(t2)
        assert e.value.code == tb.capi.TBK_ERR_UNSUPPORTED and "hopping terms" in str(e.value)
        r3 = srv.result(t3)[0]
        st = srv.stats()
    assert st["done"] == 2 and st["failed"] == 1 and st["reserved_bytes"] == 0
    assert np.all(np.isfinite(r1)) and np.all(np.isfinite(r3)) and not np.array_equal(r1, r3)


def _kubo_lattice(tb):
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (24, 20))
    G = np.zeros((3, 3))
    G[1, 0] = 2 * np.pi / 32
    X.set_gauge_linear(G, np.zeros(3))
    X.set_scalar_disorder(0.5, 3)
    return X


@pytest.mark.parametrize("kind", ["bastin", "greenwood"])
def test_kubo_requests_equal_direct_solve(gpu, kind):
    """A conductivity request through the server gives the bits of the direct
    tbk_kubo_mu solve on the same H~, commutators, seed and kernel, also while
    DoS requests run beside it; the DoS results keep their alone bits."""
    tb = gpu
    X = _kubo_lattice(tb)
    M, R, seed, lo, hi = 48, 4, 7, -4.4, 4.4
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([0, 1], complex)
    Gf = tb.GreenFunction(M, H, lo, hi)
    vx = tb.commutator(Gf.scaled_HE, X.op_position(0))
    vy = tb.commutator(Gf.scaled_HE, X.op_position(1))
    kw = dict(M=M, R=R, seed=seed, kernel=tb.Lorentz(6.0), tensor=True, recursion="dd")
    if kind == "bastin":
        direct = tb.kubo_mu(Gf.scaled_HE, None, None, vx, vy, **kw)
    else:
        direct = tb.kubo_mu(Gf.scaled_HE, vx, vx, None, None, **kw)
    dos_cases = CASES[:4]
    with tb.DosServer(autotune=False, steps_per_round=8) as srv:
        alone = []
        for i, (k, L, W, Mm, Rr, prec) in enumerate(dos_cases):
            Xd = lattice(tb, k, L, W, seed=200 + i)
            alone.append(srv.result(srv.submit(Xd, Mm, Rr, seed=i, e_min=bounds(k, W)[0], e_max=bounds(k, W)[1],
                                               precision=prec))[0])
        tickets = []
        for i, (k, L, W, Mm, Rr, prec) in enumerate(dos_cases[:2]):
            Xd = lattice(tb, k, L, W, seed=200 + i)
            tickets.append(srv.submit(Xd, Mm, Rr, seed=i, e_min=bounds(k, W)[0], e_max=bounds(k, W)[1], precision=prec))
        tk = srv.submit_kubo(X, kind, M, R, seed, lo, hi, axes=(0, 1), kernel=tb.Lorentz(6.0), precision="dd",
                             extend=[0, 1], scalar=complex)
        for i, (k, L, W, Mm, Rr, prec) in enumerate(dos_cases[2:]):
            Xd = lattice(tb, k, L, W, seed=202 + i)
            tickets.append(srv.submit(Xd, Mm, Rr, seed=2 + i, e_min=bounds(k, W)[0], e_max=bounds(k, W)[1],
                                      precision=prec))
        mu, times = srv.result(tk, timeout_s=300)
        assert mu.shape == (M, M) and np.array_equal(mu, direct)
        for i, t in enumerate(tickets):
            assert np.array_equal(srv.result(t, timeout_s=300)[0], alone[i])
        assert srv.stats()["failed"] == 0


def test_kubo_request_over_budget_is_refused(gpu):
    tb = gpu
    X = tb.PartialLattice(tb.FCC().add_hopping("A", 1, 1.0), (64, 64, 64))
    with tb.DosServer(budget_gb=2.0, autotune=False) as srv:
        with pytest.raises(tb.TbkError, match="budget"):
            srv.submit_kubo(X, "greenwood", 1024, 8, 0, -13.0, 13.0, axes=(0,), extend=[1, 1, 1], scalar=float)
