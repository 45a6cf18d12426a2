"""The TMA-staged warp-specialised step kernel (TBK_FLAG_STAGED, complex64):
parity with the CPU oracle, and its failure path.

Failure path: tbk_set_wait_limit lowers the number of polls the kernel's
mbarrier ring waits make before giving up.  With 0 polls every ring wait gives
up at once (the producer issues nothing, the consumers stop): the call must
return TBK_ERR_TIMEOUT, and the next call with the default limit must give the
oracle's moments.  With 2 polls the outcome depends on timing; either result
is accepted, and the copies the producer had in flight are always waited for
before its CTA retires.  No wait here can hang: every one is bounded.
"""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu
MIXED_TOL = 2e-5


def _system(tb, kind, L):
    cell = tb.Honeycomb().add_hopping("A", 1, -2.7) if kind == "honeycomb" else tb.Square().add_hopping("A", 1, 1.0)
    X = tb.PartialLattice(cell, L)
    X.set_scalar_disorder(1.0, 3)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    a = 8.7 if kind == "honeycomb" else 4.6
    return tb.GreenFunction(8, H, -a, a).scaled_HE


def _err(mu, ref):
    return float(np.max(np.abs(mu - ref)) / abs(ref[0]))


@pytest.mark.parametrize("kind,L,R", [("square", (64, 48), 8), ("honeycomb", (96, 80), 32), ("square", (40, 40), 3)])
def test_staged_parity_vs_oracle(gpu, kind, L, R):
    tb = gpu
    from tight_binding_gb300 import capi

    Ht = _system(tb, kind, L)
    cp, ri, v = Ht.to_csc()
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, R, 1)
    bras = orc.random_phase_kets(n, R, 2)
    ref_dbl = orc.cheb_moments(n, cp, ri, v, 96, kets, kets)
    ref_brk = orc.cheb_moments(n, cp, ri, v, 48, bras, kets)
    s = tb.KpmSolver(Ht, R, precision="mixed", doubling=True, flags=capi.FLAG_STAGED)
    assert _err(s.run(96, kets, kets), ref_dbl) <= MIXED_TOL
    b = tb.KpmSolver(Ht, R, precision="mixed", doubling=False, flags=capi.FLAG_STAGED)
    assert _err(b.run(48, bras, kets), ref_brk) <= MIXED_TOL


def test_staged_wait_timeout_then_recovery(gpu):
    tb = gpu
    from tight_binding_gb300 import capi

    Ht = _system(tb, "honeycomb", (64, 64))
    cp, ri, v = Ht.to_csc()
    n = len(cp) - 1
    kets = orc.random_phase_kets(n, 32, 4)
    ref = orc.cheb_moments(n, cp, ri, v, 64, kets, kets)
    s = tb.KpmSolver(Ht, 32, precision="mixed", doubling=True, flags=capi.FLAG_STAGED)
    try:
        capi.check(capi.lib().tbk_set_wait_limit(0))
        with pytest.raises(tb.TbkError) as ei:
            s.run(64, kets, kets)
        assert ei.value.code == capi.TBK_ERR_TIMEOUT
        capi.check(capi.lib().tbk_set_wait_limit(2))
        try:
            mu = s.run(64, kets, kets)
            assert _err(mu, ref) <= MIXED_TOL
        except tb.TbkError as e:
            assert e.code == capi.TBK_ERR_TIMEOUT
    finally:
        capi.check(capi.lib().tbk_set_wait_limit(-1))
    assert _err(s.run(64, kets, kets), ref) <= MIXED_TOL
    # the one-pass kernel (no waits) is unaffected by the limit at any time
    assert _err(tb.KpmSolver(Ht, 32, precision="mixed", doubling=True).run(64, kets, kets), ref) <= MIXED_TOL
    assert capi.lib().tbk_set_wait_limit(1 << 30) == capi.TBK_ERR_INVALID
