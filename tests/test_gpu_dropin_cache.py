"""The drop-in's plan cache (tbk_cheb_braket_*): repeated calls on the same
host CSC reuse the device matrix and plan, and give the bits of an uncached
call; a changed value, structure or width is seen by the device comparison and
rebuilds; tbk_cheb_braket_release frees the cache and later calls still work.
"""
import numpy as np
import pytest

import oracle as orc

pytestmark = pytest.mark.gpu


def _csc(tb, L=24, W=1.0, seed=1):
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (L, L))
    X.set_scalar_disorder(W, seed)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    cp, ri, v = tb.GreenFunction(8, H, -5.0, 5.0).scaled_HE.to_csc()
    return len(cp) - 1, cp, ri, v


def _call(capi, n, cp, ri, v, M, bras, kets, flags):
    mu = np.zeros(M)
    K = np.asfortranarray(kets)
    B = K if bras is kets else np.asfortranarray(bras)
    capi.check(capi.lib().tbk_cheb_braket_real(n, len(ri), capi.ptr(cp), capi.ptr(ri), capi.ptr(v), M, capi.ptr(B),
                                               capi.ptr(K), K.shape[1], flags, capi.ptr(mu)))
    return mu


@pytest.mark.parametrize("prec", ["fp64", "mixed", "dd"])
def test_repeated_calls_equal_uncached(gpu, prec):
    tb = gpu
    from tight_binding_gb300 import capi

    p = {"fp64": capi.PREC_FP64, "mixed": capi.PREC_MIXED, "dd": capi.PREC_DD}[prec]
    n, cp, ri, v = _csc(tb)
    kets = orc.random_phase_kets(n, 8, 0)
    ref = _call(capi, n, cp, ri, v, 128, kets, kets, p | capi.FLAG_DOUBLING | capi.FLAG_NO_CACHE)
    for _ in range(4):                 # build, second identical run (graph capture), replays
        mu = _call(capi, n, cp, ri, v, 128, kets, kets, p | capi.FLAG_DOUBLING)
        assert np.array_equal(mu, ref)


def test_changed_matrix_is_seen(gpu):
    tb = gpu
    from tight_binding_gb300 import capi

    n, cp, ri, v = _csc(tb)
    kets = orc.random_phase_kets(n, 4, 2)
    bras = orc.random_phase_kets(n, 4, 3)
    f = capi.PREC_FP64
    a = _call(capi, n, cp, ri, v, 64, bras, kets, f)
    v2 = v.copy()
    v2[len(v2) // 2] += 1e-3                          # one value, same structure
    b = _call(capi, n, cp, ri, v2, 64, bras, kets, f)
    assert not np.array_equal(a, b)
    assert np.array_equal(b, _call(capi, n, cp, ri, v2, 64, bras, kets, f | capi.FLAG_NO_CACHE))
    assert np.max(np.abs(b - orc.cheb_moments(n, cp, ri, v2, 64, bras, kets))) <= 1e-10 * abs(b[0])
    # another lattice size, then back to the first matrix, other widths and flags
    n3, cp3, ri3, v3 = _csc(tb, L=20, W=0.5, seed=4)
    k3 = orc.random_phase_kets(n3, 3, 1)
    c = _call(capi, n3, cp3, ri3, v3, 32, k3, k3, f)
    assert np.max(np.abs(c - orc.cheb_moments(n3, cp3, ri3, v3, 32, k3, k3))) <= 1e-10 * abs(c[0])
    assert np.array_equal(_call(capi, n, cp, ri, v, 64, bras, kets, f), a)
    k5 = orc.random_phase_kets(n, 5, 9)
    for flags in (f, capi.PREC_MIXED | capi.FLAG_DOUBLING, f | capi.FLAG_DOUBLING):
        got = _call(capi, n, cp, ri, v, 48, k5, k5, flags)
        want = _call(capi, n, cp, ri, v, 48, k5, k5, flags | capi.FLAG_NO_CACHE)
        assert np.array_equal(got, want)


def test_release(gpu):
    tb = gpu
    from tight_binding_gb300 import capi

    n, cp, ri, v = _csc(tb, L=16)
    kets = orc.random_phase_kets(n, 2, 5)
    a = _call(capi, n, cp, ri, v, 32, kets, kets, capi.PREC_FP64)
    capi.lib().tbk_cheb_braket_release()
    capi.lib().tbk_cheb_braket_release()              # twice: nothing left to free
    assert np.array_equal(_call(capi, n, cp, ri, v, 32, kets, kets, capi.PREC_FP64), a)
    capi.lib().tbk_cheb_braket_release()
