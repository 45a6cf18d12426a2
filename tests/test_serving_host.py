"""Host side of the serving API: admission footprints and request checks
(no device needed)."""
import ctypes as C

import pytest

from serving_cases import lattice


def test_footprint_grows_with_width_and_precision(tb):
    X = lattice(tb, "square", 64)
    p1, r1 = tb.request_footprint(X, 256, 8, "mixed", -4.1, 4.1)
    p2, r2 = tb.request_footprint(X, 256, 16, "mixed", -4.1, 4.1)
    p3, r3 = tb.request_footprint(X, 256, 8, "fp64", -4.1, 4.1)
    p4, r4 = tb.request_footprint(X, 1024, 8, "mixed", -4.1, 4.1)
    assert r2 > r1 and r3 > r1 and r4 > r1
    assert p1 >= r1 and p3 >= r3
    n = 64 * 64
    # two complex64 blocks of 8 vectors, the ELL (4 neighbours) and the diagonal
    assert r1 >= 2 * n * 8 * 8 + n * 4 * 8 + n * 4
    # fp64 request: complex128 blocks and FP64 values
    assert r3 >= 2 * n * 8 * 16 + n * 4 * 12


def test_footprint_multi_atom_and_3d(tb):
    for kind, L, n in (("kagome", 16, 3 * 256), ("lieb", 16, 3 * 256), ("fcc", 8, 512)):
        X = lattice(tb, kind, L, W=1.0, seed=3)
        p, r = tb.request_footprint(X, 128, 4, "mixed", -13, 13)
        assert r >= 2 * n * 4 * 8 and p >= r


def test_request_checks(tb):
    X = lattice(tb, "square", 8)
    for kw in (dict(n_mom=1, R=4), dict(n_mom=16, R=0)):
        with pytest.raises(tb.TbkError) as e:
            tb.request_footprint(X, kw["n_mom"], kw["R"], "mixed", -4.1, 4.1)
        assert e.value.code == tb.capi.TBK_ERR_INVALID
    with pytest.raises(tb.TbkError):
        tb.request_footprint(X, 16, 4, "mixed", 4.1, -4.1)
    from tight_binding_gb300.serving import _request
    q = _request(X, 16, 4, 0, -4.1, 4.1)
    q.precision = 9
    assert tb.capi.lib().tbk_request_footprint(C.byref(q), None, None) == tb.capi.TBK_ERR_INVALID


def test_server_needs_a_device(tb):
    if tb.device_count() > 0:
        pytest.skip("a device is visible")
    with pytest.raises(tb.TbkError) as e:
        tb.DosServer(autotune=False)
    assert e.value.code == tb.capi.TBK_ERR_CUDA


def test_conductivity_request_footprint_and_checks(tb):
    """Conductivity requests: the footprint carries both stored block sides
    (grows with M), is above the DoS footprint of the same lattice, and bad
    axes are refused before any device work."""
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (256, 256))
    dos, _ = tb.request_footprint(X, 512, 16, precision="dd")
    k1, _ = tb.request_footprint(X, 512, 16, precision="dd", kind="bastin")
    k2, _ = tb.request_footprint(X, 1024, 16, precision="dd", kind="bastin")
    assert k1 > dos and k2 > k1
    stores = 2 * 512 * 65536 * 16 * 8
    assert k1 >= stores
    with pytest.raises(tb.TbkError, match="axis out of range"):
        tb.request_footprint(X, 64, 4, kind="greenwood", axes=(2,))


def test_unknown_request_kind_is_refused(tb):
    import ctypes as C
    from tight_binding_gb300 import capi
    from tight_binding_gb300.serving import _request
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (8, 8))
    q = _request(X, 16, 2, 0, -4.1, 4.1)
    q.kind = 7
    a, b = C.c_int64(), C.c_int64()
    assert capi.lib().tbk_request_footprint(C.byref(q), C.byref(a), C.byref(b)) == capi.TBK_ERR_INVALID
    assert b"unknown request kind" in capi.lib().tbk_last_error()
