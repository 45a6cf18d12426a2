"""Device Hamiltonian builder vs the oracle's setFromTriplets restatement:
structure (col_ptr, row_idx) bit-exact; values bit-exact except where a Peierls
phase goes through cos/sin (CUDA vs libm, compared to a few ulp)."""
import json
from pathlib import Path

import numpy as np
import pytest

import oracle as orc
from helpers import landau_gauge, spec_from, with_onsite_zeros

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"

MODE = {"sparse": orc.MODE_SPARSE, "periodic": orc.MODE_PERIODIC_BARE, "bare": orc.MODE_BARE}


def _build_both(tb, cell, span, mode, cplx, extend=None, gauge=None, scalar=None, disorder=None, removed=None):
    X = tb.PartialLattice(cell, span)
    N = X.get_total_number()
    glin = None
    if gauge is not None:
        G, c = gauge
        X.set_gauge_linear(G, c)
        glin = np.concatenate([np.asarray(G).reshape(-1), c])
    V = None
    ocell = cell
    if scalar is not None:
        X.set_scalar_values(scalar)
        V = scalar
        ocell = with_onsite_zeros(cell)
    if disorder is not None:
        W, seed = disorder
        X.set_scalar_disorder(W, seed)
        V = orc.uniform_disorder(N, W, seed)
        ocell = with_onsite_zeros(cell)
    if removed is not None:
        X.remove_sites(removed)
    scalar_t = complex if cplx else float
    if mode == "sparse":
        H = X.get_Hamiltonian_sparse(scalar_t)
    elif mode == "periodic":
        H = X.get_Hamiltonian_periodic_extend_bare_sparse(extend, scalar_t)
    else:
        H = X.get_Hamiltonian_bare_sparse(scalar_t)
    spec = spec_from(ocell if mode != "bare" else cell, span, mode=MODE[mode], is_complex=cplx, extend=extend,
                     gauge_linear=glin if mode != "bare" else None, scalar_site=V if mode != "bare" else None,
                     removed=None if removed is None else removed.astype(np.int32))
    ref = orc.build_csc(spec)
    return H, ref


def _assert_same(H, ref, exact_values=True):
    cp, ri, v = H.to_csc()
    rcp, rri, rv = ref
    assert np.array_equal(cp, rcp)
    assert np.array_equal(ri, rri)
    if exact_values:
        assert np.array_equal(v, rv)
    else:
        assert np.max(np.abs(v - rv)) <= 4e-16 * max(1.0, np.max(np.abs(rv)))


CASES = [
    # id, model factory, span, mode, complex, extend, extras
    ("square_pbc", lambda tb: tb.Square().add_hopping("A", 1, 1.0), (16, 12), "periodic", False, [1, 1], {}),
    ("square_2x2_pbc_duplicates", lambda tb: tb.Square().add_hopping("A", 1, 1.0), (2, 2), "periodic", True, [1, 1], {}),
    ("square_1x3_self_hops", lambda tb: tb.Square().add_hopping("A", 1, 0.7), (1, 3), "periodic", True, [1, 1], {}),
    ("square_open", lambda tb: tb.Square().add_hopping("A", 1, 1.0), (9, 7), "sparse", False, None, {}),
    ("honeycomb_open", lambda tb: tb.Honeycomb().add_hopping("A", 1, -2.7), (8, 6), "sparse", True, None, {}),
    ("kagome_open", lambda tb: _kagome(tb), (5, 6), "sparse", False, None, {}),
    ("lieb_pbc", lambda tb: tb.Lieb().add_hopping("A", 1, 1.0), (6, 5), "periodic", False, [1, 1], {}),
    ("fcc_pbc", lambda tb: tb.FCC().add_hopping("A", 1, 1.0), (4, 5, 3), "periodic", False, [1, 1, 1], {}),
    ("cubic_mixed_bc", lambda tb: tb.Cubic().add_hopping("A", 1, 1.0), (4, 3, 5), "periodic", True, [1, 0, 1], {}),
    ("chain_pbc", lambda tb: tb.Chain().add_hopping("A", 1, 1.0), (10,), "periodic", False, [1], {}),
    ("ti_sp_complex", lambda tb: tb.TI_sp(), (5, 4), "sparse", True, None, {}),
    ("ti_sp_bare", lambda tb: tb.TI_sp(), (5, 4), "bare", True, None, {}),
    ("sawtooth", lambda tb: tb.sawtooth_chain_p(0.25, 0.3535), (12,), "sparse", False, None, {}),
    ("stub_pbc", lambda tb: tb.stub_1d_p(1.0, 0.5), (9,), "periodic", True, [1], {}),
]


def _kagome(tb):
    k = tb.Kagome()
    for a in "ABC":
        k.add_hopping(a, 1, 1.0)
    return k


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_builder_structure_and_values(gpu, case):
    tb = gpu
    _, factory, span, mode, cplx, extend, extra = case
    H, ref = _build_both(tb, factory(tb), span, mode, cplx, extend=extend, **extra)
    _assert_same(H, ref)


def test_builder_disorder_on_device(gpu):
    tb = gpu
    cell = tb.Honeycomb().add_hopping("A", 1, -2.7)
    H, ref = _build_both(tb, cell, (16, 16), "periodic", False, extend=[1, 1], disorder=(1.0, 1))
    _assert_same(H, ref)   # counter-based RNG: identical draws on host and device


def test_builder_scalar_field_values(gpu):
    tb = gpu
    cell = tb.Square().add_hopping("A", 1, 1.0)
    V = np.linspace(-0.3, 0.4, 8 * 8)
    H, ref = _build_both(tb, cell, (8, 8), "sparse", True, scalar=V)
    _assert_same(H, ref)


@pytest.mark.parametrize("mode,extend", [("sparse", None), ("periodic", [0, 1])])
def test_builder_landau_gauge(gpu, mode, extend):
    tb = gpu
    cell = tb.Square().add_hopping("A", 1, 1.0)
    H, ref = _build_both(tb, cell, (12, 10), mode, True, extend=extend, gauge=landau_gauge(2 * np.pi / 64))
    _assert_same(H, ref, exact_values=False)
    # Hermitian
    M = H.to_scipy()
    assert abs(M - M.conj().T).max() < 1e-15


def test_builder_gauge_per_site(gpu):
    tb = gpu
    cell = tb.Honeycomb().add_hopping("A", 1, 1.0)
    X = tb.PartialLattice(cell, (6, 5))
    B = 0.05
    X.set_gauge_field(lambda r: np.stack([-B * r[:, 1] / 2, B * r[:, 0] / 2, 0 * r[:, 0]], axis=1))
    H = X.get_Hamiltonian_sparse(complex)
    A = np.stack([-B * X.site_positions()[:, 1] / 2, B * X.site_positions()[:, 0] / 2,
                  0 * X.site_positions()[:, 0]], axis=1)
    ref = orc.build_csc(spec_from(cell, (6, 5), mode=orc.MODE_SPARSE, is_complex=True, gauge_site=A))
    _assert_same(H, ref, exact_values=False)


def test_builder_vacancies(gpu):
    tb = gpu
    cell = tb.Honeycomb().add_hopping("A", 1, 1.0)
    rng = np.random.default_rng(5)
    removed = (rng.random(2 * 7 * 6) < 0.2).astype(np.uint8)
    H, ref = _build_both(tb, cell, (7, 6), "sparse", False, removed=removed)
    _assert_same(H, ref)


def test_rescale_and_commutator_bit_exact(gpu):
    tb = gpu
    cell = tb.Square().add_hopping("A", 1, 1.0)
    X = tb.PartialLattice(cell, (9, 8))
    H = X.get_Hamiltonian_sparse(complex)
    G = tb.GreenFunction(16, H, -4.1, 4.3)
    cp, ri, v = H.to_csc()
    ref = orc.rescale_csc(len(cp) - 1, cp, ri, v, G.a, G.b)
    got = G.scaled_HE.to_csc()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    # velocity: X H~ - H~ X (TB/snippets.h:316) and op_velocity (real, open BC)
    Xop = X.op_position(0)
    xd = orc.position_diag(spec_from(cell, (9, 8)), 0)
    assert np.array_equal(Xop.to_csc()[2], xd)
    V = tb.commutator(G.scaled_HE, Xop)
    cpv, riv, vv = V.to_csc()
    assert np.array_equal(cpv, ref[0]) and np.array_equal(riv, ref[1])
    assert np.array_equal(vv, orc.commutator_values(len(cp) - 1, ref[0], ref[1], ref[2], xd))
    vel = X.op_velocity(1)
    Hr = X.get_Hamiltonian_sparse(float).to_csc()
    yd = orc.position_diag(spec_from(cell, (9, 8)), 1)
    assert np.array_equal(vel.to_csc()[2], orc.commutator_values(len(cp) - 1, Hr[0], Hr[1], Hr[2], yd))


def test_config_sizes_counts(gpu):
    tb = gpu
    counts = json.loads((GOLD / "counts.json").read_text())
    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, -2.7), (1024, 1024))
    X.set_scalar_disorder(1.0, 1)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    c = counts["honeycomb_1024x1024_pbc_disorder"]
    assert H.shape[0] == c["N"] and H.nnz == c["nnz_H"]
    G = tb.GreenFunction(8, H, -8.2, 8.2)
    assert G.scaled_HE.nnz == c["nnz_Ht"]
    X2 = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (256, 256))
    H2 = X2.get_Hamiltonian_periodic_extend_bare_sparse([0, 1], complex)
    c2 = counts["square_256x256_openx_pbcy"]
    assert H2.nnz == c2["nnz_H"]
    assert tb.GreenFunction(8, H2, -4.1, 4.1).scaled_HE.nnz == c2["nnz_Ht"]
    X3 = tb.PartialLattice(tb.FCC().add_hopping("A", 1, 1.0), (128, 128, 128))
    X3.set_scalar_disorder(2.0, 4)
    H3 = X3.get_Hamiltonian_periodic_extend_bare_sparse([1, 1, 1], float)
    assert H3.nnz == counts["fcc_128_pbc_disorder"]["nnz_H"]


CONFIG_SYSTEMS = {
    # name: (cell factory, span, extend, complex, disorder (W, seed), Landau B, rescale bounds)
    "honeycomb_1024_pbc_disorder": (lambda tb: tb.Honeycomb().add_hopping("A", 1, -2.7), (1024, 1024), [1, 1],
                                    False, (1.0, 1), None, (-8.7, 8.7)),
    "square_256_openx_pbcy_landau": (lambda tb: tb.Square().add_hopping("A", 1, 1.0), (256, 256), [0, 1], True,
                                     None, 2 * np.pi / 64, (-4.0, 4.0)),
    "fcc_128_pbc_disorder": (lambda tb: tb.FCC().add_hopping("A", 1, 1.0), (128, 128, 128), [1, 1, 1], False,
                             (2.0, 4), None, (-13.0, 13.0)),
}


@pytest.mark.parametrize("name", sorted(CONFIG_SYSTEMS))
def test_config_sizes_full_arrays(gpu, name):
    """The benchmark lattices at full size: every col_ptr / row_idx entry of H
    and of H~ = (H - bI)/a bit-exact with the oracle; values bit-exact, except
    the Landau-gauge phases (device cos/sin against libm), which agree to 4e-16
    absolute (|t| = 1)."""
    tb = gpu
    mk, span, extend, cplx, disorder, B, (lo, hi) = CONFIG_SYSTEMS[name]
    cell = mk(tb)
    H, ref = _build_both(tb, cell, span, "periodic", cplx, extend=extend,
                         gauge=landau_gauge(B) if B is not None else None, disorder=disorder)
    cp, ri, v = H.to_csc()
    assert np.array_equal(cp, ref[0]) and np.array_equal(ri, ref[1])
    if B is None:
        assert np.array_equal(v, ref[2])
    else:
        assert np.max(np.abs(v - ref[2])) <= 4e-16
    G = tb.GreenFunction(8, H, lo, hi)
    got = G.scaled_HE.to_csc()
    # the oracle rescales the device's own values, so the rescale itself is checked bit for bit
    want = orc.rescale_csc(len(cp) - 1, cp, ri, v, G.a, G.b)
    for x, y in zip(got, want):
        assert np.array_equal(x, y)


def test_builder_random_vacancies_device_compaction(gpu):
    """remove_atoms_random on both sublattices of a 256 x 192 honeycomb: the
    device prefix-sum compaction gives the oracle's index_c build bit-exact."""
    tb = gpu
    cell = tb.Honeycomb().add_hopping("A", 1, -2.7)
    X = tb.PartialLattice(cell, (256, 192))
    X.remove_atoms_random("A", 2500, seed=3)
    X.remove_atoms_random("B", 1800, seed=4)
    removed = X.removed_sites()
    assert int(removed.sum()) == 4300
    H = X.get_Hamiltonian_sparse(float)
    spec = spec_from(cell, (256, 192), mode=orc.MODE_SPARSE, is_complex=False, removed=removed.astype(np.int32))
    _assert_same(H, orc.build_csc(spec))
    n_kept = X.get_kept_number()
    cp = H.to_csc()[0]
    assert n_kept == 2 * 256 * 192 - 4300 and cp[n_kept] == cp[-1]


def test_builder_every_site_removed(gpu):
    """remove_atoms_random of every cell on both sublattices: the open-BC
    Hamiltonian keeps its total_number shape with no entries (the reference's
    index_c is all -1), as the oracle builds it."""
    tb = gpu
    cell = tb.Honeycomb().add_hopping("A", 1, 1.0)
    X = tb.PartialLattice(cell, (5, 4))
    X.remove_atoms_random("A", 20, seed=1)
    X.remove_atoms_random("B", 20, seed=2)
    assert X.get_kept_number() == 0
    H = X.get_Hamiltonian_sparse(float)
    ref = orc.build_csc(spec_from(cell, (5, 4), mode=orc.MODE_SPARSE, is_complex=False,
                                  removed=X.removed_sites().astype(np.int32)))
    _assert_same(H, ref)
    assert H.to_csc()[0][-1] == 0


def _scipy_csc(M):
    import scipy.sparse as sp
    cp, ri, v = M.to_csc()
    n = len(cp) - 1
    return sp.csc_matrix((v, ri, cp), shape=(n, n))


def test_bond_velocity_matches_commutator_without_wrap(gpu):
    """Open boundaries: the bond-displacement velocity (scale 1/a) equals
    X H~ - H~ X entry by entry (complex gauge, disorder, two-atom cell)."""
    tb = gpu
    X = tb.PartialLattice(tb.Honeycomb().add_hopping("A", 1, -2.7), (9, 7))
    X.set_gauge_linear(*landau_gauge(0.05))
    X.set_scalar_disorder(0.8, 2)
    H = X.get_Hamiltonian_sparse(complex)
    G = tb.GreenFunction(8, H, -8.6, 8.6)
    for axis in (0, 1):
        comm = _scipy_csc(tb.commutator(G.scaled_HE, X.op_position(axis))).toarray()
        bond = _scipy_csc(X.op_velocity_bond(axis, scalar=complex, scale=1.0 / G.a, mode="sparse")).toarray()
        assert np.max(np.abs(comm - bond)) <= 1e-14 * np.max(np.abs(comm))


def test_bond_velocity_periodic_is_translation_invariant(gpu):
    """Periodic square lattice: every bond carries +-t (scale 1) along its own
    displacement, including the wrapping bonds where [X, H] jumps by L - 1."""
    tb = gpu
    X = tb.PartialLattice(tb.Square().add_hopping("A", 1, 1.0), (6, 5))
    V = _scipy_csc(X.op_velocity_bond(0, extend=[1, 1], scalar=float)).toarray()
    assert set(np.unique(np.round(V, 12))) == {-1.0, 0.0, 1.0}
    assert np.allclose(V, -V.T)
    assert np.allclose(V.sum(axis=0), 0.0)
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1, 1], float)
    comm = _scipy_csc(tb.commutator(H, X.op_position(0))).toarray()
    assert np.max(np.abs(comm)) == pytest.approx(5.0)         # the wrap: x jumps by L - 1
