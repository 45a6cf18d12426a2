"""Host-side checks that need no GPU: the C ABI library loads and exports every
symbol include/tbk.h declares; the unit-cell model follows the reference's rules."""
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def _declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(tbk_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol(tb):
    from tight_binding_gb300 import capi

    L = capi.lib()
    declared = _declared_symbols()
    assert len(declared) > 30
    missing = [n for n in declared if not hasattr(L, n)]
    assert not missing, missing
    # the ctypes table covers the header too
    assert not (set(declared) - set(capi.SIGNATURES)), set(declared) - set(capi.SIGNATURES)


def test_version_and_device_count_without_gpu(tb):
    from tight_binding_gb300 import capi

    assert capi.lib().tbk_version() >= 10000
    assert tb.device_count() >= 0


def test_unit_cell_rules(tb):
    sq = tb.Square()
    sq.add_hopping("A", 1, 1.0)
    f, t, v, tt = sq.hoppings()
    assert len(f) == 2 and np.all(f >= t)            # +-x, +-y collapse to one stored hop each
    sq.add_hopping("A", "A", (1, 0), 2.0)            # already exists (as itself or its h.c.)
    assert sq.last_warnings() == 1 and sq.info()[2] == 2
    sq.add_hopping("A", 0, 1.0j)                     # on-site must be real
    assert sq.last_warnings() == 1 and sq.info()[2] == 2
    sq.add_hopping("A", 0, 0.5)
    assert sq.info()[2] == 3


def test_canonical_from_ge_to(tb):
    h = tb.Honeycomb()
    h.add_hopping("A", "B", (0, 0), 1.0 + 2.0j)     # from < to: stored as (B, A, 0) with conj(t)
    f, t, v, tt = h.hoppings()
    assert (f[0], t[0]) == (1, 0) and tt[0] == 1.0 - 2.0j


def test_model_shell_counts(tb):
    assert tb.graphene().info()[2] == 3
    fcc = tb.FCC().add_hopping("A", 1, 1.0)
    assert fcc.info()[2] == 6                        # 12 neighbours, half stored
    k = tb.Kagome()
    for a in "ABC":
        k.add_hopping(a, 1, 1.0)
    assert k.info()[2] == 6                          # 6 distinct NN bonds per cell
    lieb = tb.Lieb()
    lieb.add_hopping("A", 1, 1.0)
    assert lieb.info()[2] == 4


def test_errors_are_reported(tb):
    with pytest.raises(tb.TbkError):
        tb.UnitCell([(1, 0, 0)], [("A", (0, 0, 0)), ("A", (0.5, 0, 0))])
    with pytest.raises(tb.TbkError):
        tb.UnitCell([(0, 0, 0)], [("A", (0, 0, 0))])
    c = tb.Square()
    with pytest.raises(tb.TbkError):
        c.add_hopping("Z", 1, 1.0)
    with pytest.raises(ValueError):
        tb.PartialLattice(c, (4,))


def test_lattice_index_scheme(tb):
    X = tb.PartialLattice(tb.Honeycomb(), (3, 5))
    assert X.get_total_number() == 30
    assert X.index_bare((0, 0), 1) == 1
    assert X.index_bare((0, 1), 0) == 2
    assert X.index_bare((1, 0), 0) == 10
    pos = X.site_positions()
    assert pos.shape == (30, 3)
    assert np.allclose(pos[X.index_bare((1, 2), 1)], np.array([1.5, -np.sqrt(3) / 2, 0]) * 1
                       + np.array([1.5, np.sqrt(3) / 2, 0]) * 2 + np.array([1, 0, 0]))


def test_remove_atoms_host_rules(tb):
    """remove_atoms / remove_atoms_random (TB/lattice.h:389-418) on the host:
    index_bare placement, seeded distinct draws on one sublattice, the
    reference's error texts, and index_c (TB/lattice.h:446-457)."""
    X = tb.PartialLattice(tb.Honeycomb(), (6, 5))
    X.remove_atoms("B", [(0, 0), (2, 3), (5, 4)])
    r = X.removed_sites()
    assert set(np.flatnonzero(r)) == {X.index_bare((0, 0), 1), X.index_bare((2, 3), 1), X.index_bare((5, 4), 1)}
    assert X.get_kept_number() == 57
    c = X.index_comp()
    assert c[X.index_bare((0, 0), 1)] == -1 and c[0] == 0 and c[2] == 1 and c.max() == 56
    Y = tb.PartialLattice(tb.Honeycomb(), (64, 48))
    Y.remove_atoms_random("A", 700, seed=5)
    m = Y.removed_sites()
    idx = np.flatnonzero(m)
    assert len(idx) == 700 and np.all(idx % 2 == 0)
    Z = tb.PartialLattice(tb.Honeycomb(), (64, 48))
    Z.remove_atoms_random("A", 700, seed=5)
    assert np.array_equal(Z.removed_sites(), m)
    Z.remove_sites(np.zeros(Z.get_total_number(), np.uint8))
    Z.remove_atoms_random("A", 700, seed=6)
    assert not np.array_equal(Z.removed_sites(), m)
    # all cells: every A removed
    W = tb.PartialLattice(tb.Honeycomb(), (4, 4))
    W.remove_atoms_random("B", 16, seed=1)
    assert np.array_equal(np.flatnonzero(W.removed_sites()), np.arange(1, 32, 2))
    with pytest.raises(tb.TbkError, match="does not exist in the unit cell"):
        X.remove_atoms("Q", [(0, 0)])
    with pytest.raises(tb.TbkError, match="larger than the total number"):
        W.remove_atoms_random("A", 17)
    with pytest.raises(tb.TbkError, match="outside the lattice"):
        X.remove_atoms("A", [(6, 0)])


def test_expansion_coefficients_host(tb):
    """Host coefficient helpers of the vector expansions: the sawtooth delta
    projection (TB/snippets.h:194-202) against the oracle's loop, and
    exp(-i H t) against scipy's Bessel J."""
    import oracle as orc
    special = pytest.importorskip("scipy.special")
    for e, N in ((0.3, 10), (-0.97, 200), (0.0, 1)):
        assert np.allclose(tb.delta_coefficients(e, N), orc.delta_coefficients(e, N), rtol=1e-13, atol=1e-13)
    for a, b, t in ((2.0, 0.3, 5.0), (4.6, -0.1, 0.0), (8.6, 0.0, -3.0)):
        c = tb.evolution_coefficients(a, b, t)
        k = np.arange(len(c))
        ref = np.exp(-1j * b * t) * (2.0 - (k == 0)) * (-1j) ** k * special.jv(k, a * t)
        assert np.max(np.abs(c - ref)) <= 1e-14
        assert abs(special.jv(len(c), a * t)) < 1e-15
    assert tb.evolution_terms(1.0, 100.0) > 100


def test_new_entry_points_reject_bad_arguments_without_gpu(tb):
    """Argument checks of the spectral-range, expansion and moment-file entry
    points run before any device work (CPU-only)."""
    import ctypes as C
    from tight_binding_gb300 import capi
    L = capi.lib()
    d = C.c_double()
    assert L.tbk_spectral_range(None, 10, 0, C.byref(d), C.byref(d), None, None, None) == capi.TBK_ERR_INVALID
    assert b"null argument" in L.tbk_last_error()
    assert L.tbk_cheb_expand(None, 4, None, 1, None, None, 0, None) == capi.TBK_ERR_INVALID
    assert L.tbk_cheb_coef_delta(0.1, -1, None) == capi.TBK_ERR_INVALID
    assert L.tbk_cheb_coef_evolution(1.0, 0.0, 1.0, 0, None) == capi.TBK_ERR_INVALID
    k = C.c_int32()
    assert L.tbk_cheb_evolution_terms(1.0, 1.0, 0.0, C.byref(k)) == capi.TBK_ERR_INVALID
    assert L.tbk_moments_save(None, None, None) == capi.TBK_ERR_INVALID


def test_expn_coef_alpha_seq_host(tb):
    """expn_coef_alpha_seq (TB/numerical.h:304-316) against the oracle's, and
    the resolvent identity 1/(z - x) = sum_k alpha_k(z) T_k(x) off the cut."""
    import oracle as orc
    for z in (0.3 + 0.01j, -0.9 + 1e-3j, 1.7 - 0.2j, 0.0 + 0.5j):
        a = tb.expn_coef_alpha_seq(z, 64)
        assert np.allclose(a, orc.expn_coef_alpha_seq(z, 64), rtol=1e-13, atol=1e-15)
    z, x = 0.2 + 0.4j, 0.35
    a = tb.expn_coef_alpha_seq(z, 400)
    T = np.cos(np.arange(400) * np.arccos(x))
    assert abs(np.sum(a * T) - 1.0 / (z - x)) <= 1e-10
