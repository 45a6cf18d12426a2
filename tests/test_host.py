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
