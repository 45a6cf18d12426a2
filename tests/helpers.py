"""Shared test helpers: the same seeded inputs for the oracle and the GPU path."""
from __future__ import annotations

import numpy as np

import oracle as orc


def spec_from(cell, span, mode=orc.MODE_SPARSE, is_complex=True, extend=None, gauge_linear=None,
              gauge_site=None, scalar_site=None, removed=None):
    """Oracle lattice spec carrying the library cell's canonical hopping table."""
    bases, pos = cell.geometry()
    f, t, v, tt = cell.hoppings()
    return orc.LatticeSpec(cell.dim, list(span), bases, pos, f, t, v, tt, mode=mode, is_complex=is_complex,
                           extend=extend, gauge_linear=gauge_linear, gauge_site=gauge_site,
                           scalar_site=scalar_site, removed=removed)


def with_onsite_zeros(cell):
    """The cell as set_scalar_field leaves it: a zero on-site hopping appended for
    every atom that has none (TB/lattice.h:499-504)."""
    c = cell.copy()
    f, t, v, _ = c.hoppings()
    have = {int(a) for a, b, w in zip(f, t, v) if a == b and not np.any(w)}
    for i, name in enumerate(c.names):
        if i not in have:
            c.add_hopping(name, 0, 0.0)
    return c


def rel_err(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def landau_gauge(B):
    """A(r) = (0, B x, 0) as the linear form G r + c."""
    G = np.zeros((3, 3))
    G[1, 0] = B
    return G, np.zeros(3)


def plane_wave_moments_square(L, t, a, M):
    """Exact Tr T_n(H/a) for the L x L periodic square lattice with NN hopping t."""
    k = 2 * np.pi * np.arange(L) / L
    e = (2 * t * (np.cos(k)[:, None] + np.cos(k)[None, :])).reshape(-1) / a
    th = np.arccos(np.clip(e, -1, 1))
    n = np.arange(M)
    return np.cos(np.outer(n, th)).sum(axis=1)
