"""Lattices of the serving workload: square / honeycomb / Kagome / Lieb (2D)
and FCC (3D), nearest-neighbour t = 1.0 from every atom, uniform on-site
disorder W, symmetric bounds z|t| + W/2 + margin."""
ATOMS = {"square": ("A",), "honeycomb": ("A", "B"), "kagome": ("A", "B", "C"), "lieb": ("A", "B", "C"),
         "fcc": ("A",)}
COORD = {"square": 4, "honeycomb": 3, "kagome": 4, "lieb": 4, "fcc": 12}


def cell(tb, kind):
    c = {"square": tb.Square, "honeycomb": tb.Honeycomb, "kagome": tb.Kagome, "lieb": tb.Lieb, "fcc": tb.FCC}[kind]()
    for a in ATOMS[kind]:
        c.add_hopping(a, 1, 1.0)      # h.c. duplicates of earlier atoms are skipped
    return c


def lattice(tb, kind, L, W=0.0, seed=0, cells=None):
    c = cells[kind] if cells is not None else cell(tb, kind)
    span = (L, L, L) if kind == "fcc" else (L, L)
    X = tb.PartialLattice(c, span)
    if W > 0:
        X.set_scalar_disorder(W, seed)
    return X


def bounds(kind, W):
    e = COORD[kind] * 1.0 + W / 2 + 0.05
    return -e, e
