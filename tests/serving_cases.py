"""Lattices of the serving workload: square / honeycomb / Kagome / Lieb (2D)
and FCC (3D), nearest-neighbour t = 1.0 from every atom, uniform on-site
disorder W, symmetric bounds z|t| + W/2 + margin."""


def cell(tb, kind):
    from tight_binding_gb300.serving import model_cell
    return model_cell(kind)


def lattice(tb, kind, L, W=0.0, seed=0, cells=None):
    c = cells[kind] if cells is not None else cell(tb, kind)
    span = (L, L, L) if kind == "fcc" else (L, L)
    X = tb.PartialLattice(c, span)
    if W > 0:
        X.set_scalar_disorder(W, seed)
    return X


def bounds(kind, W):
    from tight_binding_gb300.serving import model_bounds
    return model_bounds(kind, W)
