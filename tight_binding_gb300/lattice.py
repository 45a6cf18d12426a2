"""Python mirror of the reference's model API, backed by libtbk.

    UnitCell            TB/unit_cell.h:65-156   (ctor, add_hopping overloads)
    PartialLattice      TB/lattice.h:22-103     (index scheme, builders, x, v)
    SparseMatrix        device-resident CSC (Eigen::SparseMatrix<Scalar> layout)
    models              TB/models.h:5-151

Matrices stay on the GPU; ``SparseMatrix.to_csc()`` / ``to_scipy()`` copy them
to the host for inspection.
"""
from __future__ import annotations

import ctypes as C
from typing import Callable, Sequence

import numpy as np

from . import capi
from .capi import check, lib

Complex = complex


class SparseMatrix:
    """Device-resident sparse matrix (CSC + sliced-ELL for the recursion)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        rows, cols, cplx = C.c_int32(), C.c_int32(), C.c_int32()
        nnz = C.c_int64()
        check(lib().tbk_sparse_info(self._h, C.byref(rows), C.byref(cols), C.byref(nnz), C.byref(cplx)))
        self.shape = (rows.value, cols.value)
        self.nnz = nnz.value
        self.is_complex = bool(cplx.value)

    @classmethod
    def from_csc(cls, n_rows: int, n_cols: int, col_ptr, row_idx, values, is_complex: bool | None = None):
        cp = np.ascontiguousarray(col_ptr, dtype=np.int32)
        ri = np.ascontiguousarray(row_idx, dtype=np.int32)
        v = np.asarray(values)
        if is_complex is None:
            is_complex = np.iscomplexobj(v)
        v = np.ascontiguousarray(v, dtype=np.complex128 if is_complex else np.float64)
        h = C.c_void_p()
        check(lib().tbk_sparse_from_csc(C.byref(h), n_rows, n_cols, len(ri), capi.ptr(cp), capi.ptr(ri),
                                        capi.ptr(v), int(is_complex), 0, None))
        return cls(h.value)

    @classmethod
    def from_scipy(cls, M):
        M = M.tocsc()
        M.sort_indices()
        return cls.from_csc(M.shape[0], M.shape[1], M.indptr, M.indices, M.data, np.iscomplexobj(M.data))

    @property
    def handle(self):
        return self._h

    def to_csc(self):
        cp = np.zeros(self.shape[1] + 1, dtype=np.int32)
        ri = np.zeros(max(self.nnz, 1), dtype=np.int32)
        v = np.zeros(max(self.nnz, 1), dtype=np.complex128 if self.is_complex else np.float64)
        check(lib().tbk_sparse_download(self._h, capi.ptr(cp), capi.ptr(ri), capi.ptr(v), None))
        return cp, ri[: self.nnz], v[: self.nnz]

    def to_scipy(self):
        import scipy.sparse as sp

        cp, ri, v = self.to_csc()
        return sp.csc_matrix((v, ri, cp), shape=self.shape)

    def rows(self) -> int:
        return self.shape[0]

    def row_classes(self) -> int:
        """Number of row classes the recursion uses for this matrix (0: ELL form)."""
        n = C.c_int32()
        check(lib().tbk_sparse_row_classes(self._h, C.byref(n), None))
        return n.value

    def nonZeros(self) -> int:  # Eigen spelling
        return self.nnz

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().tbk_sparse_destroy(h)
            except Exception:
                pass
            self._h = C.c_void_p()


class UnitCell:
    """UnitCell<Dim>, TB/unit_cell.h:65-156."""

    Intra_Cell = None  # set per instance (dimension dependent)

    def __init__(self, lattice_vectors: Sequence[Sequence[float]], atoms: Sequence[tuple[str, Sequence[float]]]):
        lv = np.zeros((len(lattice_vectors), 3))
        for i, v in enumerate(lattice_vectors):
            lv[i, : len(v)] = v
        names = [a[0] for a in atoms]
        pos = np.zeros((len(atoms), 3))
        for i, a in enumerate(atoms):
            pos[i, : len(a[1])] = a[1]
        arr = (C.c_char_p * len(names))(*[n.encode() for n in names])
        h = C.c_void_p()
        check(lib().tbk_cell_create(C.byref(h), len(lattice_vectors), capi.as_dp(lv), len(atoms), arr, capi.as_dp(pos)))
        self._h = h
        self.names = list(names)
        self.dim = len(lattice_vectors)
        self.Intra_Cell = (0,) * self.dim
        self.Left_NN = (-1,) + (0,) * (self.dim - 1)
        self.Right_NN = (1,) + (0,) * (self.dim - 1)

    def copy(self) -> "UnitCell":
        new = object.__new__(UnitCell)
        h = C.c_void_p()
        check(lib().tbk_cell_copy(C.byref(h), self._h))
        new._h = h
        new.names = list(self.names)
        new.dim = self.dim
        new.Intra_Cell, new.Left_NN, new.Right_NN = self.Intra_Cell, self.Left_NN, self.Right_NN
        return new

    def add_hopping(self, from_: str, to_or_nn, lattice_vector_or_t=None, t=None) -> "UnitCell":
        """add_hopping(from, to, lattice_vector, t) or add_hopping(from, n_NN, t)."""
        if isinstance(to_or_nn, str):
            v = np.zeros(3, dtype=np.int32)
            v[: self.dim] = lattice_vector_or_t
            tt = complex(t)
            check(lib().tbk_cell_add_hopping(self._h, from_.encode(), to_or_nn.encode(), capi.as_i32p(v), tt.real, tt.imag))
        else:
            tt = complex(lattice_vector_or_t)
            check(lib().tbk_cell_add_hopping_nn(self._h, from_.encode(), int(to_or_nn), tt.real, tt.imag))
        return self

    def last_warnings(self) -> int:
        n = C.c_int32()
        check(lib().tbk_cell_last_warnings(self._h, C.byref(n)))
        return n.value

    def get_atom_number(self) -> int:
        return self.info()[1]

    def get_atom_index(self, name: str) -> int:
        i = C.c_int32()
        check(lib().tbk_cell_atom_index(self._h, name.encode(), C.byref(i)))
        return i.value

    def info(self):
        d, a, h = C.c_int32(), C.c_int32(), C.c_int32()
        check(lib().tbk_cell_info(self._h, C.byref(d), C.byref(a), C.byref(h)))
        return d.value, a.value, h.value

    def hoppings(self):
        """Canonical table: (from, to, lattice vector (n,3), t complex)."""
        _, _, n = self.info()
        f = np.zeros(max(n, 1), np.int32)
        t = np.zeros(max(n, 1), np.int32)
        v = np.zeros((max(n, 1), 3), np.int32)
        tv = np.zeros((max(n, 1), 2))
        check(lib().tbk_cell_get_hoppings(self._h, capi.as_i32p(f), capi.as_i32p(t), capi.as_i32p(v), capi.as_dp(tv)))
        return f[:n], t[:n], v[:n], tv[:n, 0] + 1j * tv[:n, 1]

    def geometry(self):
        d, a, _ = self.info()
        bases = np.zeros(3 * d)
        pos = np.zeros((a, 3))
        check(lib().tbk_cell_get_geometry(self._h, capi.as_dp(bases), capi.as_dp(pos)))
        return bases.reshape(d, 3).T.copy(), pos   # bases: 3 x dim (columns = lattice vectors)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().tbk_cell_destroy(h)
            except Exception:
                pass
            self._h = C.c_void_p()


class PartialLattice:
    """PartialLattice<Dim>, TB/lattice.h:22-103."""

    def __init__(self, cell: UnitCell, span_size: Sequence[int]):
        self.dim = cell.dim
        if len(span_size) != self.dim:
            raise ValueError("span must have one entry per lattice dimension")
        sp = np.zeros(3, dtype=np.int32)
        sp[: self.dim] = span_size
        h = C.c_void_p()
        check(lib().tbk_lattice_create(C.byref(h), cell._h, capi.as_i32p(sp)))
        self._h = h
        self.span = tuple(int(s) for s in span_size)
        self._bases, self._pos = cell.geometry()
        self.n_atoms = self._pos.shape[0]

    # -- sizes / index scheme (TB/lattice.h:27-35, 51-52)
    def get_total_number(self) -> int:
        n = C.c_int64()
        check(lib().tbk_lattice_total_number(self._h, C.byref(n)))
        return n.value

    def get_cell_number(self) -> int:
        return int(np.prod(self.span))

    def index_bare(self, i_v: Sequence[int], i_a: int) -> int:
        s = [0] * self.dim
        s[-1] = self.n_atoms
        for i in range(self.dim - 2, -1, -1):
            s[i] = s[i + 1] * self.span[i + 1]
        return int(sum(a * b for a, b in zip(i_v, s)) + i_a)

    def site_positions(self) -> np.ndarray:
        """Position of every bare site (N x 3), atom_position(a, i_v)."""
        grids = np.meshgrid(*[np.arange(s) for s in self.span], indexing="ij")
        cells = np.stack([g.reshape(-1) for g in grids], axis=1).astype(np.float64)   # row-major
        disp = cells @ self._bases.T                                                      # (cells, 3)
        return (disp[:, None, :] + self._pos[None, :, :]).reshape(-1, 3)

    # -- fields (TB/lattice.h:73-74, 495-505)
    def set_gauge_linear(self, G, c=(0.0, 0.0, 0.0)) -> None:
        G = np.ascontiguousarray(G, dtype=np.float64).reshape(3, 3)
        cc = np.ascontiguousarray(c, dtype=np.float64)
        check(lib().tbk_lattice_set_gauge_linear(self._h, capi.as_dp(G), capi.as_dp(cc)))

    def set_gauge_field(self, f: Callable[[np.ndarray], np.ndarray]) -> None:
        """gauge_field = f; f maps site positions (N x 3) to A (N x 3)."""
        A = np.ascontiguousarray(f(self.site_positions()), dtype=np.float64)
        check(lib().tbk_lattice_set_gauge_sites(self._h, capi.as_dp(A)))

    def clear_gauge_field(self) -> None:
        check(lib().tbk_lattice_clear_gauge(self._h))

    def set_scalar_field(self, f: Callable[[np.ndarray], np.ndarray]) -> None:
        """set_scalar_field(f); f maps site positions (N x 3) to V (N)."""
        V = np.ascontiguousarray(f(self.site_positions()), dtype=np.float64)
        check(lib().tbk_lattice_set_scalar_sites(self._h, capi.as_dp(V)))

    def set_scalar_values(self, V) -> None:
        V = np.ascontiguousarray(V, dtype=np.float64)
        check(lib().tbk_lattice_set_scalar_sites(self._h, capi.as_dp(V)))

    def set_scalar_disorder(self, W: float, seed: int) -> None:
        """Anderson disorder V = W (u - 1/2), generated on the device."""
        check(lib().tbk_lattice_set_scalar_disorder(self._h, float(W), int(seed)))

    # -- vacancies (TB/lattice.h:389-464)
    def remove_sites(self, removed) -> None:
        """Replace the removal flags with `removed` (N bare sites, nonzero = removed)."""
        r = np.ascontiguousarray(removed, dtype=np.uint8)
        check(lib().tbk_lattice_set_removed(self._h, r.ctypes.data_as(C.POINTER(C.c_uint8))))

    def remove_atoms(self, atom_name: str, cells) -> None:
        """remove_atoms(atom_name, i), TB/lattice.h:389-402: the atom of every listed cell."""
        c = np.ascontiguousarray(np.asarray(cells, dtype=np.int32).reshape(-1, self.dim))
        check(lib().tbk_lattice_remove_atoms(self._h, atom_name.encode(), capi.as_i32p(c), c.shape[0]))

    def remove_atoms_random(self, atom_name: str, n: int, seed: int = 0) -> None:
        """remove_atoms_random(atom_name, n), TB/lattice.h:404-418, from a seeded
        stream (the reference draws from std::random_device)."""
        check(lib().tbk_lattice_remove_atoms_random(self._h, atom_name.encode(), int(n), int(seed)))

    def removed_sites(self) -> np.ndarray:
        r = np.zeros(self.get_total_number(), dtype=np.uint8)
        check(lib().tbk_lattice_get_removed(self._h, r.ctypes.data_as(C.POINTER(C.c_uint8))))
        return r

    def index_comp(self) -> np.ndarray:
        """index_c, TB/lattice.h:446-457: bare -> compressed index, -1 where removed."""
        keep = self.removed_sites() == 0
        c = np.full(keep.shape, -1, dtype=np.int32)
        c[keep] = np.arange(int(keep.sum()), dtype=np.int32)
        return c

    def get_kept_number(self) -> int:
        n = C.c_int64()
        check(lib().tbk_lattice_kept_number(self._h, C.byref(n)))
        return n.value

    # -- builders (TB/lattice.h:216-377)
    def _build(self, mode: int, extend, scalar) -> SparseMatrix:
        ext = np.zeros(3, dtype=np.int32)
        if extend is not None:
            ext[: self.dim] = extend
        h = C.c_void_p()
        check(lib().tbk_build_hamiltonian(C.byref(h), self._h, mode, capi.as_i32p(ext), int(scalar is complex), None))
        return SparseMatrix(h.value)

    def get_Hamiltonian_sparse(self, scalar=complex) -> SparseMatrix:
        return self._build(capi.BUILD_SPARSE, None, scalar)

    def get_Hamiltonian_periodic_extend_bare_sparse(self, extend, scalar=complex) -> SparseMatrix:
        return self._build(capi.BUILD_PERIODIC_BARE, extend, scalar)

    def get_Hamiltonian_bare_sparse(self, scalar=complex) -> SparseMatrix:
        return self._build(capi.BUILD_BARE, None, scalar)

    def op_position(self, axis: int) -> SparseMatrix:
        h = C.c_void_p()
        check(lib().tbk_build_position(C.byref(h), self._h, int(axis), None))
        return SparseMatrix(h.value)

    def op_velocity_bond(self, axis: int, extend=None, scalar=complex, scale: float = 1.0,
                         mode: str = "periodic") -> SparseMatrix:
        """Bond-displacement velocity along `axis`: the Hamiltonian of `mode`
        ("periodic" with `extend`, "sparse" or "bare") with each hopping entry
        (i, j) times scale * (r_i - r_j) along the bond itself.  scale = 1/a
        gives [X, H~] on every bond that does not cross a periodic boundary
        (and the short displacement on those that do)."""
        ext = np.zeros(3, dtype=np.int32)
        if extend is not None:
            ext[: self.dim] = extend
        m = {"periodic": capi.BUILD_PERIODIC_BARE, "sparse": capi.BUILD_SPARSE, "bare": capi.BUILD_BARE}[mode]
        h = C.c_void_p()
        check(lib().tbk_build_velocity_bond(C.byref(h), self._h, m, capi.as_i32p(ext), int(scalar is complex),
                                            int(axis), float(scale), None))
        return SparseMatrix(h.value)

    def op_velocity(self, axis: int) -> SparseMatrix:
        """X H - H X with the real open-boundary H (no factor i), TB/lattice.h:338-345."""
        return commutator(self.get_Hamiltonian_sparse(float), self.op_position(axis))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().tbk_lattice_destroy(h)
            except Exception:
                pass
            self._h = C.c_void_p()


def commutator(H: SparseMatrix, X: SparseMatrix) -> SparseMatrix:
    """X H - H X for a diagonal X (values x_i h - h x_j on the pattern of H)."""
    h = C.c_void_p()
    check(lib().tbk_sparse_commutator(C.byref(h), H.handle, X.handle, None))
    return SparseMatrix(h.value)


# --------------------------------------------------------------------- models
# TB/models.h:5-151
def Honeycomb() -> UnitCell:
    s3 = np.sqrt(3.0)
    return UnitCell([(1.5, -s3 / 2, 0), (1.5, s3 / 2, 0)], [("A", (0, 0, 0)), ("B", (1, 0, 0))])


def Square() -> UnitCell:
    return UnitCell([(1, 0, 0), (0, 1, 0)], [("A", (0, 0, 0))])


def Chain() -> UnitCell:
    return UnitCell([(1, 0, 0)], [("A", (0, 0, 0))])


def Lieb() -> UnitCell:
    return UnitCell([(1, 0, 0), (0, 1, 0)], [("A", (0, 0, 0)), ("B", (0.5, 0, 0)), ("C", (0, 0.5, 0))])


def Kagome() -> UnitCell:
    s3 = np.sqrt(3.0)
    return UnitCell([(1, 0, 0), (0.5, s3 / 2, 0)], [("A", (0, 0, 0)), ("B", (0.5, 0, 0)), ("C", (0.25, s3 / 4, 0))])


def FCC() -> UnitCell:
    return UnitCell([(0.5, 0.5, 0), (0.5, 0, 0.5), (0, 0.5, 0.5)], [("A", (0, 0, 0))])


def Cubic() -> UnitCell:
    return UnitCell([(1, 0, 0), (0, 1, 0), (0, 0, 1)], [("A", (0, 0, 0))])


def stub_1d_X() -> UnitCell:
    return UnitCell([(1, 0, 0)], [("A", (0, 0, 0)), ("C", (0.5, 0, 0)), ("B", (0, 0.6, 0))])


def sawtooth_chain_X() -> UnitCell:
    return UnitCell([(1, 0, 0)], [("A", (0, 0, 0)), ("B", (0, 1, 0))])


def graphene() -> UnitCell:
    return Honeycomb().add_hopping("A", 1, 1.0)


def TI_sp() -> UnitCell:
    p = UnitCell([(1, 0, 0), (0, 1, 0)], [("s", (0, 0, 0)), ("p", (0, 0, 0))])
    ep, t_ss, t_sp = 0.6, 0.4, 0.2
    es, t_pp = -ep, -t_ss
    p.add_hopping("s", "s", (0, 0), es)
    p.add_hopping("p", "p", (0, 0), ep)
    p.add_hopping("s", "s", (1, 0), t_ss)
    p.add_hopping("s", "s", (0, 1), t_ss)
    p.add_hopping("p", "p", (1, 0), t_pp)
    p.add_hopping("p", "p", (0, 1), t_pp)
    p.add_hopping("s", "p", (1, 0), 1.0 * t_sp)
    p.add_hopping("s", "p", (0, 1), 1j * t_sp)
    p.add_hopping("s", "p", (-1, 0), -1.0 * t_sp)
    p.add_hopping("s", "p", (0, -1), -1j * t_sp)
    return p


def stub_1d_p(t: float, t_: float) -> UnitCell:
    p = stub_1d_X()
    p.add_hopping("A", "C", (0,), t)
    p.add_hopping("A", "C", (-1,), t)
    p.add_hopping("A", "B", (0,), t_)
    return p


def sawtooth_chain_p(t: float, t_: float) -> UnitCell:
    p = sawtooth_chain_X()
    p.add_hopping("A", "A", (1,), t)
    p.add_hopping("A", "B", (0,), t_)
    p.add_hopping("B", "A", (1,), t_)
    return p
