"""Kernel-polynomial (Chebyshev) API, backed by libtbk.

    Cheb_first_kind_seq_braket      TB/numerics_cuda.cuh:8-14 (drop-in, both overloads)
    bases_of_uniform_ampl_with_random_phases   TB/numerical.h:120-122 (seeded)
    kernel_seq / kernels            TB/numerical.h:393-447
    GreenFunction, GreenFunctionImag   TB/lattice.h:532-652
    density_of_states_seq / _function  TB/functions.h:5-32
    KpmSolver                       resident plan (H~ and recursion state on the GPU)
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import capi
from .capi import check, lib
from .lattice import PartialLattice, SparseMatrix

PREC = {"fp64": capi.PREC_FP64, "mixed": capi.PREC_MIXED, "dd": capi.PREC_DD}


def _prec(p) -> int:
    if isinstance(p, str):
        return PREC[p]
    return int(p)


def bases_of_uniform_ampl_with_random_phases(n: int, m: int, seed: int = 0) -> np.ndarray:
    """N x R column-major complex128 block exp(2 pi i u)/sqrt(N) (seeded)."""
    out = np.zeros((n, m), dtype=np.complex128, order="F")
    check(lib().tbk_random_phase_kets(n, m, int(seed), capi.ptr(out)))
    return out


def _block(a: np.ndarray, n: int) -> np.ndarray:
    a = np.asarray(a)
    if a.ndim == 1:
        a = a.reshape(n, 1)
    return np.asfortranarray(a, dtype=np.complex128)


def Cheb_first_kind_seq_braket(M, n: int, bras: np.ndarray, kets: np.ndarray, precision="fp64",
                               doubling: bool = False) -> np.ndarray:
    """Drop-in for cuda::Cheb_first_kind_seq_braket (TB/numerics_cuda.cuh:10-13).

    M: scipy sparse matrix or (n_rows, col_ptr, row_idx, values).  Returns
    mu[k] = Re tr(bras^dagger T_k(M) kets), k < n; n < 2 raises (the reference
    returns an empty vector).  ``doubling`` requires ``bras is kets``.
    """
    if isinstance(M, tuple):
        n_rows, cp, ri, v = M
    else:
        Mc = M.tocsc()
        Mc.sort_indices()
        n_rows, cp, ri, v = Mc.shape[0], Mc.indptr, Mc.indices, Mc.data
    cp = np.ascontiguousarray(cp, dtype=np.int32)
    ri = np.ascontiguousarray(ri, dtype=np.int32)
    cplx = np.iscomplexobj(v)
    v = np.ascontiguousarray(v, dtype=np.complex128 if cplx else np.float64)
    same = bras is kets
    K = _block(kets, n_rows)
    B = K if same else _block(bras, n_rows)
    flags = _prec(precision) | (capi.FLAG_DOUBLING if doubling else 0)
    if doubling and not same:
        raise ValueError("doubling needs bras is kets")
    mu = np.zeros(max(n, 1))
    fn = lib().tbk_cheb_braket_complex if cplx else lib().tbk_cheb_braket_real
    check(fn(n_rows, len(ri), capi.ptr(cp), capi.ptr(ri), capi.ptr(v), n, capi.ptr(B), capi.ptr(K), K.shape[1],
             flags, capi.ptr(mu)))
    return mu[:n]


class KpmSolver:
    """Resident KPM plan: H~ stays on the device, work blocks are reused."""

    def __init__(self, Ht: SparseMatrix, R: int, precision="mixed", doubling: bool = True, flags: int = 0):
        self.Ht = Ht
        self.R = R
        self.flags = _prec(precision) | (capi.FLAG_DOUBLING if doubling else 0) | flags
        h = C.c_void_p()
        check(lib().tbk_kpm_create(C.byref(h), Ht.handle, R, self.flags))
        self._h = h

    def run(self, n_mom: int, bras: np.ndarray, kets: np.ndarray, stream=None) -> np.ndarray:
        mu = np.zeros(n_mom)
        n = self.Ht.shape[0]
        K = _block(kets, n)
        B = K if bras is kets else _block(bras, n)
        check(lib().tbk_kpm_run(self._h, n_mom, capi.ptr(B), capi.ptr(K), capi.ptr(mu), stream))
        return mu

    def run_device(self, n_mom: int, bras_ptr: int, kets_ptr: int, mu_ptr: int, stream=None) -> None:
        check(lib().tbk_kpm_run(self._h, n_mom, bras_ptr, kets_ptr, mu_ptr, stream))

    def run_random(self, n_mom: int, seed: int, stream=None) -> np.ndarray:
        mu = np.zeros(n_mom)
        check(lib().tbk_kpm_run_random(self._h, n_mom, int(seed), capi.ptr(mu), stream))
        return mu

    def last_timing(self):
        ms, n, b = C.c_double(), C.c_int32(), C.c_double()
        check(lib().tbk_kpm_last_timing(self._h, C.byref(ms), C.byref(n), C.byref(b)))
        return ms.value, n.value, b.value

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().tbk_kpm_destroy(h)
            except Exception:
                pass
            self._h = C.c_void_p()


# ------------------------------------------------------------------ kernels
@dataclass(frozen=True)
class Kernel:
    kind: int
    p0: float = 0.0
    p1: float = 0.0

    def seq(self, N: int) -> np.ndarray:
        g = np.zeros(N)
        check(lib().tbk_kernel_seq(self.kind, N, self.p0, self.p1, capi.ptr(g)))
        return g


def Dirichlet() -> Kernel:
    return Kernel(capi.KERNEL_DIRICHLET)


def Fejer() -> Kernel:
    return Kernel(capi.KERNEL_FEJER)


def Lorentz(lam: float) -> Kernel:
    return Kernel(capi.KERNEL_LORENTZ, lam)


def Jackson() -> Kernel:
    return Kernel(capi.KERNEL_JACKSON)


def Lanczos(M: float) -> Kernel:
    return Kernel(capi.KERNEL_LANCZOS, M)


def Wang_and_Zunger(alpha: float, beta: float) -> Kernel:
    return Kernel(capi.KERNEL_WANG_ZUNGER, alpha, beta)


def kernel_seq(N: int, kernel: Kernel) -> np.ndarray:
    return kernel.seq(N)


# -------------------------------------------------------------- Green's function
class GreenFunctionImag:
    """Functor e -> <bras| Im G(e) |kets> from Chebyshev moments, TB/lattice.h:600-647."""

    def __init__(self, G: "GreenFunction", bras, kets, precision="fp64", kernel: Kernel | None = None):
        self.G = G
        n = G.scaled_HE.shape[0]
        same = bras is kets
        K = _block(kets, n)
        B = K if same else _block(bras, n)
        solver = KpmSolver(G.scaled_HE, K.shape[1], precision=precision, doubling=False)
        self.moments = solver.run(G.N, B, K)
        # the reference hard-codes Lorentz(N, 4) here (TB/lattice.h:613)
        self.kernel = kernel if kernel is not None else Lorentz(4.0)
        self.g = self.kernel.seq(G.N)

    @staticmethod
    def weight(x: float) -> float:
        return 1.0 / math.sqrt(1.0 - x * x)

    def __call__(self, e) -> np.ndarray | float:
        z = np.atleast_1d(np.asarray(e, dtype=np.complex128))
        zz = np.ascontiguousarray(np.stack([z.real, z.imag], axis=1))
        out = np.zeros(len(z))
        check(lib().tbk_green_imag_eval(self.G.N, capi.ptr(self.g), capi.ptr(self.moments), len(z), capi.ptr(zz),
                                        capi.ptr(out), None))
        return out if np.ndim(e) else float(out[0])

    def fft(self, n: int = 1):
        N = self.G.N * max(n, 1)
        E = np.zeros(N)
        v = np.zeros(N)
        check(lib().tbk_green_imag_fft(self.G.N, capi.ptr(self.g), capi.ptr(self.moments), max(n, 1), capi.ptr(E),
                                       capi.ptr(v), None))
        return E, v

    def slice_range(self, e_min: float, e_max: float, n: int = 1):
        N = self.G.N * n
        return int(round(math.acos(e_max) / math.pi * N)), int(round(math.acos(e_min) / math.pi * N))


class GreenFunction:
    """GreenFunction<Scalar>(N, HE, E_min, E_max), TB/lattice.h:553-559: a, b and
    scaled_HE = (HE - b I)/a computed in FP64 on the device."""

    def __init__(self, N: int, HE: SparseMatrix, E_min: float, E_max: float):
        self.N = N
        self.E_min, self.E_max = E_min, E_max
        self.a = (E_max - E_min) / 2
        self.b = (E_max + E_min) / 2
        h = C.c_void_p()
        check(lib().tbk_sparse_rescale(C.byref(h), HE.handle, self.a, self.b, None))
        self.scaled_HE = SparseMatrix(h.value)

    def scale(self, x, id_=1.0):
        return (x - self.b * id_) / self.a

    def spectral_range(self):
        return self.E_min, self.E_max

    def imag(self, bras, kets, precision="fp64", kernel: Kernel | None = None) -> GreenFunctionImag:
        return GreenFunctionImag(self, bras, kets, precision=precision, kernel=kernel)


# ------------------------------------------------------------------ DoS entry points
def density_of_states_function(G: GreenFunction, R: int = 4, seed: int = 0, precision="fp64"):
    """TB/functions.h:5-13: returns E -> -1/(4 pi) f(G.scale(E + 0i, i))."""
    kets = bases_of_uniform_ampl_with_random_phases(G.scaled_HE.shape[0], R, seed)
    f = G.imag(kets, kets, precision=precision)

    def dos(E):
        omega_t = G.scale(np.asarray(E, dtype=np.complex128) + 0j, 1.0j)
        return -1.0 / R / math.pi * f(omega_t)   # the reference writes -1.0 / 4 / pi with R = 4

    return dos


def density_of_states_seq(X: PartialLattice, N: int, E_list, E_min: float, E_max: float, scalar=complex,
                          R: int = 4, seed: int = 0, precision="fp64", kernel: Kernel | None = None) -> np.ndarray:
    """TB/functions.h:15-32: periodic {1,1} Hamiltonian, GreenFunction(N, H, E_min-1e-8,
    E_max+1e-8), R random-phase kets, rho(e) = -f(e)/(R pi) on already rescaled e."""
    H = X.get_Hamiltonian_periodic_extend_bare_sparse([1] * X.dim, scalar)
    G = GreenFunction(N, H, E_min - 1e-8, E_max + 1e-8)
    kets = bases_of_uniform_ampl_with_random_phases(X.get_total_number(), R, seed)
    f = G.imag(kets, kets, precision=precision, kernel=kernel)
    e = np.ascontiguousarray(E_list, dtype=np.float64)
    return -1.0 / R / math.pi * f(e)


def dos_from_moments(mu: np.ndarray, kernel: Kernel, R: float, e) -> np.ndarray:
    """rho(e) = -f(e)/(R pi) with f from the given kernel, all on the device."""
    mu = np.ascontiguousarray(mu, dtype=np.float64)
    e = np.ascontiguousarray(e, dtype=np.float64)
    rho = np.zeros(len(e))
    check(lib().tbk_dos_from_moments(len(mu), capi.ptr(mu), kernel.kind, kernel.p0, kernel.p1, float(R), len(e),
                                     capi.ptr(e), capi.ptr(rho), None))
    return rho
