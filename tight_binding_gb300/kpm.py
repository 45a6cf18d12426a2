"""Kernel-polynomial (Chebyshev) API, backed by libtbk.

    Cheb_first_kind_seq_braket      TB/numerics_cuda.cuh:8-14 (drop-in, both overloads)
    bases_of_uniform_ampl_with_random_phases   TB/numerical.h:120-122 (seeded)
    kernel_seq / kernels            TB/numerical.h:393-447
    GreenFunction, GreenFunctionImag   TB/lattice.h:532-652
    spectral_range                  TB/numerical.h:24-46 (device Lanczos, no size cap)
    cheb_expand, time_evolve        Cheb_first_kind_seq_view sums, TB/numerical.h:346-361
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


def trace_braket(bras_T, kets) -> float:
    """TB/numerical.h:126-135: sum_ij Re b_ij Re k_ij + Im b_ij Im k_ij (host)."""
    b = np.asarray(bras_T)
    k = np.asarray(kets)
    return float(np.sum(b.real * k.real + b.imag * k.imag))


def trace_braket_complex(bras_T, kets) -> complex:
    """TB/numerical.h:136-144: sum_ij conj(b_ij) k_ij (host)."""
    return complex(np.sum(np.conj(np.asarray(bras_T)) * np.asarray(kets)))


def expn_coef_alpha_seq(z: complex, n: int) -> np.ndarray:
    """TB/numerical.h:304-316: alpha_k(z) with 1/(z - x) = sum_k alpha_k(z) T_k(x)."""
    a = np.zeros(n, dtype=np.complex128)
    z = complex(z)
    check(lib().tbk_expn_coef_alpha_seq(z.real, z.imag, int(n), capi.ptr(a)))
    return a


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


def spectral_range(A: SparseMatrix, iters: int = 200, seed: int = 0) -> tuple[float, float, float, float]:
    """(E_min, E_max, res_min, res_max) of a Hermitian matrix by `iters` device
    Lanczos steps: the extreme Ritz values and their residual norms (an
    eigenvalue lies within res of each).  Replaces the reference's CPU Spectra
    solve matrix_spectral_range_sparse (TB/numerical.h:24-46), which refuses
    matrices above 5,000 rows; Ritz values lie inside the spectrum, so callers
    keep a margin (GreenFunction's epsilon)."""
    e0, e1, r0, r1 = C.c_double(), C.c_double(), C.c_double(), C.c_double()
    check(lib().tbk_spectral_range(A.handle, int(iters), int(seed), C.byref(e0), C.byref(e1), C.byref(r0),
                                   C.byref(r1), None))
    return e0.value, e1.value, r0.value, r1.value


class GreenFunction:
    """GreenFunction<Scalar>, TB/lattice.h:553-576: a, b and scaled_HE = (HE - b I)/a
    computed in FP64 on the device.  The three constructors:

        GreenFunction(N, HE, E_min, E_max)         a = (E_max - E_min)/2
        GreenFunction(N, HE, ref_HE, epsilon=0.01) range of ref_HE by Lanczos,
                                                   a = (E_max - E_min)/(2 - epsilon)
        GreenFunction(N, HE)                       = GreenFunction(N, HE, HE)

    (the third also tabulates dense T_n(H~) below 5,000 rows in the reference,
    TB/lattice.h:571-576; that dense table is not built here)."""

    def __init__(self, N: int, HE: SparseMatrix, E_min=None, E_max=None, epsilon: float | None = None,
                 lanczos_iters: int = 200):
        self.N = N
        if E_min is None or isinstance(E_min, SparseMatrix):
            ref = HE if E_min is None else E_min
            eps = 0.01 if epsilon is None else float(epsilon)
            if E_max is not None:          # GreenFunction(N, HE, ref_HE, epsilon) positionally
                eps = float(E_max)
            E_min, E_max, _, _ = spectral_range(ref, lanczos_iters)
            self.a = (E_max - E_min) / (2 - eps)
        else:
            self.a = (E_max - E_min) / 2
        self.E_min, self.E_max = E_min, E_max
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


# ------------------------------------------------------ expansions applied to vectors
def cheb_expand(Ht: SparseMatrix, coef, kets, precision="dd") -> np.ndarray:
    """sum_k coef[k] T_k(Ht) kets on the device (kets: n or n x R complex;
    returns the same shape).  The walk the reference writes with
    Cheb_first_kind_seq_view (TB/numerical.h:346-361) plus a host sum.
    precision "dd" (default: double-float recursion, FP64-class accuracy on
    the FP32 pipe, faster than "fp64" on this GPU), "fp64" or "mixed"."""
    kets = np.asarray(kets)
    n = Ht.shape[0]
    K = _block(kets, n)
    c = np.ascontiguousarray(coef, dtype=np.complex128)
    out = np.zeros(K.shape, dtype=np.complex128, order="F")
    check(lib().tbk_cheb_expand(Ht.handle, len(c), capi.ptr(c), K.shape[1], capi.ptr(K), capi.ptr(out),
                                _prec(precision), None))
    return out.reshape(kets.shape) if kets.ndim == 1 else out


class Cheb_first_kind_seq_view:
    """Cheb_first_kind_seq_view(x, v), TB/numerical.h:346-361: next() returns
    (i, T_i(x) v) for i = 0, 1, 2, ...; the recursion state stays on the device
    (one step per call, the block copied to the host)."""

    def __init__(self, x: SparseMatrix, v, precision="fp64"):
        v = np.asarray(v)
        self._vec = v.ndim == 1
        self._K = _block(v, x.shape[0])
        h = C.c_void_p()
        check(lib().tbk_cheb_view_create(C.byref(h), x.handle, self._K.shape[1], capi.ptr(self._K), _prec(precision)))
        self._h = h

    def next(self):
        out = np.zeros(self._K.shape, dtype=np.complex128, order="F")
        i = C.c_int32()
        check(lib().tbk_cheb_view_next(self._h, C.byref(i), capi.ptr(out), None))
        return i.value, (out[:, 0] if self._vec else out)

    def __iter__(self):
        while True:
            yield self.next()

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                lib().tbk_cheb_view_destroy(h)
            except Exception:
                pass
            self._h = C.c_void_p()


def Cheb_first_kind_seq_on_bases(x: SparseMatrix, n: int, v, precision="fp64") -> list:
    """TB/numerical.h:333-344: [T_0(x) v, ..., T_{n-1}(x) v] (all blocks on the host)."""
    view = Cheb_first_kind_seq_view(x, v, precision)
    return [view.next()[1] for _ in range(n)]


def sparse_apply(A: SparseMatrix, kets, precision="dd") -> np.ndarray:
    """A @ kets on the device (T_1(A) kets)."""
    return cheb_expand(A, [0.0, 1.0], kets, precision)


def delta_coefficients(e: float, N: int) -> np.ndarray:
    """a_d(k) T_k(e), k = 0 .. N: the single-energy projection of
    conductivity_test_sawtooth (TB/snippets.h:175, 194-202)."""
    c = np.zeros(N + 1, dtype=np.complex128)
    check(lib().tbk_cheb_coef_delta(float(e), int(N), capi.ptr(c)))
    return c


def evolution_terms(a: float, t: float, tol: float = 1e-15) -> int:
    k = C.c_int32()
    check(lib().tbk_cheb_evolution_terms(float(a), float(t), float(tol), C.byref(k)))
    return k.value


def evolution_coefficients(a: float, b: float, t: float, n_terms: int | None = None, tol: float = 1e-15) -> np.ndarray:
    """exp(-i H t), H = a Ht + b: exp(-i b t) (2 - delta_k0) (-i)^k J_k(a t)."""
    n_terms = evolution_terms(a, t, tol) if n_terms is None else int(n_terms)
    c = np.zeros(n_terms, dtype=np.complex128)
    check(lib().tbk_cheb_coef_evolution(float(a), float(b), float(t), n_terms, capi.ptr(c)))
    return c


def time_evolve(G: "GreenFunction", t: float, kets, precision="dd", tol: float = 1e-15) -> np.ndarray:
    """exp(-i HE t) kets for the Hamiltonian of G (HE = a scaled_HE + b)."""
    return cheb_expand(G.scaled_HE, evolution_coefficients(G.a, G.b, t, tol=tol), kets, precision)


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
